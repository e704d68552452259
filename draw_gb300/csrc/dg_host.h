// dg_host.h -- host-side state of the GB300 rasterizer, shared by the C ABI
// (dg_api.cu) and the render server (dg_server.cu): scene and camera state,
// resident resources, the per-frame host setup of Scene::render and the
// launch of one render job on a job slot.
//
// Host floating point follows the reference's Rust semantics: the files
// including this header are compiled with -ffp-contract=off, so every
// expression rounds each operation to f32 in source order.
#pragma once

#include <cmath>
#include <cstring>
#include <vector>

#include "dg_internal.cuh"

namespace dgh {

// ------------------------------------------------------------ host vectors
struct HV3 {
    float x, y, z;
};
inline HV3 h3(float x, float y, float z) { return HV3{x, y, z}; }
inline HV3 hadd(HV3 a, HV3 b) { return h3(a.x + b.x, a.y + b.y, a.z + b.z); }
inline HV3 hsub(HV3 a, HV3 b) { return h3(a.x - b.x, a.y - b.y, a.z - b.z); }
inline HV3 hmul(HV3 a, float s) { return h3(a.x * s, a.y * s, a.z * s); }
inline HV3 hdiv(HV3 a, float s) { return h3(a.x / s, a.y / s, a.z / s); }
inline float hdot(HV3 a, HV3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }       // linalg.rs:182-184
inline float hnorm(HV3 a) { return std::sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }  // linalg.rs:167-171
inline HV3 hnormalized(HV3 a) { return hdiv(a, hnorm(a)); }                           // linalg.rs:173-175
inline HV3 hcross(HV3 a, HV3 b) {                                                      // linalg.rs:186-200
    return h3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}

struct HM4 {
    float m[4][4];
};

struct Camera {  // scene/mod.rs:282-294
    HV3 position, direction, up;
    float top, bottom, right, left;
    float near_, far_;
    HV3 u, v, w;
};

struct Scene {  // scene/mod.rs:749-757
    uint64_t width = 0, height = 0;
    Camera cam;
    std::vector<int32_t> objects;
    std::vector<HV3> lights;
    int32_t exponent = 2;
    int32_t interpolation = DG_INTERP_AFFINE;  // extension (dg_scene_set_interpolation)
};

dg_status camera_init(Camera& c, HV3 pos, HV3 dir, float ratio, float near_, float far_, float fov_x);
void camera_update_basis(Camera& c);
dg_status camera_op(Scene& s, int32_t op, const float* a);
// gen_transformation_matrix (scene/mod.rs:817-899) and gen_view_planes (:481-593).
dg_status frame_setup(Scene& s, float M[4][4], float planes[6][4]);

// ------------------------------------------------------------- resources
struct TexMap {
    uint32_t* d_words = nullptr;
    uint64_t len = 0;
    uint32_t w = 0, h = 0, comps = 0;
    uint32_t filter = DG_FILTER_NEAREST;  // extension (dg_texmap_set_filter)
};

struct Object {
    bool alive = false;
    float4* d_pos = nullptr;
    float4* d_nrm = nullptr;
    float2* d_uv = nullptr;
    uint4* d_tri_pos = nullptr;
    uint4* d_tri_uv = nullptr;
    uint4* d_tri_nrm = nullptr;
    DgMatDev* d_mats = nullptr;
    uint32_t nv = 0, nn = 0, nuv = 0, ntri_opaque = 0, nmats = 0;
    // Transparent meshes (object.rs:45-53: material alpha < 1), concatenated in
    // mesh order: mesh m holds triangles [tmesh_off[m], tmesh_off[m + 1]) as
    // (position indices, material), (uv indices, m), (normal indices). The
    // painter's sort of every frame reorders each mesh and the order persists
    // (scene/mod.rs:1100-1115): d_tt[tcur] holds the current order, and a
    // render writes the next one into d_tt[1 - tcur].
    uint4* d_tt[2][3] = {};
    int tcur = 0;
    uint32_t nt = 0;
    std::vector<uint32_t> tmesh_off;
};

struct Canvas {
    bool alive = false;
    uint64_t w = 0, h = 0;
    uint32_t* d_colour = nullptr;
    float* d_depth = nullptr;
    uint64_t* d_vis = nullptr;
    uint32_t* d_cells = nullptr;  // DgFrameDev::cells; zeroed at allocation
    uint32_t epoch = 0;           // advanced for every frame rendered into the canvas
    bool depth_init = false;
    float depth_max = 0.0f;
    float off_x = 0.0f, off_y = 0.0f;
    // dg_canvas_read_async: the copy runs on the context's copy stream after
    // ev_rendered; ev_read marks its end. While read_pending, the next operation
    // that looks the canvas up first makes the context stream wait for ev_read.
    cudaEvent_t ev_rendered = nullptr, ev_read = nullptr;
    uint32_t* h_err = nullptr;  // pinned: the error word copied with the frame
    bool read_pending = false;
};

// The buffers one frame renders into.
struct FrameTarget {
    uint32_t* colour;
    float* depth;
    uint64_t* vis;  // all DG_VIS_EMPTY on entry; left so on exit
    uint64_t w, h;
    float clear_depth;
    float off_x, off_y;
    uint32_t* cells;  // DgFrameDev::cells (or null)
    uint32_t epoch;   // differs from the frame's other renders into the same cells
};

// Words of DgFrameDev::cells for a w x h canvas.
inline uint64_t dg_cell_count(uint64_t w, uint64_t h) { return ((w + 31u) / 32u) * ((h + 31u) / 32u); }

// Scratch, staging and stream of one render job in flight. The context owns
// one; the render server owns one per concurrent batch.
struct JobSlot {
    cudaStream_t stream = nullptr;
    uint16_t* d_vmask = nullptr;  // plane-sign masks of the job's vertices
    size_t vmask_cap = 0;
    float4* d_vrec = nullptr;  // vertex records (screen centre, eye distance, masks)
    size_t vrec_cap = 0;
    float4* d_vshade = nullptr;
    size_t vshade_cap = 0;
    uint8_t* d_vmark = nullptr;  // zeroed at allocation; the queue pass clears what setup sets
    size_t vmark_cap = 0;
    DgQueueRec* d_queue = nullptr;
    DgQueueRec* d_small = nullptr;  // small-triangle list
    size_t small_cap = 0;
    // transparent pass scratch (DgJobDev)
    uint64_t* d_tkey[2] = {};
    uint32_t* d_tval[2] = {};
    size_t tsort_cap = 0;
    DgTriRec* d_ttrec = nullptr;
    uint4* d_tbox = nullptr;
    uint2* d_tmeta = nullptr;
    float* d_talpha = nullptr;
    uint32_t* d_tcnt = nullptr;
    unsigned long long* d_tscan = nullptr;
    size_t tout_cap = 0;  // clip outputs the arrays above hold (tscan: one more)
    uint64_t* d_fkey[2] = {};
    uint32_t* d_fval[2] = {};
    size_t frag_cap = 0;
    uint32_t* d_hist = nullptr;
    size_t hist_cap = 0;  // entries
    uint2* d_items = nullptr;  // raster work items
    size_t queue_cap = 0;
    size_t items_cap = 0;
    uint32_t* d_surv = nullptr;  // cull survivors
    size_t surv_cap = 0;
    uint32_t* d_rec_of = nullptr;  // first triangle record of each survivor
    size_t rec_of_cap = 0;
    DgTriRec* d_trec = nullptr;
    size_t trec_cap = 0;
    float4* d_trec_w = nullptr;  // perspective weights per record (grown only for perspective frames)
    size_t trec_w_cap = 0;
    float4* d_ttrec_w = nullptr;  // the same for the transparent records
    size_t ttrec_w_cap = 0;
    uint32_t small_max_px = DG_SMALL_MAX_PX_AUTO;  // dg_tuning knobs
    uint32_t setup_blocks_per_sm = DG_SETUP_BLOCKS_PER_SM;
    uint32_t queue_blocks_per_sm = DG_QUEUE_BLOCKS_PER_SM;
    uint32_t cull_blocks_per_sm = DG_CULL_BLOCKS_PER_SM;
    uint32_t tile_rows = 0;  // 0: chosen per job (build_job)
    uint32_t item_units = DG_ITEM_UNITS;
    uint32_t record_limit = 0;
    unsigned long long* d_counters = nullptr;  // the job counters (DG_CNT_*, DG_NCOUNTERS words)
    uint32_t* d_err = nullptr;
    static const int kStage = 4;  // pinned staging ring for job descriptors
    void* h_stage[kStage] = {};
    void* d_stage[kStage] = {};
    size_t stage_cap[kStage] = {};
    cudaEvent_t stage_ev[kStage] = {};
    int stage = 0;
    bool timing = false;
    cudaEvent_t ev[DG_NKERNELS + 1] = {};
    bool ev_valid = false;
    uint64_t last_vtx = 0, last_tri = 0, last_h2d = 0, last_launches = 0;
    uint64_t last_tile_rows = 0, last_small_max_px = 0;  // the last job's resolve tile height, first frame's threshold
    uint64_t scratch_bytes = 0;  // device bytes held by the scratch buffers
};

}  // namespace dgh

namespace dgh {
// Scratch of dg_canvas_draw_triangles_2d (grow-only, on the context stream).
struct OverlaySlot {
    DgTriRec* d_rec = nullptr;
    size_t rec_cap = 0;
    uint4* d_box = nullptr;
    size_t box_cap = 0;
    unsigned long long* d_scan = nullptr;
    size_t scan_cap = 0;
    uint64_t* d_fkey[2] = {};
    uint32_t* d_fval[2] = {};
    size_t frag_cap[4] = {};
    uint32_t* d_hist = nullptr;
    size_t hist_cap = 0;
    unsigned long long* d_cnt = nullptr;
    size_t cnt_cap = 0;
    uint32_t* d_rgba = nullptr;  // staging of dg_canvas_read_rgba
    size_t rgba_cap = 0;
};
}  // namespace dgh

struct dg_ctx {
    int device = 0;
    int nsm = 152;
    cudaStream_t own_stream = nullptr;
    cudaStream_t copy_stream = nullptr;  // device-to-host copies of dg_canvas_read_async
    std::vector<dgh::TexMap> tex;  // [0] = 1x1 white default map
    DgTexDev* d_tex = nullptr;
    size_t d_tex_cap = 0;
    bool tex_dirty = true;
    std::vector<dgh::Object> objects;
    std::vector<dgh::Scene> scenes;
    std::vector<dgh::Canvas> canvases;
    dgh::JobSlot main;  // the slot of dg_scene_render / dg_render_batch (main.stream = the context stream)
    dgh::OverlaySlot overlay;
};

namespace dgh {

dg_status set_device(dg_ctx* c);
dg_status slot_init(dg_ctx* c, JobSlot& s, cudaStream_t stream);
void slot_free(JobSlot& s);
// Returns the lowest error code the slot's kernels raised since the last call, and clears it.
dg_status slot_take_errors(JobSlot& s);
// Uploads the texture table if textures were added.
dg_status sync_tex_table(dg_ctx* c, cudaStream_t s);
// Device bytes slot s's scratch will hold after launching a job of V vertices,
// T triangles, L lights per vertex and P pixels (same sizing rules as launch_frames).
uint64_t slot_scratch_after(const JobSlot& s, uint64_t V, uint64_t T, uint32_t L, uint64_t P);
// Builds and launches one render job over n frames on slot s (asynchronous).
dg_status launch_frames(dg_ctx* c, JobSlot& s, Scene* const* scenes, const FrameTarget* targets, uint32_t n);

// Host part of one render job: the per-frame and per-segment descriptors (the
// bytes uploaded before the kernels run), the job descriptor the kernels take
// by value (its frames/segs pointers are set by enqueue_job) and the grid sizes.
struct JobBuild {
    std::vector<DgFrameDev> frames;
    std::vector<DgSegDev> segs;
    size_t fbytes = 0, sbytes = 0;
    DgJobDev job{};
    DgLaunchCfg cfg{};
    uint64_t total_vtx = 0, total_tri = 0, launches = 0;
    std::vector<int32_t> transparent_objects;  // objects whose transparent order the job advances
};
// Host frame setup of every frame (camera basis, matrix, view planes) and the
// scratch sizing of slot s (grows its buffers; synchronizes s only when one grows).
dg_status build_job(dg_ctx* c, JobSlot& s, Scene* const* scenes, const FrameTarget* targets, uint32_t n,
                    JobBuild& b);
// Resolves scene and canvas ids into frames (DG_E_INVALID for a bad id,
// DG_E_DEPTH_UNINIT for a canvas without init_depth).
dg_status resolve_frames(dg_ctx* c, const int32_t* scenes, const int32_t* canvases, uint32_t n,
                         std::vector<Scene*>& sc, std::vector<FrameTarget>& tg);
// dg_scene_render / dg_render_batch on the context's own slot and stream.
dg_status render_job(dg_ctx* c, const int32_t* scenes, const int32_t* canvases, uint32_t n);
// Enqueues the counter reset and the kernels of a built job whose descriptors
// are (or will be, in stream order) at d_stage on the device.
dg_status enqueue_job(JobBuild& b, JobSlot& s, void* d_stage, cudaStream_t stream, bool timing);
// After a job is enqueued: the painter's order it wrote becomes each
// transparent object's current order.
void advance_transparent(dg_ctx* c, const JobBuild& b);

}  // namespace dgh
