// dg_noalloc.cu -- dg_render_noalloc: one frame of one mesh rendered with the
// same kernels as dg_scene_render, for callers that cannot allocate device
// memory while they draw (a host or plugin that owns a fixed device-memory
// budget, or a frame loop that must not stall on the device-wide
// synchronization of cudaMalloc/cudaFree). Every byte of scratch the kernels
// need lives in g_noalloc_scratch below, a statically sized __device__ array
// that each GPU loading the library keeps until the process exits; this file
// calls no cudaMalloc, cudaFree or other allocating routine.
//
// The scratch is shared by every call and keeps the last call's contents, so
// each call first resets what must start empty (visibility keys, vertex marks,
// counters, the error word). Calls whose GPU work overlaps race on it.
//
// The job descriptor travels as a kernel parameter: k_noalloc_begin, the first
// kernel of every call, writes it into the scratch array together with those
// resets, so no host buffer has to outlive the call.
#include <cstring>
#include <mutex>

#include "dg_internal.cuh"

namespace {

constexpr size_t kAlign = 256;
constexpr size_t align_up(size_t x) { return (x + kAlign - 1) / kAlign * kAlign; }

constexpr uint32_t kQueueCap = 16384;  // queued triangles; more are rasterized in place by their warp

// Scratch layout (byte offsets, each sub-buffer 256-byte aligned).
struct NoallocDesc {  // the job descriptor the kernels read
    DgFrameDev frame;
    DgSegDev seg;
    DgTexDev tex[DG_NOALLOC_MAX_TEXMAPS + 1];  // [0] = 1x1 white default map
    DgMatDev mats[DG_NOALLOC_MAX_MATERIALS];
};
constexpr size_t kOffDesc = 0;
constexpr uint32_t kVrowExtra = 4096;  // light/halfway rows for clip vertices
constexpr uint32_t kTrecCap = (uint32_t)dg_trec_cap(DG_NOALLOC_MAX_TRIANGLES);  // triangle records
constexpr size_t kOffVrec = align_up(kOffDesc + sizeof(NoallocDesc));
constexpr size_t kOffVmask = align_up(kOffVrec + (size_t)DG_NOALLOC_MAX_VERTICES * sizeof(float4));
constexpr size_t kOffVshade = align_up(kOffVmask + (size_t)DG_NOALLOC_MAX_VERTICES * sizeof(uint16_t));
constexpr size_t kOffVmark = align_up(kOffVshade + (size_t)(DG_NOALLOC_MAX_VERTICES + kVrowExtra) *
                                                       DG_NOALLOC_MAX_LIGHTS * 2 * sizeof(float4));
constexpr size_t kOffQueue = align_up(kOffVmark + (size_t)DG_NOALLOC_MAX_VERTICES * sizeof(uint8_t));
constexpr size_t kOffSmall = align_up(kOffQueue + (size_t)kQueueCap * sizeof(DgQueueRec));
constexpr size_t kOffQbase = align_up(kOffSmall + (size_t)kQueueCap * sizeof(DgQueueRec));
constexpr size_t kOffSurv = align_up(kOffQbase + (size_t)dg_items_cap(kQueueCap) * sizeof(uint2));
constexpr size_t kOffRecOf = align_up(kOffSurv + (size_t)DG_NOALLOC_MAX_TRIANGLES * sizeof(uint32_t));
constexpr size_t kOffTrec = align_up(kOffRecOf + (size_t)DG_NOALLOC_MAX_TRIANGLES * sizeof(uint32_t));
constexpr size_t kOffCounters = align_up(kOffTrec + (size_t)kTrecCap * sizeof(DgTriRec));
constexpr size_t kOffErr = align_up(kOffCounters + DG_NCOUNTERS * sizeof(unsigned long long));
constexpr size_t kOffWhite = align_up(kOffErr + sizeof(uint32_t));
constexpr size_t kOffVis = align_up(kOffWhite + 8);
constexpr size_t kScratchBytes = align_up(kOffVis + (size_t)DG_NOALLOC_MAX_PIXELS * sizeof(uint64_t));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char* g_scratch_ptr[kMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once per device).
dg_status scratch_on_current_device(unsigned char** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return DG_E_CUDA;
    }
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_scratch_ptr[dev]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            return DG_E_CUDA;
        }
        g_scratch_ptr[dev] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_ptr[dev];
    return DG_OK;
}

// Writes the call's job descriptor into the scratch array and resets what the
// previous call left behind: counters, error word, vertex marks, the 1x1 white
// default map's texel word, and the visibility keys of npx pixels.
__global__ void k_noalloc_begin(const __grid_constant__ NoallocDesc d, unsigned char* base, uint32_t npx) {
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
    static_assert(sizeof(NoallocDesc) % 16 == 0 && kOffDesc % 16 == 0, "descriptor copied in 16-byte words");
    const uint4* src = reinterpret_cast<const uint4*>(&d);
    uint4* dst = reinterpret_cast<uint4*>(base + kOffDesc);
    for (uint32_t i = t; i < sizeof(NoallocDesc) / 16; i += stride) dst[i] = src[i];
    if (t < DG_NCOUNTERS) reinterpret_cast<unsigned long long*>(base + kOffCounters)[t] = 0ull;
    if (t == 0) {
        *reinterpret_cast<uint32_t*>(base + kOffErr) = 0u;
        reinterpret_cast<uint32_t*>(base + kOffWhite)[0] = 0xFFFFFFFFu;
        reinterpret_cast<uint32_t*>(base + kOffWhite)[1] = 0xFFFFFFFFu;
    }
    uint32_t* vmark = reinterpret_cast<uint32_t*>(base + kOffVmark);
    for (uint32_t i = t; i < DG_NOALLOC_MAX_VERTICES / 4; i += stride) vmark[i] = 0u;
    unsigned long long* vis = reinterpret_cast<unsigned long long*>(base + kOffVis);
    for (uint32_t i = t; i < npx; i += stride) vis[i] = DG_VIS_EMPTY;
}

#define NA_CUDA(x)                              \
    do {                                        \
        if ((x) != cudaSuccess) {               \
            cudaGetLastError();                 \
            return DG_E_CUDA;                   \
        }                                       \
    } while (0)

}  // namespace

extern "C" dg_status dg_render_noalloc(const dg_frame_params* p, const dg_device_mesh* m, const dg_material* mats,
                                       uint32_t nmat, const dg_device_texmap* texmaps, uint32_t ntex, void* bgra_out,
                                       void* depth_out, void* stream, int32_t* status_out) {
    if (!p || !m || (nmat && !mats) || (ntex && !texmaps) || !bgra_out || !depth_out) return DG_E_INVALID;
    if (!m->pos || !m->nrm || !m->uv || !m->tri_pos || !m->tri_uv || !m->tri_nrm) return DG_E_INVALID;
    if (p->width == 0 || p->height == 0 || p->canvas_width == 0 || p->canvas_height == 0) return DG_E_INVALID;
    if (p->nlights == 0) return DG_E_INVALID;
    const uint64_t npx = (uint64_t)p->canvas_width * p->canvas_height;
    if (m->nv > DG_NOALLOC_MAX_VERTICES || m->ntri > DG_NOALLOC_MAX_TRIANGLES || npx > DG_NOALLOC_MAX_PIXELS ||
        p->nlights > DG_NOALLOC_MAX_LIGHTS || ntex > DG_NOALLOC_MAX_TEXMAPS || nmat > DG_NOALLOC_MAX_MATERIALS)
        return DG_E_LIMIT;
    if (m->ntri && nmat == 0) return DG_E_INVALID;
    for (uint32_t i = 0; i < nmat; i++) {
        for (int32_t id : {mats[i].map_ka, mats[i].map_kd})
            if (id < -1 || id >= (int32_t)ntex) return DG_E_INVALID;
        if (mats[i].alpha < 1.0f) return DG_E_LIMIT;  // the transparent pass is not part of this entry point
    }
    for (uint32_t i = 0; i < ntex; i++) {
        const dg_device_texmap& t = texmaps[i];
        if (!t.bytes || (reinterpret_cast<uintptr_t>(t.bytes) & 3u) || t.components == 0 ||
            t.len % t.components != 0 || t.len / t.components != (uint64_t)t.width * t.height)
            return DG_E_INVALID;
    }

    unsigned char* base = nullptr;
    dg_status st = scratch_on_current_device(&base);
    if (st) return st;
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    // Host-side frame setup (Scene::render's matrix and planes) into a stack descriptor.
    NoallocDesc d;
    std::memset(&d, 0, sizeof(d));
    DgFrameDev& f = d.frame;
    const float ratio = (float)p->width / (float)p->height;
    st = dg_host_frame_setup(p->width, p->height, p->cam_pos, p->cam_dir, ratio, p->near_, p->far_, p->fov_x_deg,
                             f.M, f.plane);
    if (st) return st;
    f.cam[0] = p->cam_pos[0];
    f.cam[1] = p->cam_pos[1];
    f.cam[2] = p->cam_pos[2];
    f.clear_depth = p->clear_depth;
    f.nlights = p->nlights;
    for (uint32_t l = 0; l < p->nlights; l++)
        for (int k = 0; k < 3; k++) f.light[l][k] = p->lights[l][k];
    f.exponent = p->exponent;
    f.off_x = (float)p->offset_x;
    f.off_y = (float)p->offset_y;
    f.width = p->canvas_width;
    f.height = p->canvas_height;
    f.vis = reinterpret_cast<uint64_t*>(base + kOffVis);
    f.colour = static_cast<uint32_t*>(bgra_out);
    f.depth = static_cast<float*>(depth_out);
    f.seg_begin = 0;
    f.seg_count = 1;
    f.tile_begin = 0;
    f.tiles_x = (p->canvas_width + DG_TILE_W - 1) / DG_TILE_W;
    f.pix_begin = 0;
    f.small_max_px = DG_SMALL_MAX_PX;
    const uint32_t tiles = f.tiles_x * ((p->canvas_height + DG_TILE_H - 1) / DG_TILE_H);

    DgSegDev& sg = d.seg;
    sg.frame = 0;
    sg.tri_begin = 0;
    sg.vtx_begin = 0;
    sg.seq_base = 0;
    sg.ntri = m->ntri;
    sg.nv = m->nv;
    sg.nmats = nmat;
    sg.pos = static_cast<const float4*>(m->pos);
    sg.nrm = static_cast<const float4*>(m->nrm);
    sg.uv = static_cast<const float2*>(m->uv);
    sg.tri_pos = static_cast<const uint4*>(m->tri_pos);
    sg.tri_uv = static_cast<const uint4*>(m->tri_uv);
    sg.tri_nrm = static_cast<const uint4*>(m->tri_nrm);
    sg.mats = reinterpret_cast<const DgMatDev*>(base + kOffDesc + offsetof(NoallocDesc, mats));

    // texture table: [0] the 1x1 white default map (scene/mod.rs:128-135), then the caller's maps
    d.tex[0].words = reinterpret_cast<const uint32_t*>(base + kOffWhite);
    d.tex[0].len = 3;
    d.tex[0].width = d.tex[0].height = 1;
    d.tex[0].comps = 3;
    d.tex[0].fw = d.tex[0].fh = 1.0f;
    d.tex[0].small = 1;
    for (uint32_t i = 0; i < ntex; i++) {
        d.tex[i + 1].words = static_cast<const uint32_t*>(texmaps[i].bytes);
        d.tex[i + 1].len = texmaps[i].len;
        d.tex[i + 1].width = texmaps[i].width;
        d.tex[i + 1].height = texmaps[i].height;
        d.tex[i + 1].comps = texmaps[i].components;
        d.tex[i + 1].fw = (float)texmaps[i].width;
        d.tex[i + 1].fh = (float)texmaps[i].height;
        d.tex[i + 1].small = dg_tex_small(texmaps[i].len, texmaps[i].width, texmaps[i].height);
    }
    for (uint32_t i = 0; i < nmat; i++) {
        for (int k = 0; k < 3; k++) {
            d.mats[i].ka[k] = mats[i].ka[k];
            d.mats[i].kd[k] = mats[i].kd[k];
            d.mats[i].ks[k] = mats[i].ks[k];
        }
        d.mats[i].alpha = mats[i].alpha;
        d.mats[i].map_ka = (uint32_t)(mats[i].map_ka + 1);
        d.mats[i].map_kd = (uint32_t)(mats[i].map_kd + 1);
    }
    DgJobDev job;
    std::memset(&job, 0, sizeof(job));
    job.frames = reinterpret_cast<const DgFrameDev*>(base + kOffDesc + offsetof(NoallocDesc, frame));
    job.segs = reinterpret_cast<const DgSegDev*>(base + kOffDesc + offsetof(NoallocDesc, seg));
    job.nframes = 1;
    job.nsegs = 1;
    job.total_vtx = m->nv;
    job.total_tri = m->ntri;
    job.total_tiles = tiles;
    job.shade_stride = p->nlights;
    job.vrec = reinterpret_cast<float4*>(base + kOffVrec);
    job.vmask = reinterpret_cast<uint16_t*>(base + kOffVmask);
    job.vshade = reinterpret_cast<float4*>(base + kOffVshade);
    job.vrow_extra = kVrowExtra;
    job.vmark = reinterpret_cast<uint8_t*>(base + kOffVmark);
    job.surv = reinterpret_cast<uint32_t*>(base + kOffSurv);
    job.rec_of = reinterpret_cast<uint32_t*>(base + kOffRecOf);
    job.trec = reinterpret_cast<DgTriRec*>(base + kOffTrec);
    job.trec_cap = kTrecCap;
    job.queue = reinterpret_cast<DgQueueRec*>(base + kOffQueue);
    job.small = reinterpret_cast<DgQueueRec*>(base + kOffSmall);
    job.small_cap = kQueueCap;
    job.items = reinterpret_cast<uint2*>(base + kOffQbase);
    job.items_cap = (uint32_t)dg_items_cap(kQueueCap);
    job.queue_cap = kQueueCap;
    job.item_units = DG_ITEM_UNITS;
    job.cnt = reinterpret_cast<unsigned long long*>(base + kOffCounters);
    job.total_px = (uint32_t)npx;
    job.tile_rows = DG_TILE_H;
    job.tex = reinterpret_cast<const DgTexDev*>(base + kOffDesc + offsetof(NoallocDesc, tex));
    job.ntex = ntex + 1;
    job.err = reinterpret_cast<uint32_t*>(base + kOffErr);

    int dev = 0, nsm = 0;
    NA_CUDA(cudaGetDevice(&dev));
    NA_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));

    // The descriptor goes by value as a kernel parameter (no host staging buffer).
    k_noalloc_begin<<<(unsigned)nsm * 4u, 256, 0, s>>>(d, base, (uint32_t)npx);
    NA_CUDA(cudaGetLastError());

    DgLaunchCfg cfg{};
    cfg.vertex_blocks = (unsigned)nsm * DG_VERTEX_BLOCKS_PER_SM;
    cfg.cull_blocks = (unsigned)nsm * DG_CULL_BLOCKS_PER_SM;
    cfg.setup_blocks = (unsigned)nsm * DG_SETUP_BLOCKS_PER_SM;
    cfg.queue_blocks = (unsigned)nsm * DG_QUEUE_BLOCKS_PER_SM;
    NA_CUDA(dg_launch_job(job, cfg, s, nullptr));

    if (status_out) {
        uint32_t err = 0;
        NA_CUDA(cudaStreamSynchronize(s));
        NA_CUDA(cudaMemcpy(&err, base + kOffErr, sizeof(err), cudaMemcpyDeviceToHost));
        *status_out = DG_OK;
        for (int b = 1; b < 32; b++)
            if (err & (1u << b)) {
                *status_out = (dg_status)b;
                break;
            }
    }
    return DG_OK;
}
