// dg_internal.cuh -- device-side data layout shared by the host API (dg_api.cu)
// and the kernels (dg_kernels.cu) of the GB300 rasterizer.
//
// HBM layout (all resident until their owner is destroyed):
//   texture map   : image bytes packed into u32 words (+1 pad word), row 0 = top
//   object        : pos float4[V] (w = 1), nrm float4[N], uv float2[U],
//                   tri_pos uint4[T] = (p0,p1,p2,material), tri_uv uint4[T],
//                   tri_nrm uint4[T]; opaque meshes first, in submission order
//   canvas        : colour u32[W*H] (BGRA bytes, row 0 = top), depth f32[W*H]
//                   (y*W+x, y = 0 at the bottom), vis u64[W*H] (visibility keys,
//                   kept at DG_VIS_EMPTY between frames)
//   render scratch: vrec float4[V_total] (snapped centre x,y, eye distance,
//                   plane-sign masks), vmask u16[V_total] (the masks alone, for
//                   the cull's gathers), vshade float4[V_total*L*2] (light, halfway),
//                   raster-queue records + their work-unit bases, counters
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/draw_gpu.h"

#define DG_MAXL DG_MAX_LIGHTS

// DRAW_CHECKED builds (draw_gb300/_build.py build(checked=True)): the kernels
// test the data-dependent indices of their gathers and scatters (mesh indices,
// queue entries, light/halfway rows, raster boxes) against the buffers' sizes;
// an index out of range records DG_E_CUDA in the job's error word and the
// access is skipped. Off in the normal build, where the host validates the
// indices and the kernels' own arithmetic keeps the rest in range.
#ifdef DRAW_CHECKED
#define DG_CHECKED 1
#else
#define DG_CHECKED 0
#endif
#define DG_IN_RANGE(cond, err) (!DG_CHECKED || dg_check_range((cond), (err)))
__device__ __forceinline__ bool dg_check_range(bool ok, uint32_t* err) {
    if (!ok) atomicOr(err, 1u << 6 /* DG_E_CUDA */);
    return ok;
}
// DRAW_TIMELINE builds (draw_gb300/_build.py build(timeline=True)): each
// kernel of a render job records in the global timer (ns) when its first block
// started, when its first and its last block passed the wait for the previous
// kernel, and when its last block finished (thread 0 of each block, with
// atomics; they add a few microseconds to a frame). dg_timeline_read returns
// the record. Off in the normal build.
#ifdef DRAW_TIMELINE
#define DG_TIMELINE 1
#else
#define DG_TIMELINE 0
#endif
#define DG_VIS_EMPTY 0xFFFFFFFFFFFFFFFFull

// Triangles whose clipped bounding box has at most DgFrameDev.small_max_px
// pixels go to the small-triangle list, whose entries the queue pass
// rasterizes one per lane; larger ones go to the raster queue: their row-major
// bounding-box pixels are cut into units of DG_UNIT_PX (one per lane of a warp)
// and the units into work items of at most DgJobDev.item_units (default
// DG_ITEM_UNITS), which the queue pass spreads over all warps. Unless the
// tuning fixes it, a frame's threshold is DG_SMALL_MAX_PX, or
// DG_SMALL_MAX_PX_MICRO when the frame has at least as many triangles as
// pixels: lanes that each loop over a box of up to 64 pixels pay off only when
// there are millions of such boxes to sort by size (the 3840x2160 frame of 10M
// micro triangles 1,533 -> 1,423 us), while a frame of few small triangles
// waits on its longest lane (the headline frame 88 -> 107 us at 64).
#define DG_SMALL_MAX_PX 16u
#define DG_SMALL_MAX_PX_MICRO 64u
#define DG_UNIT_PX 32u
#define DG_ITEM_UNITS 8u
// Resolve tile: 32 x tile_rows pixels (tile_rows 8, 16 or 32, chosen per job
// unless the tuning fixes it; DG_TILE_H in the no-allocation path), one CTA of
// 256 threads.
#define DG_TILE_W 32u
#define DG_TILE_H 32u
#define DG_PACK_SHIFT 40

// Device descriptors are 16-byte aligned with sizes that are multiples of 16,
// so kernels read them with 16-byte loads.
struct alignas(16) DgTexDev {
    const uint32_t* words;  // image bytes, little-endian in u32 words, one pad word at the end
    uint64_t len;           // image length in bytes
    uint32_t width, height, comps;
    float fw, fh;           // width as f32, height as f32
    uint32_t small;         // 1 if len < 2^32 and width, height < 2^24 (32-bit texel offsets suffice)
    uint32_t filter;        // DG_FILTER_NEAREST (the reference) or DG_FILTER_BILINEAR (extension)
    uint32_t pad;
};

struct alignas(16) DgMatDev {
    float ka[3], kd[3], ks[3];
    float alpha;
    uint32_t map_ka, map_kd;  // indices into the context's texture table
};

// One frame of a render job (a (scene, canvas) pair).
struct alignas(16) DgFrameDev {
    float M[4][4];       // viewport * orth * persp * view
    float plane[6][4];   // near, far, right, left, top, bottom: (n.x, n.y, n.z, k)
    float cam[3];
    float clear_depth;   // Canvas::depth_max
    float light[DG_MAXL][3];
    uint32_t nlights;
    int32_t exponent;
    float off_x, off_y;  // Canvas::offset
    uint32_t width, height;
    uint64_t* vis;
    uint32_t* colour;
    float* depth;
    uint32_t seg_begin, seg_count;  // this frame's segments (ascending seq_base)
    uint32_t tile_begin, tiles_x;   // this frame's resolve tiles
    uint32_t pix_begin;             // job-wide index of this frame's first pixel
    uint32_t tt_begin;              // job-wide index of this frame's first transparent triangle
    uint32_t epoch;                 // this frame's mark in `cells`
    // One word per 32x32 pixel cell of the canvas, row-major (tiles_x per row):
    // the setup pass writes `epoch` into every cell that a triangle's bounding
    // box reaches, so a cell whose word differs from `epoch` got no fragment
    // this frame and k_resolve writes the clear values there without reading
    // its keys. Null: every tile takes the full path.
    uint32_t* cells;
    uint32_t flags;  // DG_FRAME_PERSPECTIVE: perspective-correct shading attributes (extension)
    uint32_t small_max_px;  // this frame's small-triangle threshold (bounding-box pixels, <= 4096)
};
#define DG_FRAME_PERSPECTIVE 1u
// The frame has at least as many triangles as pixels: its small triangles
// (boxes of at most small_max_px pixels) get no light/halfway rows; the
// resolve pass computes their vertices' vectors for the pixels they win
// (DG_TRI_LAZY in the record's tie word).
#define DG_FRAME_LAZY 2u
static_assert(sizeof(DgTexDev) == 48 && sizeof(DgMatDev) == 48, "descriptor sizes");
inline uint32_t dg_tex_small(uint64_t len, uint64_t w, uint64_t h) {
    return (len < (1ull << 32) && w < (1ull << 24) && h < (1ull << 24)) ? 1u : 0u;
}
static_assert(sizeof(DgFrameDev) % 16 == 0, "frame descriptor size");
// 16-byte words of DgFrameDev read with vector loads by the kernels.
static_assert(offsetof(DgFrameDev, plane) == 64 && offsetof(DgFrameDev, cam) == 160 &&
                  offsetof(DgFrameDev, clear_depth) == 172 && offsetof(DgFrameDev, nlights) == 272 &&
                  offsetof(DgFrameDev, off_x) == 280 && offsetof(DgFrameDev, off_y) == 284,
              "frame descriptor layout");

// The opaque triangles and the vertices of one object within one frame.
struct DgSegDev {
    uint32_t frame;
    uint32_t tri_begin;  // job-wide index of the segment's first triangle
    uint32_t vtx_begin;  // job-wide index of the segment's first vertex (vmask/vshade row)
    uint32_t seq_base;   // frame-local submission index of the first triangle
    uint32_t ntri, nv;
    uint32_t nmats, pad;
    const float4* pos;
    const float4* nrm;
    const float2* uv;
    const uint4* tri_pos;
    const uint4* tri_uv;
    const uint4* tri_nrm;
    const DgMatDev* mats;
    // The object's transparent triangles (the transparent pass): position
    // indices + material, uv indices + mesh within the object (w), normal
    // indices, in their current order (src) and after this frame's painter's
    // sort (dst), which becomes the current order of the next frame.
    uint32_t t_begin;     // job-wide index of the first transparent triangle
    uint32_t nt;          // transparent triangles of the object
    uint32_t tmesh_base;  // job-wide index of the object's first transparent mesh
    uint32_t obj_rank;    // the object's position within its frame
    const uint4* tsrc[3];
    uint4* tdst[3];
};

// Edge constants of one triangle: f_k(x, y) = ((A[k]*x + B[k]*y) + C[k]) - D[k]
// (canvas.rs:597-616 with the products of the vertex coordinates precomputed;
// the per-pixel value is the same IEEE result), k = 0: f_bc (alpha), 1: f_ca
// (beta), 2: f_ab (gama).
struct DgEdges {
    float A[3], B[3], C[3], D[3];
    float den[3];  // f_alpha = f_bc(a), f_beta = f_ca(b), f_gama = f_ab(c)
    uint32_t tie;  // bit k: den[k] * f_k(-1, -1) > 0 (the reference's tie rule); DG_EDGE_FAST
};

// Set in DgEdges.tie when every den is finite and > 0 (edges are stored
// normalized to a den without sign bit): coverage is then a sign test.
#define DG_EDGE_FAST 8u
// Set in a triangle record's tie word when its vertices have no light/halfway
// rows (DG_FRAME_LAZY): shading computes them from the vertex positions, with
// the same functions that fill the rows, so the values are identical.
#define DG_TRI_LAZY 16u

// One triangle (or one clip output of it) as the raster and shade passes read
// it: twelve 16-byte words. Attribute fields hold the three vertices' values
// in x, y, z (clip outputs: the values VertexAttributes arithmetic gives the
// new vertices, canvas.rs:242-291); the w slots carry the triangle's material.
struct alignas(16) DgTriRec {
    DgEdges e;                    // words 0-3
    float da, db, dc, ka_x;       // word 4: vertex depths (eye distances)
    float u[3], ka_y;             // word 5: texture coordinates
    float v[3], ka_z;             // word 6
    float nx[3], kd_x;            // words 7-9: normals
    float ny[3], kd_y;
    float nz[3], kd_z;
    uint32_t vrow[3];             // word 10: rows of the light/halfway table of the three vertices
    float ks_x;
    float ks_y, ks_z;             // word 11
    uint32_t map_ka, map_kd;      // texture table indices
};
static_assert(sizeof(DgTriRec) == 192, "triangle record size");

// A triangle queued for the load-balanced raster pass (32 bytes). Its clipped
// bounding box's pixels, numbered row-major, are cut into units of DG_UNIT_PX
// consecutive pixels, one per lane. Entries of the small-triangle list use the
// same layout with npx holding the box height and nunits unused.
struct alignas(16) DgQueueRec {
    uint32_t rec;     // its DgTriRec
    uint32_t seq;     // frame-local key low word
    uint32_t frame;
    uint32_t xlo, ylo;  // clipped bounding box origin
    uint32_t w;         // bounding box width in pixels
    uint32_t npx;       // bounding box pixels
    uint32_t nunits;    // ceil(npx / DG_UNIT_PX)
};

#define DG_NONE 0xFFFFFFFFu
// Job counters (unsigned long long each), each on its own 128-byte line: the
// hot ones take one atomic per warp or block from every pass, and counters that
// share a line share one L2 slice, which serializes their updates (measured: the
// setup pass of the 3840x2160 frame of 10M micro triangles, 702 -> 639 us).
#define DG_CNT_LINE 16
#define DG_CNT_QUEUE (0 * DG_CNT_LINE)    // (queued records << DG_PACK_SHIFT) | work items
#define DG_CNT_COVERED (1 * DG_CNT_LINE)  // covered pixels (shaded by the resolve pass)
#define DG_CNT_INPLACE (2 * DG_CNT_LINE)  // large triangles rasterized by their own lane (queue or record overflow)
#define DG_CNT_SURV (3 * DG_CNT_LINE)     // triangles that passed the cull pass
#define DG_CNT_TREC (4 * DG_CNT_LINE)     // triangle records requested (statistics)
#define DG_CNT_VROW (5 * DG_CNT_LINE)     // light/halfway rows handed out to clip vertices
#define DG_CNT_UNITS (6 * DG_CNT_LINE)    // work units of the queued triangles
#define DG_CNT_SMALL (7 * DG_CNT_LINE)    // entries of the small-triangle list
#define DG_CNT_TRECX (8 * DG_CNT_LINE)    // records handed out after the first total_tri (multi-output clips)
#define DG_CNT_TFRAG (10 * DG_CNT_LINE)   // transparent fragments emitted
#define DG_NCOUNTERS (12 * DG_CNT_LINE)   // words of the counter array (k_vertex zeroes them: <= 256)

struct DgJobDev {
    const DgFrameDev* frames;
    const DgSegDev* segs;
    uint32_t nframes, nsegs;
    uint32_t total_vtx, total_tri, total_tiles;
    uint32_t shade_stride;  // lights per row of vshade (max over frames)
    float4* vrec;           // [total_vtx] snapped screen centre, eye distance, plane-sign mask bits
    uint16_t* vmask;        // [total_vtx] bit p: plane p has f > 0; bit 8 + p: f <= 0 (near, far, 4 lateral)
    float4* vshade;         // rows [0, total_vtx): job vertices; then rows for clip vertices
    uint32_t vrow_extra;    // rows after total_vtx available to clip vertices
    uint8_t* vmark;         // one byte per job vertex: needs light/halfway vectors (kept zero between jobs)
    uint32_t* surv;         // [total_tri] job-wide indices of the triangles that passed the cull pass
    uint32_t* rec_of;       // [total_tri] first DgTriRec of each surviving triangle, or DG_NONE
    DgTriRec* trec;
    // Per triangle record, (1/w_a, 1/w_b, 1/w_c, 0) of its three vertices' clip
    // w: written and read only for frames with DG_FRAME_PERSPECTIVE (null when
    // no frame of the job has it). ttrec_w: the same for ttrec.
    float4* trec_w;
    float4* ttrec_w;
    uint32_t ext;  // 1: a frame uses perspective-correct interpolation or a texture map the bilinear filter
    uint32_t lazy;  // 1: a frame has DG_FRAME_LAZY
    uint32_t trec_cap;
    uint32_t queue_cap;
    DgQueueRec* queue;
    uint2* items;           // work items: (queue record, first unit)
    uint32_t items_cap;
    DgQueueRec* small;      // small-triangle list (nunits unused), rasterized one triangle per lane
    uint32_t small_cap;
    uint32_t item_units;    // work units per raster work item (>= 1)
    uint32_t total_px;      // pixels of all frames
    uint32_t tile_rows;     // resolve tile height (8, 16 or 32)
    unsigned long long* cnt;  // the job counters (DG_CNT_*, DG_NCOUNTERS words), zero at the start of the job
    const DgTexDev* tex;
    uint32_t ntex;          // entries of tex
    uint32_t* err;
    // Transparent pass (all null/zero when the job has no transparent triangle).
    uint32_t ntt;           // transparent triangles of the job
    uint32_t fcap;          // capacity of the fragment buffers
    uint64_t* tkey[2];      // painter's sort: keys and source slots, [ntt] each
    uint32_t* tval[2];
    DgTriRec* ttrec;        // [4 ntt] records of clip outputs, 4 j + o for sorted slot j
    uint4* tbox;            // [4 ntt] (xlo, ylo, width, frame) of each output's bounding box
    uint2* tmeta;           // [4 ntt] (object rank within the frame, frame-local transparent key)
    float* talpha;          // [4 ntt] material alpha
    uint32_t* tcnt;         // [4 ntt] bounding-box pixels of each output, 0 for none
    unsigned long long* tscan;  // [4 ntt + 1] exclusive prefix sums of tcnt
    uint64_t* fkey[2];      // fragments: (job-wide pixel << 32 | transparent key), output record
    uint32_t* fval[2];
    uint32_t* sort_hist;    // radix sort histograms, 256 per tile of DG_SORT_TILE keys
    uint32_t hist_tiles;    // tiles sort_hist has room for
};

// Launch plan of the transparent pass: the digit shifts of its two radix
// sorts (painter's sort keys, fragment keys) and the grid of its grid-stride
// kernels.
struct DgTransparentPlan {
    uint32_t tsort_shift[8], n_tsort;  // painter's sort digits
    uint32_t fsort_shift[8], n_fsort;  // fragment sort digits
    unsigned blocks;                   // grid of the grid-stride kernels
};

// The descriptors of a small job (one frame, at most DG_INLINE_SEGS segments)
// travel as a kernel parameter of k_vertex instead of a host-to-device copy:
// k_vertex reads them from its parameter and writes them to job.frames and
// job.segs, where the later kernels of the job read them.
#define DG_INLINE_SEGS 4
struct alignas(16) DgInlineDesc {
    DgFrameDev frame;
    DgSegDev segs[DG_INLINE_SEGS];
    uint32_t nsegs;  // 0: the descriptors were copied to the device by the host
    uint32_t pad[3];
};

// Host-side launchers (dg_kernels.cu).
struct DgLaunchCfg {
    unsigned vertex_blocks;  // grid caps / sizes in 256-thread blocks
    unsigned cull_blocks;
    unsigned setup_blocks;
    unsigned queue_blocks;
    const DgInlineDesc* inl;  // host memory, read at launch; null: descriptors already on the device
    DgTransparentPlan tplan;
};
// k_vertex's grid cap: its resident blocks (launch bounds 256 x 8), one wave
// that loops over the vertices (measured against a block per 256 vertices: the
// headline frame 88.8 -> 87.8 us, the stress frame's vertex pass 64 -> 59 us).
#define DG_VERTEX_BLOCKS_PER_SM 8u
#define DG_SETUP_BLOCKS_PER_SM 4u
#define DG_CLIP_DEFER 512u  // k_setup_raster: clipped survivors a block sets up in its second pass
// k_queue_raster's grid: 3 waves of its 4 resident blocks per SM. The passes'
// work items are taken in a fixed strided order, so later waves even out
// blocks that drew short items (measured against 8: a 512x512 frame of a
// 100k-triangle sphere 50.4 -> 46.4 us, the headline frame 89.4 -> 89.1 us).
#define DG_QUEUE_BLOCKS_PER_SM 12u
#define DG_CULL_BLOCKS_PER_SM 32u
#define DG_NKERNELS 5  // vertex, cull, setup_raster, queue_raster, resolve (+ the transparent pass)
#define DG_SORT_TILE 4096u  // keys per radix-sort tile (256 threads x 16)
// Launches the whole pipeline of one job on stream s. ev, if not null, holds
// DG_NKERNELS + 1 events recorded around the kernels (per-kernel timing). The
// first kernel zeroes the job counters when the job has vertices; the caller
// zeroes them otherwise.
cudaError_t dg_launch_job(const DgJobDev& job, const DgLaunchCfg& cfg, cudaStream_t s, cudaEvent_t* ev);
// DRAW_TIMELINE builds: copies the kernel timeline (4 words per kernel, as
// dg_timeline_read returns them) to out after s drains and clears it; false in
// other builds.
bool dg_timeline_copy(unsigned long long* out, cudaStream_t s, cudaError_t* err);
// The transparent pass (dg_transparent.cu), in three parts launched by
// dg_launch_job: part 0 after the opaque setup (painter's sort, gather,
// transparent setup), part 1 after the opaque raster (fragment emission and
// sort), part 2 after the opaque resolve (the ordered blend).
cudaError_t dg_launch_transparent(int part, const DgJobDev& job, const DgTransparentPlan& plan, cudaStream_t s);

// One batch of 2D overlay triangles (Canvas::draw_triangle, canvas.rs:435-575)
// drawn into one canvas in order. The host sets every triangle up (snapped
// centres, clipped bounding box, edges, attributes in rec words 4-6: u, v, the
// vertex colours as packed BGR0 words, the vertex alphas in the w slots) and the
// prefix sums of the boxes' pixels; the GPU rasterizes, sorts the fragments by
// (pixel, triangle) and blends each pixel's fragments in order.
struct DgOverlayJob {
    const DgTriRec* rec;              // [n]
    const uint4* box;                 // [n] (x_min, y_min, width, 0)
    const unsigned long long* scan;   // [n + 1] exclusive prefix sums of the boxes' pixels
    uint32_t n;
    uint32_t width, height;
    uint32_t* colour;                 // the canvas (BGRA, row 0 = top)
    const float* depth;               // y*W+x
    DgTexDev tex;                     // the RGBA map
    uint64_t* fkey[2];                // fragment keys (pixel << 32 | triangle) and triangles
    uint32_t* fval[2];
    uint32_t fcap;
    uint32_t* hist;
    unsigned long long* cnt;          // [0] fragments emitted
    uint32_t* err;
    uint32_t sort_shift[8], n_sort;
};
cudaError_t dg_launch_overlay(const DgOverlayJob& job, unsigned blocks, cudaStream_t s);
// Scratch rows and records sized for a job of T triangles (shared sizing rule).
constexpr uint64_t dg_trec_cap(uint64_t T) { return T + T / 8u + 4096u; }
constexpr uint64_t dg_items_cap(uint64_t queue_cap) { return 2u * queue_cap + 65536u; }
constexpr uint64_t dg_vrow_extra(uint64_t T) { uint64_t x = 65536u + T / 8u; return x < 6u * T + 6u ? x : 6u * T + 6u; }
cudaError_t dg_launch_fill(uint32_t* colour, float* depth, uint64_t n, uint32_t colour_value, float depth_value,
                           int fill_colour, int fill_depth, cudaStream_t s);
cudaError_t dg_launch_vis_reset(uint64_t* vis, uint64_t n, cudaStream_t s);
cudaError_t dg_launch_bgra_to_rgba(const uint32_t* src, uint32_t* dst, uint64_t n, cudaStream_t s);

// Host frame setup without a context (dg_api.cu).
dg_status dg_host_frame_setup(uint64_t width, uint64_t height, const float pos[3], const float dir[3], float ratio,
                              float near_, float far_, float fov_x_deg, float M[4][4], float planes[6][4]);
