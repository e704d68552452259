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
//                   plane-sign masks), vshade float4[V_total*L*2] (light, halfway),
//                   raster-queue records + their work-unit bases, counters
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/draw_gpu.h"

#define DG_MAXL DG_MAX_LIGHTS
#define DG_VIS_EMPTY 0xFFFFFFFFFFFFFFFFull

// Triangles whose clipped bounding box has at most this many pixels are
// rasterized by the warp that set them up (default of DgJobDev.small_max_px);
// larger ones go to the raster queue, whose pixels are spread over all warps
// in units of DG_UNIT_PX row-major bounding-box pixels.
#define DG_SMALL_MAX_PX 32u
#define DG_UNIT_PX 32u
// Resolve tile: 32 x 8 pixels, one CTA of 256 threads.
#define DG_TILE_W 32u
#define DG_TILE_H 8u
#define DG_PACK_SHIFT 40

struct DgTexDev {
    const uint32_t* words;  // image bytes, little-endian in u32 words, one pad word at the end
    uint64_t len;           // image length in bytes
    uint32_t width, height, comps;
    float fw, fh;           // width as f32, height as f32
};

struct DgMatDev {
    float ka[3], kd[3], ks[3];
    float alpha;
    uint32_t map_ka, map_kd;  // indices into the context's texture table
};

// One frame of a render job (a (scene, canvas) pair).
struct DgFrameDev {
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
    uint32_t pad[2];
};

// The opaque triangles and the vertices of one object within one frame.
struct DgSegDev {
    uint32_t frame;
    uint32_t tri_begin;  // job-wide index of the segment's first triangle
    uint32_t vtx_begin;  // job-wide index of the segment's first vertex (vrec/vshade row)
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
};

// A triangle queued for the load-balanced raster pass (64 bytes).
struct DgQueueRec {
    float ax, ay, bx, by, cx, cy;  // snapped centres
    float da, db, dc;              // vertex depths
    uint32_t seq;                  // frame-local key low word
    uint32_t frame;
    uint32_t xlo, ylo;             // clipped bounding box origin
    uint32_t w;                    // bounding box width in pixels
    uint32_t npx;                  // bounding box pixels
    uint32_t nunits;               // ceil(npx / DG_UNIT_PX), 0 if the record is rasterized elsewhere
};

struct DgJobDev {
    const DgFrameDev* frames;
    const DgSegDev* segs;
    uint32_t nframes, nsegs;
    uint32_t total_vtx, total_tri, total_tiles;
    uint32_t shade_stride;  // lights per vertex row of vshade (max over frames)
    float4* vrec;
    float4* vshade;
    uint32_t* vmark;        // one bit per job vertex: needs light/halfway vectors (kept zero between jobs)
    DgQueueRec* queue;
    uint32_t* queue_base;   // first work unit of each record (ascending)
    uint32_t queue_cap;
    uint32_t small_max_px;  // in-warp raster threshold (bounding-box pixels)
    unsigned long long* queue_counter;  // (records << 40) | work units
    unsigned long long* stats;          // [0] covered pixels, [1] queued triangles rasterized in place
    const DgTexDev* tex;
    uint32_t* err;
};

// Host-side launchers (dg_kernels.cu).
cudaError_t dg_launch_vertex(const DgJobDev& job, cudaStream_t s);
// max_blocks / blocks: grid size in 256-thread blocks (the setup grid is also capped by the work).
cudaError_t dg_launch_setup_raster(const DgJobDev& job, unsigned max_blocks, cudaStream_t s);
cudaError_t dg_launch_queue_raster(const DgJobDev& job, unsigned blocks, cudaStream_t s);
#define DG_SETUP_BLOCKS_PER_SM 16u
#define DG_QUEUE_BLOCKS_PER_SM 8u
cudaError_t dg_launch_resolve(const DgJobDev& job, cudaStream_t s);
cudaError_t dg_launch_fill(uint32_t* colour, float* depth, uint64_t n, uint32_t colour_value, float depth_value,
                           int fill_colour, int fill_depth, cudaStream_t s);
cudaError_t dg_launch_vis_reset(uint64_t* vis, uint64_t n, cudaStream_t s);

// Host frame setup without a context (dg_api.cu).
dg_status dg_host_frame_setup(uint64_t width, uint64_t height, const float pos[3], const float dir[3], float ratio,
                              float near_, float far_, float fov_x_deg, float M[4][4], float planes[6][4]);
