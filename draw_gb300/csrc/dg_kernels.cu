// dg_kernels.cu -- sm_103a kernels of the GB300 rasterizer.
//
// Pipeline of one render job (one or many frames), all on one stream:
//   k_vertex        per position vertex: eye distance, projected and snapped
//                   screen centre, plane-sign masks (scene/mod.rs:917-926,
//                   :1047-1058, canvas.rs:585-587)
//   k_cull          per input triangle: lateral and near reject from the sign
//                   masks, back-face cull; survivors are compacted
//   k_setup_raster  per survivor: near/far clipping, triangle records, bounding
//                   box, edge functions; tiny triangles are rasterized by their
//                   warp (pixels of all 32 lanes' boxes flattened with a warp
//                   prefix scan), the others are queued (scene/mod.rs:933-1063,
//                   canvas.rs:585-681)
//   k_queue_raster  light/halfway vectors of the marked vertices, then the
//                   queued triangles' bounding-box pixels in 32-pixel units
//                   spread evenly over all warps
//   k_resolve       per 32 x tile_rows tile: a tile that no triangle box reached
//                   (its 32x32 cell lacks the frame's epoch) gets the clear
//                   values without reading its keys; otherwise empty pixels
//                   get the clear colour and depth, covered ones are compacted into the tile's
//                   shade list and their winning fragment is shaded once
//                   (canvas.rs:682-745, 906-930)
//
// Exactness. The reference writes a fragment when its depth is strictly below
// the stored depth (canvas.rs:923) and processes fragments in submission
// order, so the final pixel is the fragment with the smallest
// (depth, submission index) among those with depth < the clear depth. Each
// covered pixel therefore does one 64-bit atomicMin of
// key = (order-preserving depth bits << 32) | (triangle index * 4 + clip output)
// into the canvas's visibility buffer; the result does not depend on thread
// order. Every expression uses __fadd_rn/__fsub_rn/__fmul_rn/__fdiv_rn/
// __fsqrt_rn in the reference's evaluation order (no contraction), Rust's
// saturating float->int casts, and wrapping usize arithmetic for texel offsets.
#include "dg_device.cuh"

#include <nvtx3/nvToolsExt.h>

namespace {

// ================================================================ kernels
// Each pass is a device function over the whole grid (grid-stride or
// block-uniform loops) wrapped by its kernel; the five kernels run as a chain
// with programmatic dependent launch.
// seg(i) and frame(i) give the job's descriptors (from global memory, or from
// k_vertex's parameter for a small job).
#if DG_TIMELINE
// [kernel][first start, first wait passed, last wait passed, last end]
__device__ unsigned long long g_timeline[DG_NKERNELS][4] = {
    {~0ull, ~0ull, 0ull, 0ull}, {~0ull, ~0ull, 0ull, 0ull}, {~0ull, ~0ull, 0ull, 0ull},
    {~0ull, ~0ull, 0ull, 0ull}, {~0ull, ~0ull, 0ull, 0ull}};
__device__ __forceinline__ unsigned long long timeline_now() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// A block's start on construction, its end on destruction (every return path).
struct TimelineBlock {
    int k;
    __device__ explicit TimelineBlock(int kernel) : k(kernel) {
        if (threadIdx.x == 0) atomicMin(&g_timeline[k][0], timeline_now());
    }
    __device__ ~TimelineBlock() {
        if (threadIdx.x == 0) atomicMax(&g_timeline[k][3], timeline_now());
    }
};
__device__ __forceinline__ void timeline_waited(int k) {
    if (threadIdx.x == 0) {
        const unsigned long long t = timeline_now();
        atomicMin(&g_timeline[k][1], t);
        atomicMax(&g_timeline[k][2], t);
    }
}
#define DG_TL_BLOCK(k) TimelineBlock dg_timeline_block_(k)
#define DG_TL_WAITED(k) timeline_waited(k)
#else
#define DG_TL_BLOCK(k) ((void)0)
#define DG_TL_WAITED(k) ((void)0)
#endif

template <class SEG, class FRM>
__device__ __forceinline__ void dev_vertex(const DgJobDev& job, uint32_t nsegs, SEG seg, FRM frame) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < job.total_vtx; v += stride) {
        uint32_t si = last_le(nsegs, v, [&](uint32_t i) { return seg(i).vtx_begin; });
        const DgSegDev& sg = seg(si);
        const DgFrameDev& fr = frame(sg.frame);
        float4 p4 = __ldg(sg.pos + (v - sg.vtx_begin));
        V3 p = {p4.x, p4.y, p4.z};
        uint32_t mask = 0;
#pragma unroll
        for (int pl = 0; pl < 6; pl++) {
            float f = plane_f(fr, pl, p);
            if (f > 0.0f) mask |= 1u << pl;
            if (f <= 0.0f) mask |= 1u << (8 + pl);
        }
        job.vrec[v] = vertex_screen(fr, p4, mask);
        job.vmask[v] = (uint16_t)mask;
    }
}

// Also zeroes the job counters (the later kernels read them only after waiting
// for this one) and, for a small job, writes the descriptors of its parameter
// `in` to job.frames and job.segs.
__global__ void __launch_bounds__(256, 8) k_vertex(const __grid_constant__ DgJobDev job,
                                                   const __grid_constant__ DgInlineDesc in) {
    DG_TL_BLOCK(0);
    allow_next_kernel();
    DG_TL_WAITED(0);  // the first kernel of a job waits on nothing (a stream-ordered launch)
    if (blockIdx.x == 0) {
        static_assert(DG_NCOUNTERS <= 256, "block 0 of k_vertex zeroes the counters");
        if (threadIdx.x < DG_NCOUNTERS) job.cnt[threadIdx.x] = 0ull;
        if (in.nsegs) {
            constexpr uint32_t fw = sizeof(DgFrameDev) / 8, sw = sizeof(DgSegDev) / 8;
            static_assert(sizeof(DgFrameDev) % 8 == 0 && sizeof(DgSegDev) % 8 == 0, "8-byte words");
            uint2* fd = reinterpret_cast<uint2*>(const_cast<DgFrameDev*>(job.frames));
            uint2* sd = reinterpret_cast<uint2*>(const_cast<DgSegDev*>(job.segs));
            const uint2* fs = reinterpret_cast<const uint2*>(&in.frame);
            const uint2* ss = reinterpret_cast<const uint2*>(in.segs);
            for (uint32_t i = threadIdx.x; i < fw + in.nsegs * sw; i += blockDim.x) {
                if (i < fw)
                    fd[i] = fs[i];
                else
                    sd[i - fw] = ss[i - fw];
            }
        }
    }
    if (in.nsegs)
        dev_vertex(job, in.nsegs, [&](uint32_t i) -> const DgSegDev& { return in.segs[i]; },
                   [&](uint32_t) -> const DgFrameDev& { return in.frame; });
    else
        dev_vertex(job, job.nsegs, [&](uint32_t i) -> const DgSegDev& { return job.segs[i]; },
                   [&](uint32_t i) -> const DgFrameDev& { return job.frames[i]; });
}


// Cull pass: one thread per input triangle. A triangle is dropped when one
// lateral plane has all three vertices at f <= 0 (Triangle::clip_against_planes,
// scene/mod.rs:59-66), when all three are at f <= 0 for the near plane (the
// near clip then outputs nothing, :67-87 with ViewPlane::clip :662-690), or when
// it faces away from the camera (:1016-1027). All three are pure predicates of
// the triangle, so testing them in this order gives the reference's surviving
// set; the plane tests read only the vertex records' sign masks. Survivors are
// appended (in any order: the visibility key carries the submission index).
__device__ __forceinline__ void dev_cull(const DgJobDev& job) {
    __shared__ uint32_t s_warp[8];
    __shared__ unsigned long long s_base;
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t stride = gridDim.x * blockDim.x;
    // block-uniform loop: survivors are appended with one atomic per block
    for (uint32_t base = blockIdx.x * blockDim.x; base < job.total_tri; base += stride) {
        const uint32_t g = base + threadIdx.x;
        bool keep = false;
        if (g < job.total_tri) {
            const uint32_t si = seg_of_tri(job, g);
            const DgSegDev& sg = job.segs[si];
            const uint4 tp = __ldg(sg.tri_pos + (g - sg.tri_begin));
            const uint16_t* vm = job.vmask + sg.vtx_begin;
            const bool ok = DG_IN_RANGE(tp.x < sg.nv && tp.y < sg.nv && tp.z < sg.nv, job.err);
            const uint32_t m = ok ? (uint32_t)__ldg(vm + tp.x) & (uint32_t)__ldg(vm + tp.y) & (uint32_t)__ldg(vm + tp.z)
                                  : 0xFFFFu;
            if (((m >> 8) & 0x3Du) == 0u) {
                const float4 pa = __ldg(sg.pos + tp.x), pb = __ldg(sg.pos + tp.y), pc = __ldg(sg.pos + tp.z);
                const V3 a = {pa.x, pa.y, pa.z}, b = {pb.x, pb.y, pb.z}, c = {pc.x, pc.y, pc.z};
                // Triangle::calc_normal and get_center; skip when (cam - centre) . n <= 0
                const V3 n = vcross(vsub(b, a), vsub(c, b));
                const V3 zero = {0.0f, 0.0f, 0.0f};
                const V3 ctr = vdiv(vadd(vadd(vadd(zero, a), b), c), 3.0f);
                const DgFrameDev& fr = job.frames[sg.frame];
                const V3 cam = {fr.cam[0], fr.cam[1], fr.cam[2]};
                keep = !(vdot(vsub(cam, ctr), n) <= 0.0f);
            }
        }
        const unsigned kb = __ballot_sync(FULL, keep);
        if (lane == 0u) s_warp[wid] = (uint32_t)__popc(kb);
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (uint32_t w = 0; w < 8u; w++) {
                const uint32_t c = s_warp[w];
                s_warp[w] = run;
                run += c;
            }
            s_base = run ? atomicAdd(job.cnt + DG_CNT_SURV, (unsigned long long)run) : 0ull;
        }
        __syncthreads();
        if (keep) job.surv[s_base + s_warp[wid] + __popc(kb & ((1u << lane) - 1u))] = g;
        __syncthreads();  // s_warp and s_base are reused by the next iteration
    }
}

__global__ void __launch_bounds__(256) k_cull(const DgJobDev job) {
    DG_TL_BLOCK(1);
    wait_previous_kernel();
    DG_TL_WAITED(1);
    dev_cull(job);
}


// Setup pass over the cull survivors (dense, one per thread): near/far
// clipping, triangle records, bounding boxes and edge functions; tiny
// triangles are rasterized by their warp, the others are queued
// (scene/mod.rs:1029-1063, canvas.rs:585-681).
// Hands out n consecutive slots of counter c to every lane of the (converged)
// warp with one atomic; returns this lane's first slot.
__device__ __forceinline__ unsigned long long warp_alloc(unsigned long long* c, uint32_t n) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t incl = n;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t v = __shfl_up_sync(FULL, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    unsigned long long old = 0;
    if (total != 0u) {
        if (lane == 31u) old = atomicAdd(c, (unsigned long long)total);
        old = __shfl_sync(FULL, old, 31);
    }
    return old + (incl - n);
}

__device__ __forceinline__ void dev_setup(const DgJobDev& job) {
    __shared__ uint32_t s_records;  // statistics: record requests of the block
    __shared__ uint32_t s_nclip;    // clipped survivors the block deferred
    __shared__ uint32_t s_clip_i[DG_CLIP_DEFER], s_clip_g[DG_CLIP_DEFER];  // their survivor slots and indices
    if (threadIdx.x == 0) {
        s_records = 0u;
        s_nclip = 0u;
    }
    __syncthreads();
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned long long ns64 = __ldcg(job.cnt + DG_CNT_SURV);
    const uint32_t nsurv = (uint32_t)(ns64 < job.total_tri ? ns64 : job.total_tri);
    // Pass 0 sets up the survivors, strided over the grid, but defers those that
    // need near/far clipping (up to DG_CLIP_DEFER per block) to pass 1, where the
    // block's warps set them up 32 at a time: the long clip path then runs with
    // all lanes busy instead of holding a warp of mostly unclipped lanes. Both
    // passes are block-uniform (pass 1 starts after a barrier).
    for (int pass = 0; pass < 2; pass++) {
        uint32_t lim = nsurv, start = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u, step = gridDim.x * blockDim.x;
        if (pass == 1) {
            __syncthreads();
            lim = s_nclip < DG_CLIP_DEFER ? s_nclip : DG_CLIP_DEFER;
            start = threadIdx.x & ~31u;
            step = blockDim.x;
        }
        for (uint32_t base = start; base < lim; base += step) {
            const bool valid = base + lane < lim;
            uint32_t i = base + lane, g = 0;
            if (pass == 1) {
                i = valid ? s_clip_i[base + lane] : 0u;
                g = valid ? s_clip_g[base + lane] : 0u;
            } else if (valid) {
                g = __ldcg(job.surv + i);
            }
            int nout = 0;
            uint32_t si = 0, t = 0, row0 = 0, nrows = 0;
            uint4 tp = make_uint4(0, 0, 0, 0), tuv = tp, tnr = tp;
            float4 r[3];
            bool clipped = false;
            ClipProg P;  // built once per clipped triangle, used by every output
            if (valid) {
                si = seg_of_tri(job, g);
                const DgSegDev& sg = job.segs[si];
                t = g - sg.tri_begin;
                tp = __ldg(sg.tri_pos + t);
                tuv = __ldg(sg.tri_uv + t);  // for the triangle record, loaded alongside the vertex records
                tnr = __ldg(sg.tri_nrm + t);
                triangle_vertices(job, sg, job.frames[sg.frame], tp, r);
                const uint32_t m = __float_as_uint(r[0].w) & __float_as_uint(r[1].w) & __float_as_uint(r[2].w);
                uint32_t dslot = DG_CLIP_DEFER;
                if ((m & 0x3u) == 0x3u) {
                    nout = 1;  // inside near and far: the triangle passes unchanged
                } else if (pass == 0 && (dslot = atomicAdd(&s_nclip, 1u)) < DG_CLIP_DEFER) {
                    s_clip_i[dslot] = i;  // set up in pass 1 (nout stays 0 here)
                    s_clip_g[dslot] = g;
                } else {
                    const DgFrameDev& fr = job.frames[sg.frame];
                    float4 pa = __ldg(sg.pos + tp.x), pb = __ldg(sg.pos + tp.y), pc = __ldg(sg.pos + tp.z);
                    build_clip(fr, V3{pa.x, pa.y, pa.z}, V3{pb.x, pb.y, pb.z}, V3{pc.x, pc.y, pc.z}, P);
                    nout = P.nout;
                    clipped = true;
                    if (nout > 0 && P.nv > 3) nrows = (uint32_t)(P.nv - 3);  // light rows for the new vertices
                }
                // its vertices need light/halfway vectors for shading (in a DG_FRAME_LAZY
                // frame an unclipped triangle is marked below, unless its record is lazy)
                if (nout > 0 && (clipped || !(job.frames[sg.frame].flags & DG_FRAME_LAZY))) {
                    const uint32_t vv[3] = {sg.vtx_begin + tp.x, sg.vtx_begin + tp.y, sg.vtx_begin + tp.z};
                    for (int k = 0; k < 3; k++) job.vmark[vv[k]] = 1u;  // plain stores: every writer writes 1
                }
            }
            // Rows of the light/halfway table for clip vertices, one atomic per warp.
            {
                const unsigned long long r0 = warp_alloc(job.cnt + DG_CNT_VROW, nrows);
                if (nrows != 0u) {
                    if (r0 + nrows <= job.vrow_extra) {
                        row0 = (uint32_t)r0;
                        clip_shade_rows(job, job.frames[job.segs[si].frame], P, job.total_vtx + row0);
                    } else {
                        nrows = DG_NONE;  // no room: k_resolve shades these pixels the long way
                    }
                }
            }
            // Triangle records: a triangle with one output uses record i (its survivor
            // slot); the clip outputs of one with more take consecutive records after
            // the first total_tri (one atomic per warp).
            uint32_t rbase = DG_NONE;
            {
                const uint32_t multi = (nout > 1 && nrows != DG_NONE) ? (uint32_t)nout : 0u;
                const unsigned long long rb = (unsigned long long)job.total_tri + warp_alloc(job.cnt + DG_CNT_TRECX, multi);
                if (nout == 1 && nrows != DG_NONE) {
                    if (i < job.trec_cap) rbase = i;
                } else if (multi && rb + (unsigned long long)nout <= job.trec_cap) {
                    rbase = (uint32_t)rb;
                }
            }
            {
                const uint32_t nrec = __reduce_add_sync(FULL, (uint32_t)nout);
                if (lane == 0u && nrec) atomicAdd(&s_records, nrec);  // 32-bit shared atomic, one per warp
            }
            if (valid) job.rec_of[g] = rbase;  // a deferred triangle's entry is rewritten in pass 1

            for (int rr = 0;; rr++) {
                bool has = rr < nout;
                if (__ballot_sync(FULL, has) == 0u) break;
                RTri tr;
                EdgeSet e;
                bool small = false;  // goes to the small-triangle list
                uint32_t nu = 0;     // work units to queue (0: not queued)
                uint32_t qpx = 0;    // bounding-box pixels of the queued triangle
                bool inplace = false;
                bool boxed = false;  // the triangle has a box (no NaN centre)
                tr.xlo = tr.xhi = tr.ylo = tr.yhi = 0;
                tr.frame = 0;
                if (has) {
                    const DgSegDev& sg = job.segs[si];
                    const DgFrameDev& fr = job.frames[sg.frame];
                    tr.frame = sg.frame;
                    tr.seq = ((sg.seq_base + t) << 2) | (uint32_t)rr;
                    if (!clipped) {
                        tr.ax = r[0].x; tr.ay = r[0].y;
                        tr.bx = r[1].x; tr.by = r[1].y;
                        tr.cx = r[2].x; tr.cy = r[2].y;
                        tr.da = r[0].z; tr.db = r[1].z; tr.dc = r[2].z;
                    } else {
                        clip_output_tri(fr, P, rr, r, tr);
                    }
                    bool nan = isnan(tr.ax) || isnan(tr.ay) || isnan(tr.bx) || isnan(tr.by) || isnan(tr.cx) ||
                               isnan(tr.cy);
                    if (!nan) {  // any NaN centre makes every barycentric NaN: nothing is covered
                        bbox_axis(tr.ax, tr.bx, tr.cx, fr.width, tr.xlo, tr.xhi);
                        bbox_axis(tr.ay, tr.by, tr.cy, fr.height, tr.ylo, tr.yhi);
                        boxed = true;
                        make_edges(tr.ax, tr.ay, tr.bx, tr.by, tr.cx, tr.cy, e);
                        const uint64_t px = (uint64_t)(tr.xhi - tr.xlo + 1u) * (uint64_t)(tr.yhi - tr.ylo + 1u);
                        if ((fr.flags & DG_FRAME_LAZY) && !clipped) {
                            if (rbase != DG_NONE && px <= fr.small_max_px) {
                                e.tie |= DG_TRI_LAZY;  // no rows: shading computes the vertices' vectors
                            } else {
                                const uint32_t vv[3] = {sg.vtx_begin + tp.x, sg.vtx_begin + tp.y, sg.vtx_begin + tp.z};
                                for (int k = 0; k < 3; k++) job.vmark[vv[k]] = 1u;
                            }
                        }
                        if (rbase != DG_NONE) {
                            float4* wout = (fr.flags & DG_FRAME_PERSPECTIVE) && job.trec_w
                                               ? job.trec_w + rbase + (uint32_t)rr
                                               : nullptr;
                            if (!clipped)
                                write_record(job, job.trec + rbase, sg, tp, tuv, tnr, e, r, fr, wout);
                            else
                                write_clip_record(job, job.trec + rbase + (uint32_t)rr, sg, tp, tuv, tnr, e, tr, P, rr,
                                                  job.total_vtx + row0, fr, wout);
                        }
                        if (rbase == DG_NONE) {
                            inplace = true;
                        } else if (px <= fr.small_max_px) {
                            small = true;
                        } else {
                            qpx = (uint32_t)px;  // below 2^31: the canvas has fewer pixels
                            nu = (uint32_t)((px + DG_UNIT_PX - 1u) / DG_UNIT_PX);
                        }
                    }
                }
                // Every fragment of a triangle lies in its box: mark the box's 32x32 cells in
                // the frame's cell map. A box of more than 16 cells is marked by the whole
                // warp, row by row (a near triangle's box can span the canvas).
                {
                    uint32_t* cells = nullptr;
                    uint32_t ep = 0, cw = 0, ncx = 0, ncy = 0;
                    if (boxed) {
                        const DgFrameDev& fm = job.frames[tr.frame];
                        cells = fm.cells;
                        ep = fm.epoch;
                        cw = fm.tiles_x;
                        if (cells != nullptr) {
                            ncx = (tr.xhi >> 5) - (tr.xlo >> 5) + 1u;
                            ncy = (tr.yhi >> 5) - (tr.ylo >> 5) + 1u;
                        }
                    }
                    const uint32_t c0 = (tr.ylo >> 5) * cw + (tr.xlo >> 5), ncell = ncx * ncy;
                    if (ncell <= 16u) {
                        for (uint32_t cy = 0; cy < ncy; cy++)
                            for (uint32_t cx = 0; cx < ncx; cx++) cells[c0 + cy * cw + cx] = ep;
                    }
                    unsigned big = __ballot_sync(FULL, ncell > 16u);
                    while (big) {
                        const int L = __ffs(big) - 1;
                        big &= big - 1u;
                        uint32_t* lc = reinterpret_cast<uint32_t*>(
                            __shfl_sync(FULL, (unsigned long long)reinterpret_cast<uintptr_t>(cells), L));
                        const uint32_t ly = __shfl_sync(FULL, ncy, L), lx = __shfl_sync(FULL, ncx, L);
                        const uint32_t l0 = __shfl_sync(FULL, c0, L), lw = __shfl_sync(FULL, cw, L);
                        const uint32_t le = __shfl_sync(FULL, ep, L);
                        for (uint32_t cy = 0; cy < ly; cy++)
                            for (uint32_t cx = lane; cx < lx; cx += 32u) lc[l0 + cy * lw + cx] = le;
                    }
                }
                // Queue the large triangles of this output index with one 64-bit atomic per warp: it hands out
                // the queue records and their work items together; the warp then writes all its
                // items, each lane taking every 32nd.
                const unsigned qmask = __ballot_sync(FULL, nu != 0u);
                if (qmask) {
                    const uint32_t ni = (nu + job.item_units - 1u) / job.item_units;
                    uint32_t incl = ni, uincl = nu;
    #pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t v = __shfl_up_sync(FULL, incl, o);
                        const uint32_t vu = __shfl_up_sync(FULL, uincl, o);
                        if (lane >= (uint32_t)o) {
                            incl += v;
                            uincl += vu;
                        }
                    }
                    const uint32_t total_items = __shfl_sync(FULL, incl, 31);
                    const uint32_t total_units = __shfl_sync(FULL, uincl, 31);
                    const int leader = __ffs(qmask) - 1;
                    unsigned long long old = 0;
                    if ((int)lane == leader) {
                        old = atomicAdd(job.cnt + DG_CNT_QUEUE,
                                        ((unsigned long long)__popc(qmask) << DG_PACK_SHIFT) | total_items);
                        atomicAdd(job.cnt + DG_CNT_UNITS, (unsigned long long)total_units);
                    }
                    old = __shfl_sync(FULL, old, leader);
                    const uint64_t rec = (old >> DG_PACK_SHIFT) + __popc(qmask & ((1u << lane) - 1u));
                    const uint64_t ibase = (old & ((1ull << DG_PACK_SHIFT) - 1ull)) + (incl - ni);
                    const bool fits = nu != 0u && rec < job.queue_cap && ibase + ni <= job.items_cap;
                    if (fits) {
                        uint4* qd = reinterpret_cast<uint4*>(job.queue + rec);
                        qd[0] = make_uint4(rbase + (uint32_t)rr, tr.seq, tr.frame, tr.xlo);
                        qd[1] = make_uint4(tr.ylo, tr.xhi - tr.xlo + 1u, qpx, nu);
                    } else if (nu != 0u) {
                        inplace = true;  // queue full: this lane rasterizes the box itself
                    }
                    // Items of a lane that did not fit are marked empty (their slots are handed out).
                    // Lanes with at least 32 items: the whole warp writes them, one lane after another.
                    unsigned big = __ballot_sync(FULL, ni >= 32u);
                    while (big) {
                        const int L = __ffs(big) - 1;
                        big &= big - 1u;
                        const uint32_t lni = __shfl_sync(FULL, ni, L);
                        const uint32_t orec = (uint32_t)__shfl_sync(FULL, (unsigned long long)rec, L);
                        const uint64_t oib = __shfl_sync(FULL, (unsigned long long)ibase, L);
                        const bool ofits = __shfl_sync(FULL, fits ? 1u : 0u, L) != 0u;
                        for (uint32_t k = lane; k < lni; k += 32u)
                            if (oib + k < job.items_cap)
                                job.items[oib + k] = ofits ? make_uint2(orec, k * job.item_units) : make_uint2(DG_NONE, 0u);
                    }
                    // The other lanes' items numbered together: item j belongs to the first lane
                    // whose inclusive count exceeds it.
                    const uint32_t ns = ni < 32u ? ni : 0u;
                    uint32_t sincl = ns;
    #pragma unroll
                    for (int o = 1; o < 32; o <<= 1) {
                        const uint32_t v = __shfl_up_sync(FULL, sincl, o);
                        if (lane >= (uint32_t)o) sincl += v;
                    }
                    const uint32_t stotal = __shfl_sync(FULL, sincl, 31);
                    const uint32_t sexcl = sincl - ns;
                    for (uint32_t b0 = 0; b0 < stotal; b0 += 32u) {
                        const uint32_t j = b0 + lane;
                        int lo = 0, hi = 31;
    #pragma unroll
                        for (int it = 0; it < 5; it++) {
                            const int mid = (lo + hi) >> 1;
                            if (__shfl_sync(FULL, sincl, mid) > j)
                                hi = mid;
                            else
                                lo = mid + 1;
                        }
                        const uint32_t orec = (uint32_t)__shfl_sync(FULL, (unsigned long long)rec, lo);
                        const uint64_t oib = __shfl_sync(FULL, (unsigned long long)ibase, lo);
                        const uint32_t oex = __shfl_sync(FULL, sexcl, lo);
                        const bool ofits = __shfl_sync(FULL, fits ? 1u : 0u, lo) != 0u;
                        const uint32_t k = j - oex;  // item index within its record
                        if (j < stotal && oib + k < job.items_cap)
                            job.items[oib + k] = ofits ? make_uint2(orec, k * job.item_units) : make_uint2(DG_NONE, 0u);
                    }
                }
                // Small triangles go to the small-triangle list (one atomic per warp), which the
                // queue pass rasterizes one triangle per lane.
                const unsigned smask = __ballot_sync(FULL, small);
                if (smask) {
                    const int leader = __ffs(smask) - 1;
                    unsigned long long old = 0;
                    if ((int)lane == leader) old = atomicAdd(job.cnt + DG_CNT_SMALL, (unsigned long long)__popc(smask));
                    old = __shfl_sync(FULL, old, leader);
                    const uint64_t slot = old + __popc(smask & ((1u << lane) - 1u));
                    if (small) {
                        if (slot < job.small_cap) {
                            uint4* qd = reinterpret_cast<uint4*>(job.small + slot);
                            qd[0] = make_uint4(rbase + (uint32_t)rr, tr.seq, tr.frame, tr.xlo);
                            qd[1] = make_uint4(tr.ylo, tr.xhi - tr.xlo + 1u, tr.yhi - tr.ylo + 1u, 0u);
                        } else {
                            inplace = true;  // list full
                        }
                    }
                }
                if (inplace) {  // this lane rasterizes the box itself
                    atomicAdd(job.cnt + DG_CNT_INPLACE, 1ull);
                    raster_box(e, tr.da, tr.db, tr.dc, tr.seq, tr.xlo, tr.ylo, tr.xhi - tr.xlo + 1u, tr.yhi - tr.ylo + 1u,
                               job.frames[tr.frame]);
                }
            }
        }
    }
    __syncthreads();
    if (threadIdx.x == 0 && s_records) atomicAdd(job.cnt + DG_CNT_TREC, (unsigned long long)s_records);  // statistics only
}

__global__ void __launch_bounds__(256) k_setup_raster(const DgJobDev job) {
    DG_TL_BLOCK(2);
    wait_previous_kernel();
    DG_TL_WAITED(2);
    dev_setup(job);
}

// The raster queue: the bounding-box pixels of every queued triangle in
// row-major units of DG_UNIT_PX (one pixel per lane), grouped into work items
// of at most job.item_units units that the warps take in a strided order.
// One candidate fragment of a queued triangle (its pixel passed prereject):
// the coverage test with the divisions, the depth, the strict test against the
// clear depth and the keyed minimum.
// rcp (uniform over the warp): the edge set passed edge_rcp_ok and yr holds the
// reciprocals of its three dens.
// The edge set and the vertex depths are read from the record R (cached: every
// call of a work item reads the same words), which keeps them out of the unit
// loop's registers.
__device__ __forceinline__ void finish_fragment(const DgTriRec* R, uint32_t seq, uint32_t x, uint32_t y,
                                                float clear_depth, unsigned long long* vis, uint32_t width, bool rcp,
                                                float3 yr) {
    EdgeSet e;
    load_edges(R, e);
    const float4 dd = __ldg(reinterpret_cast<const float4*>(R) + 4);
    float al, be, ga;
    const float xf = (float)x, yf = (float)y;
    const float n0 = edge_eval(e, 0, xf, yf), n1 = edge_eval(e, 1, xf, yf), n2 = edge_eval(e, 2, xf, yf);
    bool cov;
    if (rcp) {  // the candidate passed the sign test: only the barycentrics remain
        al = div_rcp(n0, e.den[0], yr.x);
        be = div_rcp(n1, e.den[1], yr.y);
        ga = div_rcp(n2, e.den[2], yr.z);
        cov = true;
    } else if (e.tie & DG_EDGE_FAST) {
        al = fD(n0, e.den[0]);
        be = fD(n1, e.den[1]);
        ga = fD(n2, e.den[2]);
        cov = true;
    } else {
        cov = covered_divide(e, n0, n1, n2, al, be, ga);
    }
    if (cov) {
        const float depth = interp(al, be, ga, dd.x, dd.y, dd.z);
        if (depth < clear_depth) atomicMin(vis + (uint64_t)y * width + x, depth_key(depth, seq));
    }
}

__device__ __forceinline__ void dev_queue(const DgJobDev& job) {
    __shared__ uint32_t s_bx[8][64], s_by[8][64];  // per-warp candidate buffers
    __shared__ uint32_t s_sorted[256];             // a group of small triangles in box-size order
    __shared__ uint32_t s_bucket[16];              // their counts, then offsets, per box-size class
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t* bx = s_bx[threadIdx.x >> 5];
    uint32_t* by = s_by[threadIdx.x >> 5];
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    // Prologue: light/halfway vectors of the vertices the setup pass marked, 32
    // vertices per warp; the marks are cleared for the next job.
    const uint32_t ngroups = (job.total_vtx + 31u) >> 5;
    for (uint32_t w = warp; w < ngroups; w += nwarps) {
        const uint32_t v = (w << 5) + lane;
        if (v < job.total_vtx && __ldcg(job.vmark + v)) {
            shade_vertex(job, v);
            job.vmark[v] = 0u;
        }
    }
    const unsigned long long cnt = __ldcg(job.cnt + DG_CNT_QUEUE);
    const uint64_t ni64 = cnt & ((1ull << DG_PACK_SHIFT) - 1ull);
    const uint32_t nitems = (uint32_t)(ni64 < job.items_cap ? ni64 : job.items_cap);
    const unsigned long long ns64 = __ldcg(job.cnt + DG_CNT_SMALL);
    const uint32_t nsmall = (uint32_t)(ns64 < job.small_cap ? ns64 : job.small_cap);
    // Small triangles: one per lane, rasterized by that lane. When there are at
    // least 32 per warp of the grid, a block takes 256 at a time and orders them by
    // box-size class (the bit length of the box's pixel count) in shared memory, so
    // that the lanes of a warp loop over boxes of about the same size
    // (block-uniform loop); fewer go in chunks of 32 to single warps, ahead of the
    // work items.
    const bool sort_small = nsmall >= nwarps * 32u;
    const uint32_t nsgroups = sort_small ? (nsmall + 255u) >> 8 : 0u;
    for (uint32_t gi = blockIdx.x; gi < nsgroups; gi += gridDim.x) {
        if (threadIdx.x < 16u) s_bucket[threadIdx.x] = 0u;
        __syncthreads();
        const uint32_t i = (gi << 8) + threadIdx.x;
        uint32_t cls = 15u, rank = 0;
        if (i < nsmall) {
            const uint4 q1 = __ldcg(reinterpret_cast<const uint4*>(job.small + i) + 1);
            const uint32_t px = q1.y * q1.z;  // at most small_max_px (<= 4096)
            cls = 32u - __clz(px);            // 0..13
            rank = atomicAdd(&s_bucket[cls], 1u);
        }
        __syncthreads();
        if (threadIdx.x == 0) {  // exclusive offsets of the classes; class 15 (no triangle) last
            uint32_t run = 0;
            for (uint32_t c = 0; c < 16u; c++) {
                const uint32_t n = s_bucket[c];
                s_bucket[c] = run;
                run += n;
            }
        }
        __syncthreads();
        if (i < nsmall) s_sorted[s_bucket[cls] + rank] = i;
        __syncthreads();
        const uint32_t nin = nsmall - (gi << 8) < 256u ? nsmall - (gi << 8) : 256u;
        if (threadIdx.x < nin) {
            const uint4* qs = reinterpret_cast<const uint4*>(job.small + s_sorted[threadIdx.x]);
            const uint4 q0 = __ldcg(qs), q1 = __ldcg(qs + 1);
            const DgTriRec* R = job.trec + q0.x;
            EdgeSet e;
            load_edges(R, e);
            const float4 dd = __ldg(reinterpret_cast<const float4*>(R) + 4);
            raster_box(e, dd.x, dd.y, dd.z, q0.y, q0.w, q1.x, q1.y, q1.z, job.frames[q0.z]);
        }
        __syncthreads();  // s_bucket and s_sorted are reused by the next group
    }
    // Work index wi: chunks of 32 small triangles (wi < nchunks), then the work items.
    const uint32_t nchunks = sort_small ? 0u : (nsmall + 31u) >> 5;
    for (uint32_t wi = warp; wi < nchunks + nitems; wi += nwarps) {
        if (wi < nchunks) {
            const uint32_t i = (wi << 5) + lane;
            if (i < nsmall) {
                const uint4* qs = reinterpret_cast<const uint4*>(job.small + i);
                const uint4 q0 = __ldcg(qs), q1 = __ldcg(qs + 1);
                const DgTriRec* R = job.trec + q0.x;
                EdgeSet e;
                load_edges(R, e);
                const float4 dd = __ldg(reinterpret_cast<const float4*>(R) + 4);
                raster_box(e, dd.x, dd.y, dd.z, q0.y, q0.w, q1.x, q1.y, q1.z, job.frames[q0.z]);
            }
            continue;
        }
        const uint32_t it = wi - nchunks;
        const uint2 item = __ldcg(job.items + it);
        if (item.x >= job.queue_cap) continue;  // an item of a triangle that did not fit the queue
        const uint4* qs = reinterpret_cast<const uint4*>(job.queue + item.x);
        const uint4 q0 = __ldcg(qs), q1 = __ldcg(qs + 1);
        const DgTriRec* R = job.trec + q0.x;
        EdgeSet e;
        load_edges(R, e);
        const uint32_t seq = q0.y;
        const DgFrameDev& fr = job.frames[q0.z];
        const float clear_depth = fr.clear_depth;
        unsigned long long* vis = reinterpret_cast<unsigned long long*>(fr.vis);
        const uint32_t width = fr.width;
        const uint32_t xlo = q0.w, ylo = q1.x, w = q1.y, npx = q1.z;
        if (!DG_IN_RANGE(w != 0u && xlo + w <= width && ylo + (npx + w - 1u) / w <= fr.height && q0.x < job.trec_cap,
                         job.err))
            continue;
        const uint32_t u_end = min(q1.w, item.y + job.item_units);
        // Stage A: every lane takes one pixel of the unit and applies the exact,
        // division-free pre-reject; candidates are packed into the warp's buffer.
        // Stage B: whenever 32 candidates are buffered, each lane finishes one of
        // them (the reference's full test with its three divisions, then the
        // depth key), so the division path runs with all lanes busy.
        uint32_t pending = 0;
        const bool fast = (e.tie & DG_EDGE_FAST) != 0u;
        const bool rcp = edge_rcp_ok(e);
        const float3 yr = rcp ? make_float3(__frcp_rn(e.den[0]), __frcp_rn(e.den[1]), __frcp_rn(e.den[2]))
                              : make_float3(0.0f, 0.0f, 0.0f);
        // This lane's pixel k = u * DG_UNIT_PX + lane of the box, as column xx and
        // row yy: one division per item, then a step of DG_UNIT_PX pixels per unit
        // (q32 rows and r32 columns, with at most one carry since xx, r32 < w).
        uint32_t k = item.y * DG_UNIT_PX + lane;
        uint32_t yy = k / w, xx = k - yy * w;
        const uint32_t q32 = DG_UNIT_PX / w, r32 = DG_UNIT_PX - q32 * w;
        // Buffers this unit's candidates and finishes 32 whenever that many are buffered.
        auto push = [&](bool cand, uint32_t x, uint32_t y) {
            const unsigned b = __ballot_sync(FULL, cand);
            if (cand) {
                const uint32_t slot = pending + __popc(b & ((1u << lane) - 1u));
                bx[slot] = x;
                by[slot] = y;
            }
            pending += __popc(b);
            if (pending >= 32u) {
                __syncwarp();
                finish_fragment(R, seq, bx[lane], by[lane], clear_depth, vis, width, rcp, yr);
                __syncwarp();
                if (lane < pending - 32u) {
                    bx[lane] = bx[32u + lane];
                    by[lane] = by[32u + lane];
                }
                __syncwarp();
                pending -= 32u;
            }
        };
        for (uint32_t u = item.y; u < u_end; u++, k += DG_UNIT_PX) {
            bool cand = false;
            const uint32_t x = xlo + xx, y = ylo + yy;
            xx += r32;
            yy += q32;
            if (xx >= w) {
                xx -= w;
                yy++;
            }
            if (k < npx) {
                const float xf = (float)x, yf = (float)y;
                const float n0 = edge_eval(e, 0, xf, yf), n1 = edge_eval(e, 1, xf, yf), n2 = edge_eval(e, 2, xf, yf);
                cand = fast ? covered_signs(e.tie, n0, n1, n2)
                            : !(prereject(n0, e.den[0]) || prereject(n1, e.den[1]) || prereject(n2, e.den[2]));
            }
            push(cand, x, y);
        }
        __syncwarp();
        if (lane < pending) finish_fragment(R, seq, bx[lane], by[lane], clear_depth, vis, width, rcp, yr);
        __syncwarp();
    }
}

// The resolve pass may start only after this kernel's blocks have waited for
// the setup pass, so that its early clear of untouched tiles (k_resolve) reads
// a complete cell map: the wait comes before the launch signal here.
__global__ void __launch_bounds__(256, 4) k_queue_raster(const DgJobDev job) {
    DG_TL_BLOCK(3);
    asm volatile("griddepcontrol.wait;" ::: "memory");
    DG_TL_WAITED(3);
    allow_next_kernel();
    dev_queue(job);
}

// Pixels of tile `tile` whose winning triangle has no record (the record
// buffers were full) kept their keys in phase 1: they are shaded here from the
// mesh (shade_without_record) and their keys reset. The tile's own CTA calls it
// at the end of k_resolve, each thread on the pixels it read in phase 1. Out of
// line, so that the long path costs the main path no registers (the job is a
// __grid_constant__ parameter: its address needs no copy).
template <uint32_t TH>
__device__ __noinline__ void shade_tile_without_records(const DgJobDev& job, uint32_t tile, const float* inv255,
                                                        const DgTexDev* stex) {
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t fi = last_le(job.nframes, tile, [&](uint32_t i) { return job.frames[i].tile_begin; });
    const DgFrameDev& fr = job.frames[fi];
    const uint32_t lt = tile - fr.tile_begin;
    const uint32_t ty = lt / fr.tiles_x, tx = lt - ty * fr.tiles_x;
    const uint32_t x = tx * DG_TILE_W + lane;
    const uint32_t W = fr.width, H = fr.height;
    uint32_t shaded = 0;
    for (uint32_t j = 0; j < TH / 8u; j++) {
        const uint32_t y = ty * TH + wid + 8u * j;
        if (x >= W || y >= H) continue;
        const uint64_t i = (uint64_t)y * W + x;
        const uint64_t key = __ldcg(reinterpret_cast<const unsigned long long*>(fr.vis) + i);
        if (key == DG_VIS_EMPTY) continue;  // empty, or shaded from its record
        fr.vis[i] = DG_VIS_EMPTY;
        float d = 0.0f;
        int errc;
        uint32_t c = shade_without_record(job, fr, (uint32_t)key, x, y, inv255, stex, d, errc);
        if (errc != DG_OK) {
            c = AZUL_BB;
            atomicOr(job.err, 1u << errc);
        }
        fr.depth[i] = d;
        fr.colour[(uint64_t)(H - 1u - y) * W + x] = c;
        shaded++;
    }
    if (shaded) atomicAdd(job.cnt + DG_CNT_COVERED, (unsigned long long)shaded);
}

// Resolve and shade, fused: one 32 x TH tile per CTA of 256 threads (TH = 8,
// 16 or 32: the tile_rows knob).
//  0. If the tile's 32x32 cell does not hold the frame's epoch, no triangle's
//     box reached it and every key is empty: the clear values, and return.
//  1. Each thread reads the visibility keys of TH/8 pixels (rows r, r+8, ...
//     of its column). An empty pixel gets the clear colour and depth
//     (this is Canvas::clear, canvas.rs:425-433); a covered one has its key
//     reset for the next frame and goes into the tile's shade list in shared
//     memory with its triangle record, in row-major order. A covered pixel
//     whose triangle has no record keeps its key for step 3.
//  2. The CTA shades its list densely: the winning fragment of every covered
//     pixel is shaded once (canvas.rs:682-741) and its colour (row H-1-y) and
//     depth (y*W+x) are written (canvas.rs:923-930).
//  3. If a pixel of the tile had no record, shade_tile_without_records.
// The resolve pass's tables, independent of the previous passes: the 256
// quotients byte / 255 and the first DG_SMEM_TEX texture descriptors.
__device__ __forceinline__ void resolve_prologue(const DgJobDev& job, float* inv255, DgTexDev* stex) {
    inv255[threadIdx.x] = fD((float)threadIdx.x, 255.0f);
    const uint32_t nst = job.ntex < DG_SMEM_TEX ? job.ntex : DG_SMEM_TEX;
    for (uint32_t i = threadIdx.x; i < nst * 3u; i += blockDim.x)
        reinterpret_cast<uint4*>(stex)[i] = __ldg(reinterpret_cast<const uint4*>(job.tex) + i);
}

// Canvas::clear (canvas.rs:425-433) of one 32 x TH tile (tile column tx, row ty):
// 16-byte stores of four pixels where the rows are 16-byte aligned.
template <uint32_t TH>
__device__ __forceinline__ void clear_tile(const DgFrameDev& fr, uint32_t tx, uint32_t ty) {
    const uint32_t W = fr.width, H = fr.height;
    const uint32_t x0 = tx * DG_TILE_W;
    const bool vec = (W & 3u) == 0u && x0 + DG_TILE_W <= W &&
                     ((reinterpret_cast<uintptr_t>(fr.depth) | reinterpret_cast<uintptr_t>(fr.colour)) & 15u) == 0u;
    if (vec) {
        const uint32_t r = threadIdx.x >> 3, c = (threadIdx.x & 7u) * 4u;
        const float cd = fr.clear_depth;
        for (uint32_t yy = r; yy < TH; yy += 32u) {
            const uint32_t y = ty * TH + yy;
            if (y < H) {
                *reinterpret_cast<float4*>(fr.depth + (uint64_t)y * W + x0 + c) = make_float4(cd, cd, cd, cd);
                *reinterpret_cast<uint4*>(fr.colour + (uint64_t)(H - 1u - y) * W + x0 + c) =
                    make_uint4(AZUL_BB, AZUL_BB, AZUL_BB, AZUL_BB);
            }
        }
        return;
    }
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t x = x0 + lane;
#pragma unroll
    for (uint32_t j = 0; j < TH / 8u; j++) {
        const uint32_t y = ty * TH + wid + 8u * j;
        if (x < W && y < H) {
            fr.depth[(uint64_t)y * W + x] = fr.clear_depth;
            fr.colour[(uint64_t)(H - 1u - y) * W + x] = AZUL_BB;
        }
    }
}

// One tile of the resolve pass (block-uniform; the tables of resolve_prologue
// must be in place). EXT: the job uses an extension mode (perspective-correct
// interpolation or bilinear fetch); false compiles the reference's shading only.
// LAZY: a frame of the job has DG_FRAME_LAZY (records of small triangles carry
// no light rows).
template <uint32_t TH, bool EXT, bool LAZY>
__device__ __forceinline__ void dev_resolve_tile(const DgJobDev& job, const uint32_t tile, const float* inv255,
                                                 const DgTexDev* stex) {
    __shared__ uint16_t s_pix[DG_TILE_W * TH];  // pixel index within the tile
    __shared__ uint32_t s_val[DG_TILE_W * TH];  // triangle record
    __shared__ uint32_t s_row[33];  // shade-list offset of each tile row; [32] = total
    const uint32_t lane = threadIdx.x & 31u, wid = threadIdx.x >> 5;
    const uint32_t fi = last_le(job.nframes, tile, [&](uint32_t i) { return job.frames[i].tile_begin; });
    const DgFrameDev& fr = job.frames[fi];
    const uint32_t lt = tile - fr.tile_begin;
    const uint32_t ty = lt / fr.tiles_x, tx = lt - ty * fr.tiles_x;
    const uint32_t x = tx * DG_TILE_W + lane;
    const uint32_t W = fr.width, H = fr.height;
    constexpr int R = TH / 8;
    if (fr.cells != nullptr && __ldcg(fr.cells + ((ty * TH) >> 5) * fr.tiles_x + tx) != fr.epoch) {
        // No triangle's box reached the tile's 32x32 cell this frame, so all its
        // keys are empty: the clear values, without reading the keys (block-uniform).
        clear_tile<TH>(fr, tx, ty);
        return;
    }
    uint64_t key[R];
#pragma unroll
    for (int j = 0; j < R; j++) {  // all loads first: R keys in flight per thread
        const uint32_t y = ty * TH + wid + 8u * j;
        key[j] = (x < W && y < H) ? __ldcg(reinterpret_cast<const unsigned long long*>(fr.vis) + (uint64_t)y * W + x)
                                  : DG_VIS_EMPTY - 1ull;  // outside the canvas
    }
    uint32_t val[R];
    unsigned hit[R];
    int no_record = 0;
#pragma unroll
    for (int j = 0; j < R; j++) {
        const uint32_t y = ty * TH + wid + 8u * j;
        const uint64_t i = (uint64_t)y * W + x;
        const bool covered_px = key[j] < DG_VIS_EMPTY - 1ull;
        val[j] = DG_NONE;
        if (key[j] == DG_VIS_EMPTY) {
            fr.depth[i] = fr.clear_depth;
            fr.colour[(uint64_t)(H - 1u - y) * W + x] = AZUL_BB;
        } else if (covered_px) {
            // the triangle record of the key: segment of the submission index, then rec_of
            const uint32_t seq = (uint32_t)key[j];
            const uint32_t tl = seq >> 2;
            const uint32_t si = fr.seg_begin + last_le(fr.seg_count, tl, [&](uint32_t k) {
                                    return job.segs[fr.seg_begin + k].seq_base;
                                });
            const DgSegDev& sg = job.segs[si];
            const uint32_t t = tl - sg.seq_base;
            if (t < sg.ntri) val[j] = __ldg(job.rec_of + sg.tri_begin + t);
            const uint32_t o = (uint32_t)key[j] & 3u;
            if (val[j] != DG_NONE && (uint64_t)val[j] + o < job.trec_cap) {
                val[j] += o;
                fr.vis[i] = DG_VIS_EMPTY;
            } else {
                val[j] = DG_NONE;  // shaded at the end, from the mesh, which resets the key
                no_record = 1;
            }
        }
        hit[j] = __ballot_sync(FULL, covered_px && val[j] != DG_NONE);
        if (lane == 0) s_row[wid + 8u * j] = __popc(hit[j]);
    }
    const int any_no_record = __syncthreads_or(no_record);
    if (wid == 0) {  // exclusive scan of the TH row counts
        const uint32_t c = lane < TH ? s_row[lane] : 0u;
        uint32_t incl = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t v = __shfl_up_sync(FULL, incl, o);
            if (lane >= (uint32_t)o) incl += v;
        }
        s_row[lane] = incl - c;
        if (lane == 31u) {
            s_row[32] = incl;
            if (incl) atomicAdd(job.cnt + DG_CNT_COVERED, (unsigned long long)incl);
        }
    }
    __syncthreads();
#pragma unroll
    for (int j = 0; j < R; j++) {
        if ((hit[j] >> lane) & 1u) {
            const uint32_t row = wid + 8u * j;
            const uint32_t slot = s_row[row] + __popc(hit[j] & ((1u << lane) - 1u));
            s_pix[slot] = (uint16_t)(row * DG_TILE_W + lane);
            s_val[slot] = val[j];
        }
    }
    __syncthreads();
    const uint32_t n = s_row[32];
    for (uint32_t k = threadIdx.x; k < n; k += blockDim.x) {
        const uint32_t pe = s_pix[k];
        const uint32_t px = tx * DG_TILE_W + (pe & 31u), py = ty * TH + (pe >> 5);
        float d = 0.0f;
        int errc;
        const float4* wp = EXT && (fr.flags & DG_FRAME_PERSPECTIVE) && job.trec_w ? job.trec_w + s_val[k] : nullptr;
        uint32_t c = shade_from_record<EXT, LAZY>(job, fr, job.trec + s_val[k], px, py, inv255, stex, d, errc, wp);
        if (errc != DG_OK) c = AZUL_BB;
        // one error-word update per warp (every pixel of a bad job may fail)
        const unsigned act = __activemask();
        const uint32_t bits = __reduce_or_sync(act, errc != DG_OK ? 1u << errc : 0u);
        if (bits != 0u && lane == (uint32_t)(__ffs(act) - 1)) atomicOr(job.err, bits);
        fr.depth[(uint64_t)py * W + px] = d;
        fr.colour[(uint64_t)(H - 1u - py) * W + px] = c;
    }
    // pixels whose triangle has no record: shaded the long way (block-uniform)
    if (any_no_record) shade_tile_without_records<TH>(job, tile, inv255, stex);
}

template <uint32_t TH, bool EXT, bool LAZY>
__global__ void __launch_bounds__(256, 4) k_resolve(const __grid_constant__ DgJobDev job) {
    DG_TL_BLOCK(4);  // tiles cleared before the wait record no wait
    __shared__ float inv255[256];
    __shared__ DgTexDev stex[DG_SMEM_TEX];
    if (job.ntt == 0u) {
        // A tile that no triangle box reached is cleared before waiting for the
        // raster pass: its keys are all empty, and the cell map it reads is complete
        // (k_queue_raster signals this kernel only after it waited for the setup
        // pass). With a transparent pass, the kernel before this one is not the queue
        // pass, and every tile waits.
        const uint32_t tile = blockIdx.x;
        const uint32_t fi = last_le(job.nframes, tile, [&](uint32_t i) { return job.frames[i].tile_begin; });
        const DgFrameDev& fr = job.frames[fi];
        const uint32_t lt = tile - fr.tile_begin;
        const uint32_t ty = lt / fr.tiles_x, tx = lt - ty * fr.tiles_x;
        if (fr.cells != nullptr && __ldcg(fr.cells + ((ty * TH) >> 5) * fr.tiles_x + tx) != fr.epoch) {
            clear_tile<TH>(fr, tx, ty);  // (block-uniform) without the shading tables
            return;
        }
    }
    resolve_prologue(job, inv255, stex);
    wait_previous_kernel();
    DG_TL_WAITED(4);
    dev_resolve_tile<TH, EXT, LAZY>(job, blockIdx.x, inv255, stex);
}

__global__ void k_fill(uint32_t* colour, float* depth, uint64_t n, uint32_t cv, float dv, int fc, int fd) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (fc) colour[i] = cv;
        if (fd) depth[i] = dv;
    }
}

// The RGBA view of a BGRA frame: bytes 0 and 2 of every pixel swapped, the
// fourth byte kept (Application::export_frame_as, app/mod.rs:345-350).
__global__ void k_bgra_to_rgba(const uint32_t* src, uint32_t* dst, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t s = src[i];
        dst[i] = (s & 0xFF00FF00u) | ((s >> 16) & 0xFFu) | ((s & 0xFFu) << 16);
    }
}

__global__ void k_vis_reset(uint64_t* vis, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        vis[i] = DG_VIS_EMPTY;
}

}  // namespace

// NVTX ranges name each pass's launch on a profiler's timeline (nvtx3 is
// header-only; without an attached tool a range costs a branch).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

bool dg_timeline_copy(unsigned long long* out, cudaStream_t s, cudaError_t* err) {
#if DG_TIMELINE
    unsigned long long init[DG_NKERNELS][4];
    for (int k = 0; k < DG_NKERNELS; k++) {
        init[k][0] = init[k][1] = ~0ull;
        init[k][2] = init[k][3] = 0ull;
    }
    cudaError_t e = cudaStreamSynchronize(s);
    if (e == cudaSuccess) e = cudaMemcpyFromSymbol(out, g_timeline, sizeof(init));
    if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_timeline, init, sizeof(init));
    *err = e;
    return true;
#else
    (void)out;
    (void)s;
    *err = cudaSuccess;
    return false;
#endif
}

cudaError_t dg_launch_job(const DgJobDev& job, const DgLaunchCfg& cfg, cudaStream_t s, cudaEvent_t* ev) {
    NvtxRange job_range("draw_gb300 render job");
    cudaError_t e;
    auto mark = [&](int i) { return ev ? cudaEventRecord(ev[i], s) : cudaSuccess; };
    if ((e = mark(0)) != cudaSuccess) return e;
    if (job.total_vtx) {
        NvtxRange r("k_vertex");
        DgInlineDesc none;
        if (!cfg.inl) none.nsegs = 0;
        const unsigned vb = cfg.vertex_blocks < 1u ? 1u : cfg.vertex_blocks;
        k_vertex<<<grid_for(job.total_vtx, vb), 256, 0, s>>>(job, cfg.inl ? *cfg.inl : none);
        if ((e = cudaGetLastError()) != cudaSuccess) return e;
    }
    if ((e = mark(1)) != cudaSuccess) return e;
    if (job.total_tri) {
        NvtxRange r("k_cull");
        const unsigned cb = cfg.cull_blocks < 1u ? 1u : cfg.cull_blocks;
        if ((e = launch_dependent(k_cull, grid_for(job.total_tri, cb), 256, job, s)) != cudaSuccess) return e;
    }
    if ((e = mark(2)) != cudaSuccess) return e;
    if (job.total_tri) {
        NvtxRange r("k_setup_raster");
        const unsigned sb = cfg.setup_blocks < 1u ? 1u : cfg.setup_blocks;
        if ((e = launch_dependent(k_setup_raster, grid_for(job.total_tri, sb), 256, job, s)) != cudaSuccess) return e;
    }
    if ((e = mark(3)) != cudaSuccess) return e;
    // transparent pass, part 0: painter's sort and setup (its vertices join the
    // lighting prologue of the queue pass)
    if ((e = dg_launch_transparent(0, job, cfg.tplan, s)) != cudaSuccess) return e;
    if (job.total_tri || job.ntt) {
        NvtxRange r("k_queue_raster");
        const unsigned qb = cfg.queue_blocks < 1u ? 1u : cfg.queue_blocks;
        if ((e = launch_dependent(k_queue_raster, qb, 256, job, s)) != cudaSuccess) return e;
    }
    if ((e = mark(4)) != cudaSuccess) return e;
    // part 1: transparent fragments, read against the opaque winners' keys
    if ((e = dg_launch_transparent(1, job, cfg.tplan, s)) != cudaSuccess) return e;
    if (job.total_tiles) {
        NvtxRange r("k_resolve");
        using KR = void (*)(const DgJobDev);
        // [lazy][ext][tile rows 8, 16, 32]
        static const KR kr_table[2][2][3] = {
            {{k_resolve<8, false, false>, k_resolve<16, false, false>, k_resolve<32, false, false>},
             {k_resolve<8, true, false>, k_resolve<16, true, false>, k_resolve<32, true, false>}},
            {{k_resolve<8, false, true>, k_resolve<16, false, true>, k_resolve<32, false, true>},
             {k_resolve<8, true, true>, k_resolve<16, true, true>, k_resolve<32, true, true>}}};
        const KR kr = kr_table[job.lazy ? 1 : 0][job.ext ? 1 : 0][job.tile_rows == 8u ? 0 : job.tile_rows == 16u ? 1 : 2];
        if ((e = launch_dependent(kr, job.total_tiles, 256, job, s)) != cudaSuccess) return e;
    }
    // part 2: the ordered blend over the opaque colours
    if ((e = dg_launch_transparent(2, job, cfg.tplan, s)) != cudaSuccess) return e;
    return mark(5);
}

cudaError_t dg_launch_fill(uint32_t* colour, float* depth, uint64_t n, uint32_t colour_value, float depth_value,
                           int fill_colour, int fill_depth, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_fill<<<grid_for(n, 4096u), 256, 0, s>>>(colour, depth, n, colour_value, depth_value, fill_colour, fill_depth);
    return cudaGetLastError();
}

cudaError_t dg_launch_bgra_to_rgba(const uint32_t* src, uint32_t* dst, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_bgra_to_rgba<<<grid_for(n, 4096u), 256, 0, s>>>(src, dst, n);
    return cudaGetLastError();
}

cudaError_t dg_launch_vis_reset(uint64_t* vis, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_vis_reset<<<grid_for(n, 4096u), 256, 0, s>>>(vis, n);
    return cudaGetLastError();
}
