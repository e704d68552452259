// dg_transparent.cu -- the transparent pass of Scene::render on the GPU
// (scene/mod.rs:1088-1247 with canvas.rs:906-930 and the Pixel arithmetic of
// canvas.rs:136-169), and the 2D overlay triangles of Canvas::draw_triangle
// (canvas.rs:435-575), the other order-dependent blend of the reference.
//
// In the reference, each object draws its opaque meshes with depth writes on,
// then its transparent meshes with depth writes off: every transparent mesh is
// first re-sorted in place by descending distance of its triangle centres from
// the camera (a stable sort; the order persists into the next frame), then its
// triangles are clipped and rasterized, and every fragment whose depth is below
// the depth buffer blends into the colour buffer:
//   colour = bg * (1 - alpha) + colour * alpha
// with each product truncated to u8 and the sum wrapping per channel.
//
// The order-independent formulation used here: let j* be the pixel's winning
// opaque fragment (the last opaque write) and d* its depth. Transparent
// fragments submitted before j* are overwritten by it; those after it (objects
// at or after j*'s object) see the depth buffer at d*. So the final colour is
// the opaque result blended, in submission order, with exactly the transparent
// fragments that come from an object at or after j*'s and whose depth is < d*
// (d* = the clear depth and every object qualifies when no opaque fragment
// covers the pixel). The pass:
//   part 0 (after the opaque setup): per-mesh painter's sort keys, a stable LSD
//          radix sort, the permutation of the triangle arrays into the new
//          persistent order, and the transparent setup (clipping, triangle
//          records, bounding boxes, vertices marked for lighting);
//   part 1 (after the opaque raster, while the visibility keys still hold j*):
//          a prefix sum over the outputs' bounding-box pixels, rasterization of
//          every bounding-box pixel with the exact coverage test, emission of
//          the qualifying fragments as (pixel, submission key) pairs and a
//          radix sort of them;
//   part 2 (after the opaque resolve has written the opaque colours): each
//          pixel's fragments are shaded and blended in submission order.
#include "dg_device.cuh"

namespace {

// ------------------------------------------------------------ radix sort
// Stable LSD radix sort of 64-bit keys with 32-bit values, one 8-bit digit per
// pass: per-tile digit histograms, one exclusive scan over (digit, tile), and a
// scatter that ranks keys within each tile in their original order (a warp's
// keys with __match_any_sync, then warp by warp).
struct DgSortArgs {
    const uint64_t* key_in;
    const uint32_t* val_in;
    uint64_t* key_out;
    uint32_t* val_out;
    uint32_t* hist;                   // 256 per tile, digit-major
    const unsigned long long* n_dev;  // element count on the device, or null for n_max
    uint32_t n_max;
    uint32_t shift;
};
constexpr uint32_t kSortItems = DG_SORT_TILE / 256u;  // keys per thread and tile

__device__ __forceinline__ uint32_t sort_count(const DgSortArgs& a) {
    if (!a.n_dev) return a.n_max;
    const unsigned long long n = __ldcg(a.n_dev);
    return (uint32_t)(n < a.n_max ? n : a.n_max);
}

__global__ void __launch_bounds__(256) k_sort_hist(const DgSortArgs a) {
    __shared__ uint32_t h[256];
    wait_previous_kernel();
    const uint32_t n = sort_count(a);
    const uint32_t ntiles = (n + DG_SORT_TILE - 1u) / DG_SORT_TILE;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        h[threadIdx.x] = 0u;
        __syncthreads();
        for (uint32_t i = 0; i < kSortItems; i++) {
            const uint32_t idx = tile * DG_SORT_TILE + i * 256u + threadIdx.x;
            if (idx < n) atomicAdd(&h[(uint32_t)(a.key_in[idx] >> a.shift) & 255u], 1u);
        }
        __syncthreads();
        a.hist[threadIdx.x * ntiles + tile] = h[threadIdx.x];
        __syncthreads();
    }
}

// Exclusive scan of n u32 counts in place (one block of 1024 threads, each a
// contiguous chunk); with sums64 set, writes u64 prefixes there instead and
// the total at sums64[n].
__device__ __forceinline__ void block_scan_1024(uint32_t* data, uint32_t n, unsigned long long* sums64) {
    __shared__ unsigned long long part[1024];
    const uint32_t chunk = (n + 1023u) / 1024u;
    const uint32_t b = threadIdx.x * chunk;
    const uint32_t e = b + chunk < n ? b + chunk : n;
    unsigned long long sum = 0;
    for (uint32_t i = b; i < e; i++) sum += data[i];
    part[threadIdx.x] = sum;
    __syncthreads();
    for (uint32_t o = 1; o < 1024u; o <<= 1) {
        const unsigned long long v = threadIdx.x >= o ? part[threadIdx.x - o] : 0ull;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    unsigned long long run = part[threadIdx.x] - sum;
    for (uint32_t i = b; i < e; i++) {
        const uint32_t c = data[i];
        if (sums64)
            sums64[i] = run;
        else
            data[i] = (uint32_t)run;
        run += c;
    }
    if (sums64 && threadIdx.x == 1023u) sums64[n] = part[1023];
}

__global__ void __launch_bounds__(1024) k_sort_scan(const DgSortArgs a) {
    wait_previous_kernel();
    const uint32_t n = sort_count(a);
    block_scan_1024(a.hist, 256u * ((n + DG_SORT_TILE - 1u) / DG_SORT_TILE), nullptr);
}

__global__ void __launch_bounds__(256) k_sort_scatter(const DgSortArgs a) {
    __shared__ uint32_t wc[8][257];  // per-warp digit counts ([256]: keys past the end)
    wait_previous_kernel();
    const uint32_t n = sort_count(a);
    const uint32_t ntiles = (n + DG_SORT_TILE - 1u) / DG_SORT_TILE;
    const uint32_t lane = threadIdx.x & 31u, w = threadIdx.x >> 5;
    for (uint32_t tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        for (uint32_t i = threadIdx.x; i < 8u * 257u; i += 256u) (&wc[0][0])[i] = 0u;
        __syncthreads();
        uint32_t dig[kSortItems], rank[kSortItems];
        const uint32_t base = tile * DG_SORT_TILE + w * (DG_SORT_TILE / 8u);
#pragma unroll
        for (uint32_t i = 0; i < kSortItems; i++) {  // the warp's keys in their order
            const uint32_t idx = base + i * 32u + lane;
            const uint32_t d = idx < n ? (uint32_t)(a.key_in[idx] >> a.shift) & 255u : 256u;
            const unsigned peers = __match_any_sync(0xFFFFFFFFu, d);
            const uint32_t before = wc[w][d];
            __syncwarp();
            if (lane == (uint32_t)(__ffs(peers) - 1)) wc[w][d] = before + (uint32_t)__popc(peers);
            __syncwarp();
            dig[i] = d;
            rank[i] = before + (uint32_t)__popc(peers & ((1u << lane) - 1u));
        }
        __syncthreads();
        {  // offsets of each warp's keys among the tile's keys of the same digit
            uint32_t run = 0;
            for (uint32_t ww = 0; ww < 8u; ww++) {
                const uint32_t c = wc[ww][threadIdx.x];
                wc[ww][threadIdx.x] = run;
                run += c;
            }
        }
        __syncthreads();
#pragma unroll
        for (uint32_t i = 0; i < kSortItems; i++) {
            const uint32_t idx = base + i * 32u + lane;
            if (idx < n) {
                const uint32_t d = dig[i];
                const uint32_t pos = a.hist[d * ntiles + tile] + wc[w][d] + rank[i];
                a.key_out[pos] = a.key_in[idx];
                a.val_out[pos] = a.val_in[idx];
            }
        }
        __syncthreads();
    }
}

// One pass per shift; an even number of passes leaves the result in buffer 0.
cudaError_t radix_sort(uint64_t* const key[2], uint32_t* const val[2], uint32_t* hist,
                       const unsigned long long* n_dev, uint32_t n_max, const uint32_t* shifts, uint32_t npass,
                       unsigned blocks, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    const unsigned tiles = (n_max + DG_SORT_TILE - 1u) / DG_SORT_TILE;
    const unsigned grid = tiles < blocks ? (tiles ? tiles : 1u) : blocks;
    for (uint32_t p = 0; p < npass && e == cudaSuccess; p++) {
        DgSortArgs a;
        a.key_in = key[p & 1u];
        a.val_in = val[p & 1u];
        a.key_out = key[(p + 1u) & 1u];
        a.val_out = val[(p + 1u) & 1u];
        a.hist = hist;
        a.n_dev = n_dev;
        a.n_max = n_max;
        a.shift = shifts[p];
        if ((e = launch_dependent(k_sort_hist, grid, 256, a, s)) != cudaSuccess) break;
        if ((e = launch_dependent(k_sort_scan, 1u, 1024, a, s)) != cudaSuccess) break;
        e = launch_dependent(k_sort_scatter, grid, 256, a, s);
    }
    return e;
}

// ----------------------------------------------------------- part 0
__device__ __forceinline__ uint32_t seg_of_ttri(const DgJobDev& job, uint32_t j) {
    return last_le(job.nsegs, j, [&](uint32_t i) { return job.segs[i].t_begin; });
}

// Painter's sort keys, scene/mod.rs:1100-1115: the distance of each
// triangle's centre (a + b + c) / 3.0 from the camera, in descending
// f32::total_cmp order, behind the job-wide index of its mesh; the value is
// the triangle's current slot.
__global__ void __launch_bounds__(256) k_tkeys(const DgJobDev job) {
    wait_previous_kernel();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < job.ntt; j += stride) {
        const DgSegDev& sg = job.segs[seg_of_ttri(job, j)];
        const DgFrameDev& fr = job.frames[sg.frame];
        const uint32_t loc = j - sg.t_begin;
        const uint4 tp = __ldg(sg.tsrc[0] + loc);
        const uint32_t mesh = __ldg(sg.tsrc[1] + loc).w;
        const float4 pa = __ldg(sg.pos + tp.x), pb = __ldg(sg.pos + tp.y), pc = __ldg(sg.pos + tp.z);
        const V3 ctr = vdiv(vadd(vadd(V3{pa.x, pa.y, pa.z}, V3{pb.x, pb.y, pb.z}), V3{pc.x, pc.y, pc.z}), 3.0f);
        const float dist = vnorm(vsub(ctr, V3{fr.cam[0], fr.cam[1], fr.cam[2]}));  // Vec3::dist, linalg.rs:177-180
        const uint32_t bits = __float_as_uint(dist);
        const uint32_t ord = (bits & 0x80000000u) ? ~bits : (bits | 0x80000000u);  // total_cmp order
        job.tkey[0][j] = ((uint64_t)(sg.tmesh_base + mesh) << 32) | (uint64_t)(~ord);
        job.tval[0][j] = j;
    }
}

// The new persistent order: slot j receives the triangle the sort put there.
__global__ void __launch_bounds__(256) k_tgather(const DgJobDev job) {
    wait_previous_kernel();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < job.ntt; j += stride) {
        const DgSegDev& sg = job.segs[seg_of_ttri(job, j)];
        const uint32_t src = job.tval[0][j] - sg.t_begin;  // same mesh, so the same segment
        const uint32_t dst = j - sg.t_begin;
#pragma unroll
        for (int k = 0; k < 3; k++) sg.tdst[k][dst] = __ldg(sg.tsrc[k] + src);
    }
}

// Transparent setup, one sorted triangle per thread: lateral reject and
// near/far clipping (no back-face test in this pass, scene/mod.rs:1117-1227),
// a triangle record and a bounding box per clip output (4 j + o), light rows
// of the clip vertices at total_vtx + vrow_extra + 6 j.
__global__ void __launch_bounds__(256) k_tsetup(const DgJobDev job) {
    wait_previous_kernel();
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < job.ntt; j += stride) {
        const uint32_t si = seg_of_ttri(job, j);
        const DgSegDev& sg = job.segs[si];
        const DgFrameDev& fr = job.frames[sg.frame];
        const uint32_t loc = j - sg.t_begin;
        const uint4 tp = __ldg(sg.tdst[0] + loc), tuv = __ldg(sg.tdst[1] + loc), tnr = __ldg(sg.tdst[2] + loc);
        float4 r[3];
        triangle_vertices(job, sg, fr, tp, r);
        const uint32_t m = __float_as_uint(r[0].w) & __float_as_uint(r[1].w) & __float_as_uint(r[2].w);
        const uint32_t rowbase = job.total_vtx + job.vrow_extra + 6u * j;
        ClipProg P;
        int nout;
        bool clipped = false;
        if ((m >> 8) & 0x3Cu) {
            nout = 0;  // outside a lateral plane (scene/mod.rs:59-66)
        } else if ((m & 0x3u) == 0x3u) {
            nout = 1;  // inside near and far
        } else {
            float4 pa = __ldg(sg.pos + tp.x), pb = __ldg(sg.pos + tp.y), pc = __ldg(sg.pos + tp.z);
            build_clip(fr, V3{pa.x, pa.y, pa.z}, V3{pb.x, pb.y, pb.z}, V3{pc.x, pc.y, pc.z}, P);
            nout = P.nout;
            clipped = true;
            if (nout > 0 && P.nv > 3) clip_shade_rows(job, fr, P, rowbase);
        }
        if (nout > 0) {  // its vertices need light/halfway vectors for shading
            const uint32_t vv[3] = {sg.vtx_begin + tp.x, sg.vtx_begin + tp.y, sg.vtx_begin + tp.z};
            for (int k = 0; k < 3; k++) job.vmark[vv[k]] = 1u;
        }
        const float alpha = tp.w < sg.nmats ? __ldg(&sg.mats[tp.w].alpha) : 1.0f;
        const uint32_t tseq = (j - fr.tt_begin) << 2;
        for (int o = 0; o < 4; o++) {
            const uint32_t ri = 4u * j + (uint32_t)o;
            uint32_t px = 0;
            if (o < nout) {
                RTri tr;
                if (!clipped) {
                    tr.ax = r[0].x; tr.ay = r[0].y;
                    tr.bx = r[1].x; tr.by = r[1].y;
                    tr.cx = r[2].x; tr.cy = r[2].y;
                    tr.da = r[0].z; tr.db = r[1].z; tr.dc = r[2].z;
                } else {
                    clip_output_tri(fr, P, o, r, tr);
                }
                const bool nan = isnan(tr.ax) || isnan(tr.ay) || isnan(tr.bx) || isnan(tr.by) || isnan(tr.cx) ||
                                 isnan(tr.cy);
                if (!nan) {  // any NaN centre makes every barycentric NaN: nothing is covered
                    EdgeSet e;
                    bbox_axis(tr.ax, tr.bx, tr.cx, fr.width, tr.xlo, tr.xhi);
                    bbox_axis(tr.ay, tr.by, tr.cy, fr.height, tr.ylo, tr.yhi);
                    make_edges(tr.ax, tr.ay, tr.bx, tr.by, tr.cx, tr.cy, e);
                    float4* wout = (fr.flags & DG_FRAME_PERSPECTIVE) && job.ttrec_w ? job.ttrec_w + ri : nullptr;
                    if (!clipped)
                        write_record(job, job.ttrec + ri, sg, tp, tuv, tnr, e, r, fr, wout);
                    else
                        write_clip_record(job, job.ttrec + ri, sg, tp, tuv, tnr, e, tr, P, o, rowbase, fr, wout);
                    px = (tr.xhi - tr.xlo + 1u) * (tr.yhi - tr.ylo + 1u);  // below 2^31: the canvas is smaller
                    job.tbox[ri] = make_uint4(tr.xlo, tr.ylo, tr.xhi - tr.xlo + 1u, sg.frame);
                    job.tmeta[ri] = make_uint2(sg.obj_rank, tseq | (uint32_t)o);
                    job.talpha[ri] = alpha;
                }
            }
            job.tcnt[ri] = px;
        }
    }
}

// ----------------------------------------------------------- part 1
__global__ void __launch_bounds__(1024) k_tscan(const DgJobDev job) {
    wait_previous_kernel();
    block_scan_1024(job.tcnt, 4u * job.ntt, job.tscan);
}

// The depth of a visibility key (the inverse of depth_key's order-preserving map).
__device__ __forceinline__ float key_depth(uint64_t key) {
    const uint32_t hi = (uint32_t)(key >> 32);
    return __uint_as_float((hi & 0x80000000u) ? (hi & 0x7FFFFFFFu) : ~hi);
}

// Every bounding-box pixel of every transparent output, numbered through the
// prefix sums: the exact coverage test, the depth, and the qualifying test
// against the pixel's opaque winner (its key is still in the visibility
// buffer): depth < d* and the triangle's object at or after the winner's.
__global__ void __launch_bounds__(256) k_traster(const DgJobDev job) {
    wait_previous_kernel();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t nr = 4u * job.ntt;
    const unsigned long long total = __ldcg(job.tscan + nr);
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total;
         base += stride) {
        const unsigned long long q = base + lane;
        bool emit = false;
        uint64_t fk = 0;
        uint32_t rec = 0;
        if (q < total) {
            uint32_t lo = 0, hi = nr;  // largest r with tscan[r] <= q
            while (hi - lo > 1u) {
                const uint32_t mid = (lo + hi) >> 1;
                if (__ldcg(job.tscan + mid) <= q)
                    lo = mid;
                else
                    hi = mid;
            }
            rec = lo;
            const uint32_t k = (uint32_t)(q - __ldcg(job.tscan + rec));
            const uint4 box = __ldcg(job.tbox + rec);
            const DgFrameDev& fr = job.frames[box.w];
            const uint32_t y = box.y + k / box.z, x = box.x + k % box.z;
            const DgTriRec* R = job.ttrec + rec;
            EdgeSet e;
            load_edges(R, e);
            float al, be, ga;
            if (covered(e, (float)x, (float)y, al, be, ga)) {
                const float4 dd = __ldg(reinterpret_cast<const float4*>(R) + 4);
                const float depth = interp(al, be, ga, dd.x, dd.y, dd.z);
                const uint64_t key = __ldcg(reinterpret_cast<const unsigned long long*>(fr.vis) + (uint64_t)y * fr.width + x);
                float dstar = fr.clear_depth;
                int objj = -1;
                if (key != DG_VIS_EMPTY) {
                    dstar = key_depth(key);
                    const uint32_t tl = (uint32_t)key >> 2;
                    objj = (int)last_le(fr.seg_count, tl, [&](uint32_t s) { return job.segs[fr.seg_begin + s].seq_base; });
                }
                const uint2 meta = __ldcg(job.tmeta + rec);
                if (depth < dstar && (int)meta.x >= objj) {
                    emit = true;
                    fk = ((uint64_t)(fr.pix_begin + y * fr.width + x) << 32) | meta.y;
                }
            }
        }
        const unsigned em = __ballot_sync(0xFFFFFFFFu, emit);
        if (em) {
            const int leader = __ffs(em) - 1;
            unsigned long long slot = 0;
            if ((int)lane == leader) slot = atomicAdd(job.cnt + DG_CNT_TFRAG, (unsigned long long)__popc(em));
            slot = __shfl_sync(0xFFFFFFFFu, slot, leader) + __popc(em & ((1u << lane) - 1u));
            if (emit) {
                if (slot < job.fcap) {
                    job.fkey[0][slot] = fk;
                    job.fval[0][slot] = rec;
                } else {
                    atomicOr(job.err, 1u << DG_E_LIMIT);  // more fragments than the buffers hold
                }
            }
        }
    }
}

// ----------------------------------------------------------- part 2
// Pixel * f32 (canvas.rs:155-169): each channel (c as f32 * f) as u8, padd 0.
__device__ __forceinline__ uint32_t px_mul(uint32_t p, float f) {
    const uint32_t b = as_u8(fM((float)(p & 0xFFu), f));
    const uint32_t g = as_u8(fM((float)((p >> 8) & 0xFFu), f));
    const uint32_t r = as_u8(fM((float)((p >> 16) & 0xFFu), f));
    return b | (g << 8) | (r << 16);
}
// Pixel + Pixel (canvas.rs:136-153): u8 channel sums (wrapping), padd 0.
__device__ __forceinline__ uint32_t px_add(uint32_t p, uint32_t q) {
    return ((p + q) & 0xFFu) | (((p >> 8) + (q >> 8)) & 0xFFu) << 8 | (((p >> 16) + (q >> 16)) & 0xFFu) << 16;
}

// The ordered blend: the first sorted fragment of each pixel folds all of the
// pixel's fragments over the opaque colour, in submission order
// (draw_pixel_coord_with_depth, canvas.rs:906-930, with depth writes off).
__global__ void __launch_bounds__(256) k_tfold(const DgJobDev job) {
    __shared__ float inv255[256];
    __shared__ DgTexDev stex[DG_SMEM_TEX];
    inv255[threadIdx.x] = fD((float)threadIdx.x, 255.0f);
    const uint32_t nst = job.ntex < DG_SMEM_TEX ? job.ntex : DG_SMEM_TEX;
    for (uint32_t i = threadIdx.x; i < nst * 3u; i += blockDim.x)
        reinterpret_cast<uint4*>(stex)[i] = __ldg(reinterpret_cast<const uint4*>(job.tex) + i);
    wait_previous_kernel();
    __syncthreads();
    const unsigned long long n64 = __ldcg(job.cnt + DG_CNT_TFRAG);
    const uint32_t n = (uint32_t)(n64 < job.fcap ? n64 : job.fcap);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t p = (uint32_t)(__ldcg(job.fkey[0] + i) >> 32);
        if (i > 0u && (uint32_t)(__ldcg(job.fkey[0] + i - 1u) >> 32) == p) continue;  // not the pixel's first
        const uint32_t fi = last_le(job.nframes, p, [&](uint32_t k) { return job.frames[k].pix_begin; });
        const DgFrameDev& fr = job.frames[fi];
        const uint32_t local = p - fr.pix_begin;
        const uint32_t y = local / fr.width, x = local - y * fr.width;
        const uint64_t ci = (uint64_t)(fr.height - 1u - y) * fr.width + x;
        uint32_t bg = fr.colour[ci];
        uint32_t bits = 0;
        for (uint32_t m = i; m < n && (uint32_t)(__ldcg(job.fkey[0] + m) >> 32) == p; m++) {
            const uint32_t rec = __ldcg(job.fval[0] + m);
            float d;
            int errc;
            const float4* wp = (fr.flags & DG_FRAME_PERSPECTIVE) && job.ttrec_w ? job.ttrec_w + rec : nullptr;
            uint32_t c = shade_from_record<true, false>(job, fr, job.ttrec + rec, x, y, inv255, stex, d, errc, wp);
            if (errc != DG_OK) bits |= 1u << errc;
            const float a = __ldcg(job.talpha + rec);
            if (a < 1.0f) c = px_add(px_mul(bg, fS(1.0f, a)), px_mul(c, a));
            bg = c;
        }
        fr.colour[ci] = bg;
        if (bits) atomicOr(job.err, bits);
    }
}

// ------------------------------------------------------------ 2D overlay
// Canvas::draw_triangle (canvas.rs:435-575): every pixel of every clipped
// bounding box and the coverage test (the same edge functions and tie rule as
// the 3D rasterizer); covered pixels become fragments.
__global__ void __launch_bounds__(256) k_o_raster(const DgOverlayJob job) {
    wait_previous_kernel();
    const uint32_t lane = threadIdx.x & 31u;
    const unsigned long long total = job.scan[job.n];
    const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
    for (unsigned long long base = (unsigned long long)blockIdx.x * blockDim.x + (threadIdx.x & ~31u); base < total;
         base += stride) {
        const unsigned long long q = base + lane;
        bool emit = false;
        uint32_t tri = 0, px = 0;
        if (q < total) {
            uint32_t lo = 0, hi = job.n;  // largest t with scan[t] <= q
            while (hi - lo > 1u) {
                const uint32_t mid = (lo + hi) >> 1;
                if (__ldg(job.scan + mid) <= q)
                    lo = mid;
                else
                    hi = mid;
            }
            tri = lo;
            const uint32_t k = (uint32_t)(q - __ldg(job.scan + tri));
            const uint4 box = __ldg(job.box + tri);
            const uint32_t y = box.y + k / box.z, x = box.x + k % box.z;
            EdgeSet e;
            load_edges(job.rec + tri, e);
            float al, be, ga;
            if (covered(e, (float)x, (float)y, al, be, ga)) {
                emit = true;
                px = y * job.width + x;
            }
        }
        const unsigned em = __ballot_sync(0xFFFFFFFFu, emit);
        if (em) {
            const int leader = __ffs(em) - 1;
            unsigned long long slot = 0;
            if ((int)lane == leader) slot = atomicAdd(job.cnt, (unsigned long long)__popc(em));
            slot = __shfl_sync(0xFFFFFFFFu, slot, leader) + __popc(em & ((1u << lane) - 1u));
            if (emit && slot < job.fcap) {
                job.fkey[0][slot] = ((uint64_t)px << 32) | tri;
                job.fval[0][slot] = tri;
            }
        }
    }
}

// TextureMap::get_rgba_slice (scene/mod.rs:137-152): (u * width) and
// (v * height) floored, wrapping usize offset, four bytes; false where the
// reference's slice index would panic.
__device__ __forceinline__ bool tex_rgba(const DgTexDev& tx, float u, float v, uint32_t& rgba) {
    const uint64_t ui = as_usize(floorf(fM(u, tx.fw)));
    const uint64_t vi = (uint64_t)tx.height - 1ull - as_usize(floorf(fM(v, tx.fh)));
    const uint64_t off = (vi * (uint64_t)tx.width + ui) * (uint64_t)tx.comps;
    if (tx.len < 4ull || off > tx.len - 4ull) return false;
    const uint64_t w = off >> 2;
    const uint32_t sh = (uint32_t)(off & 3ull) * 8u;
    const uint32_t lo = __ldg(tx.words + w);
    rgba = sh == 0u ? lo : __funnelshift_r(lo, __ldg(tx.words + w + 1), sh);
    return true;
}

// Each pixel's fragments in triangle order: the vertex colours and alphas and
// the texture coordinates interpolated with the barycentrics, the RGBA texel,
// the colour blend with the texel, and draw_pixel_coord_with_depth's depth test
// at depth 0 (the overlay never writes depth: depth updates are off outside the
// opaque pass) and blend with the canvas (canvas.rs:529-573, 906-930).
__global__ void __launch_bounds__(256) k_o_fold(const DgOverlayJob job) {
    wait_previous_kernel();
    const unsigned long long n64 = *job.cnt;
    const uint32_t n = (uint32_t)(n64 < job.fcap ? n64 : job.fcap);
    if (threadIdx.x == 0 && blockIdx.x == 0 && n64 > job.fcap) atomicOr(job.err, 1u << DG_E_LIMIT);
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const uint32_t p = (uint32_t)(job.fkey[0][i] >> 32);
        if (i > 0u && (uint32_t)(job.fkey[0][i - 1u] >> 32) == p) continue;  // not the pixel's first
        const uint32_t y = p / job.width, x = p - y * job.width;
        const uint64_t ci = (uint64_t)(job.height - 1u - y) * job.width + x;
        const bool pass = 0.0f < job.depth[(uint64_t)y * job.width + x];
        uint32_t bg = job.colour[ci];
        uint32_t bits = 0;
        for (uint32_t m = i; m < n && (uint32_t)(job.fkey[0][m] >> 32) == p; m++) {
            const DgTriRec* R = job.rec + job.fval[0][m];
            EdgeSet e;
            load_edges(R, e);
            float al, be, ga;
            covered(e, (float)x, (float)y, al, be, ga);  // the fragment passed it in k_o_raster
            const float4* q = reinterpret_cast<const float4*>(R);
            const float4 fu = __ldg(q + 4), fv = __ldg(q + 5);
            const uint4 fc = __ldg(reinterpret_cast<const uint4*>(R) + 6);
            // (alpha * color_a) + (beta * color_b) + (gama * color_c): Pixel products and sums
            const uint32_t cp0 = px_add(px_add(px_mul(fc.x, al), px_mul(fc.y, be)), px_mul(fc.z, ga));
            const float calpha = fA(fA(fM(al, fu.w), fM(be, fv.w)), fM(ga, __uint_as_float(fc.w)));
            const float cu = fA(fA(fM(fu.x, al), fM(fu.y, be)), fM(fu.z, ga));
            const float cv = fA(fA(fM(fv.x, al), fM(fv.y, be)), fM(fv.z, ga));
            uint32_t rgba;
            if (!tex_rgba(job.tex, cu, cv, rgba)) {
                bits |= 1u << DG_E_TEXTURE_RANGE;
                continue;
            }
            const float talpha = fD((float)(rgba >> 24), 255.0f);
            const uint32_t ct = ((rgba >> 16) & 0xFFu) | (((rgba >> 8) & 0xFFu) << 8) | ((rgba & 0xFFu) << 16);
            const uint32_t cp = px_add(px_mul(cp0, talpha), px_mul(ct, fS(1.0f, talpha)));
            const float fa = fM(calpha, talpha);
            if (pass) bg = fa < 1.0f ? px_add(px_mul(bg, fS(1.0f, fa)), px_mul(cp, fa)) : cp;
        }
        job.colour[ci] = bg;
        if (bits) atomicOr(job.err, bits);
    }
}

}  // namespace

cudaError_t dg_launch_overlay(const DgOverlayJob& job, unsigned blocks, cudaStream_t s) {
    if (job.n == 0u) return cudaSuccess;
    const unsigned g = blocks < 1u ? 1u : blocks;
    cudaError_t e = launch_dependent(k_o_raster, g, 256, job, s);
    if (e != cudaSuccess) return e;
    if ((e = radix_sort(job.fkey, job.fval, job.hist, job.cnt, job.fcap, job.sort_shift, job.n_sort, g, s)) !=
        cudaSuccess)
        return e;
    return launch_dependent(k_o_fold, g, 256, job, s);
}

cudaError_t dg_launch_transparent(int part, const DgJobDev& job, const DgTransparentPlan& plan, cudaStream_t s) {
    if (job.ntt == 0u) return cudaSuccess;
    const unsigned g = plan.blocks < 1u ? 1u : plan.blocks;
    cudaError_t e = cudaSuccess;
    if (part == 0) {
        if ((e = launch_dependent(k_tkeys, grid_for(job.ntt, g), 256, job, s)) != cudaSuccess) return e;
        if ((e = radix_sort(job.tkey, job.tval, job.sort_hist, nullptr, job.ntt, plan.tsort_shift, plan.n_tsort, g,
                            s)) != cudaSuccess)
            return e;
        if ((e = launch_dependent(k_tgather, grid_for(job.ntt, g), 256, job, s)) != cudaSuccess) return e;
        return launch_dependent(k_tsetup, grid_for(job.ntt, g), 256, job, s);
    }
    if (part == 1) {
        if ((e = launch_dependent(k_tscan, 1u, 1024, job, s)) != cudaSuccess) return e;
        if ((e = launch_dependent(k_traster, g, 256, job, s)) != cudaSuccess) return e;
        return radix_sort(job.fkey, job.fval, job.sort_hist, job.cnt + DG_CNT_TFRAG, job.fcap, plan.fsort_shift,
                          plan.n_fsort, g, s);
    }
    return launch_dependent(k_tfold, g, 256, job, s);
}
