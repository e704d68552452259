// dg_kernels.cu -- sm_103a kernels of the GB300 rasterizer.
//
// Pipeline of one render job (one or many frames), all on one stream:
//   k_vertex        per position vertex: eye distance, light/halfway vectors,
//                   projected and snapped screen centre, plane-sign masks
//                   (scene/mod.rs:917-926, :1047-1058, canvas.rs:585-587)
//   k_setup_raster  per input triangle: back-face cull, lateral reject,
//                   near/far clipping, bounding box, edge functions; tiny
//                   triangles are rasterized by their warp (pixels of all 32
//                   lanes' boxes flattened with a warp prefix scan), the others
//                   are queued (scene/mod.rs:933-1063, canvas.rs:585-681)
//   k_queue_raster  the queued triangles' bounding-box pixels in 32-pixel units
//                   spread evenly over all warps
//   k_resolve       per pixel: the winning fragment is shaded once
//                   (canvas.rs:682-745, 906-930) and colour/depth are written
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
#include "dg_internal.cuh"

namespace {

constexpr unsigned FULL = 0xFFFFFFFFu;
constexpr float EPS = 0.0000001f;  // linalg.rs:6
constexpr uint32_t AZUL_BB = 0xFF9BBAFFu;  // Pixel::azul_bb() as b,g,r,padd bytes (canvas.rs:131-133)

// ---------------------------------------------------------- exact f32 ops
__device__ __forceinline__ float fA(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fS(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fM(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float fD(float a, float b) { return __fdiv_rn(a, b); }

struct V3 {
    float x, y, z;
};
__device__ __forceinline__ V3 vadd(V3 a, V3 b) { return {fA(a.x, b.x), fA(a.y, b.y), fA(a.z, b.z)}; }
__device__ __forceinline__ V3 vsub(V3 a, V3 b) { return {fS(a.x, b.x), fS(a.y, b.y), fS(a.z, b.z)}; }
__device__ __forceinline__ V3 vmul(V3 a, float s) { return {fM(a.x, s), fM(a.y, s), fM(a.z, s)}; }
__device__ __forceinline__ V3 vdiv(V3 a, float s) { return {fD(a.x, s), fD(a.y, s), fD(a.z, s)}; }
// linalg.rs:182-184 and :167-171 (left-associative sums, powi(2) = x*x)
__device__ __forceinline__ float vdot(V3 a, V3 b) { return fA(fA(fM(a.x, b.x), fM(a.y, b.y)), fM(a.z, b.z)); }
__device__ __forceinline__ float vnorm(V3 a) { return __fsqrt_rn(fA(fA(fM(a.x, a.x), fM(a.y, a.y)), fM(a.z, a.z))); }
__device__ __forceinline__ V3 vnormalized(V3 a) { return vdiv(a, vnorm(a)); }  // linalg.rs:173-175 (3 divisions)
__device__ __forceinline__ V3 vcross(V3 a, V3 b) {                            // linalg.rs:186-200
    return {fS(fM(a.y, b.z), fM(a.z, b.y)), fS(fM(a.z, b.x), fM(a.x, b.z)), fS(fM(a.x, b.y), fM(a.y, b.x))};
}

// Rust `as usize` / `as u8` from f32: saturating, NaN -> 0.
__device__ __forceinline__ uint64_t as_usize(float f) {
    if (!(f > 0.0f)) return 0ull;
    if (f >= 18446744073709551616.0f) return ~0ull;
    return (uint64_t)f;
}
__device__ __forceinline__ uint32_t as_u8(float f) {
    if (!(f > 0.0f)) return 0u;
    if (f >= 255.0f) return 255u;
    return (uint32_t)f;
}

// LLVM's powi lowering: binary exponentiation starting from r = 1 (r = 1*x is exact).
__device__ __forceinline__ float powi(float a, int32_t e) {
    bool recip = e < 0;
    uint32_t n = recip ? 0u - (uint32_t)e : (uint32_t)e;
    float r = 1.0f;
    while (true) {
        if (n & 1u) r = fM(r, a);
        n >>= 1;
        if (n == 0u) break;
        a = fM(a, a);
    }
    return recip ? fD(1.0f, r) : r;
}

template <class F>
__device__ __forceinline__ uint32_t last_le(uint32_t n, uint32_t v, F key) {  // largest i < n with key(i) <= v
    uint32_t lo = 0, hi = n;
    while (hi - lo > 1u) {
        uint32_t mid = (lo + hi) >> 1;
        if (key(mid) <= v)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// ViewPlane::func, scene/mod.rs:634-636.
__device__ __forceinline__ float plane_f(const DgFrameDev& fr, int p, V3 v) {
    V3 n = {fr.plane[p][0], fr.plane[p][1], fr.plane[p][2]};
    return fA(vdot(n, v), fr.plane[p][3]);
}

// Matrix4 * Vec4 (linalg.rs:346-360, accumulators start at 0.0), then x/w, y/w
// (scene/mod.rs:1047-1058), minus the canvas offset and snapped to the pixel
// centre (canvas.rs:585-587, 896-904).
__device__ __forceinline__ void project_snap(const DgFrameDev& fr, V3 p, float& cx, float& cy) {
    float o[3];
    const int rows[3] = {0, 1, 3};
#pragma unroll
    for (int r = 0; r < 3; r++) {
        int i = rows[r];
        o[r] = fA(fA(fA(fA(0.0f, fM(fr.M[i][0], p.x)), fM(fr.M[i][1], p.y)), fM(fr.M[i][2], p.z)),
                  fM(fr.M[i][3], 1.0f));
    }
    float sx = fD(o[0], o[2]);
    float sy = fD(o[1], o[2]);
    sx = fA(sx, -fr.off_x);  // Vec2 sub is self + (-rhs) (linalg.rs:37-43)
    sy = fA(sy, -fr.off_y);
    cx = floorf(fA(sx, 0.5f));
    cy = floorf(fA(sy, 0.5f));
}

// ------------------------------------------------------------ edge set
// f_xy(x, y) = (((p.y - q.y) * x + (q.x - p.x) * y) + p.x * q.y) - q.x * p.y
// (canvas.rs:597-616) with the per-edge constants precomputed; the per-pixel
// result is the same IEEE value.
struct EdgeSet {
    float A[3], B[3], C[3], D[3];  // 0: f_bc (alpha), 1: f_ca (beta), 2: f_ab (gama)
    float den[3];                  // f_alpha, f_beta, f_gama
    uint32_t tie;                  // bit k: den[k] * f_k(-1,-1) > 0
};
__device__ __forceinline__ float edge_eval(const EdgeSet& e, int k, float x, float y) {
    return fS(fA(fA(fM(e.A[k], x), fM(e.B[k], y)), e.C[k]), e.D[k]);
}
__device__ __forceinline__ void make_edges(float ax, float ay, float bx, float by, float cx, float cy, EdgeSet& e) {
    const float px[3] = {bx, cx, ax}, py[3] = {by, cy, ay};
    const float qx[3] = {cx, ax, bx}, qy[3] = {cy, ay, by};
    const float vx[3] = {ax, bx, cx}, vy[3] = {ay, by, cy};
    e.tie = 0;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        e.A[k] = fS(py[k], qy[k]);
        e.B[k] = fS(qx[k], px[k]);
        e.C[k] = fM(px[k], qy[k]);
        e.D[k] = fM(qx[k], py[k]);
    }
#pragma unroll
    for (int k = 0; k < 3; k++) {
        e.den[k] = edge_eval(e, k, vx[k], vy[k]);
        float out = edge_eval(e, k, -1.0f, -1.0f);
        if (fM(e.den[k], out) > 0.0f) e.tie |= 1u << k;
    }
}

// Division-free early reject, exact with respect to the reference's test.
// Snapped centres and pixel coordinates are integer-valued floats, so every
// edge value is integer-valued (or +-inf/NaN): a nonzero finite numerator has
// magnitude >= 1 and num/den cannot underflow to zero for finite den. Hence
// when num and a finite den have opposite signs, num/den < 0 and the
// reference's `alpha >= 0.0` fails. Pixels that pass go through the exact test.
__device__ __forceinline__ bool prereject(float n, float d) {
    bool finite = fabsf(d) < INFINITY;
    bool neg_d = signbit(d);
    return finite && ((n < 0.0f && !neg_d) || (n > 0.0f && neg_d));
}

// canvas.rs:673-681: the barycentric coverage test with the (-1,-1) tie rule.
__device__ __forceinline__ bool covered(const EdgeSet& e, float x, float y, float& al, float& be, float& ga) {
    float n0 = edge_eval(e, 0, x, y);
    float n1 = edge_eval(e, 1, x, y);
    float n2 = edge_eval(e, 2, x, y);
    if (prereject(n0, e.den[0]) || prereject(n1, e.den[1]) || prereject(n2, e.den[2])) return false;
    al = fD(n0, e.den[0]);
    be = fD(n1, e.den[1]);
    ga = fD(n2, e.den[2]);
    if (!(al >= 0.0f && be >= 0.0f && ga >= 0.0f)) return false;
    return (al > 0.0f || (e.tie & 1u)) && (be > 0.0f || (e.tie & 2u)) && (ga > 0.0f || (e.tie & 4u));
}

__device__ __forceinline__ float interp(float al, float be, float ga, float a, float b, float c) {
    return fA(fA(fM(al, a), fM(be, b)), fM(ga, c));  // (a*alpha + b*beta) + c*gama, canvas.rs:682
}

__device__ __forceinline__ uint64_t depth_key(float depth, uint32_t seq) {
    uint32_t u = __float_as_uint(depth);
    if (u == 0x80000000u) u = 0u;  // -0.0 ties with +0.0 in the `<` test
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    return ((uint64_t)u << 32) | seq;
}

// One fragment: depth, strict test against the clear depth, then the keyed minimum.
__device__ __forceinline__ void raster_pixel(const EdgeSet& e, float da, float db, float dc, uint32_t seq, uint32_t x,
                                             uint32_t y, const DgFrameDev& fr) {
    float al, be, ga;
    if (!covered(e, (float)x, (float)y, al, be, ga)) return;
    float depth = interp(al, be, ga, da, db, dc);
    if (!(depth < fr.clear_depth)) return;
    uint64_t key = depth_key(depth, seq);
    // The result is unused, so this compiles to a fire-and-forget reduction at L2.
    atomicMin(reinterpret_cast<unsigned long long*>(fr.vis) + (uint64_t)y * fr.width + x, (unsigned long long)key);
}

// Bounding box of the snapped centres, clipped to the screen exactly like
// canvas.rs:618-658 (NaN-skipping min/max, saturating casts, Rectangle::clip's
// collapse to 0 when the box misses the screen).
__device__ __forceinline__ void bbox_axis(float a, float b, float c, uint32_t size, uint32_t& lo, uint32_t& hi) {
    float mn = INFINITY, mx = -INFINITY;
    if (a < mn) mn = a;
    if (b < mn) mn = b;
    if (c < mn) mn = c;
    if (a > mx) mx = a;
    if (b > mx) mx = b;
    if (c > mx) mx = c;
    uint64_t x0 = as_usize(mn), x1 = as_usize(mx);
    uint64_t l = x0 < x1 ? x0 : x1, h = x0 < x1 ? x1 : x0;
    uint64_t hc = h < (uint64_t)(size - 1) ? h : (uint64_t)(size - 1);
    if (l > hc) {
        l = 0;
        hc = 0;
    }
    lo = (uint32_t)l;
    hi = (uint32_t)hc;
}

// ---------------------------------------------------------- clip program
// Triangle::clip_against_planes (scene/mod.rs:43-90) and ViewPlane::clip
// (:662-746) on positions only. Each new vertex k >= 3 is recorded as
// pos[p] + (pos[q] - pos[p]) * t, so any attribute can later be evaluated with
// the same operations the reference applies to VertexAttributes.
struct ClipProg {
    V3 pos[9];
    uint8_t p[9], q[9];
    float t[9];
    uint8_t out[4][3];
    int nv, nout;
};

// Kept out of line: clipping is rare and would otherwise raise the register
// allocation (and lower the occupancy) of the common path.
__device__ __noinline__ void build_clip(const DgFrameDev& fr, V3 a, V3 b, V3 c, ClipProg& P) {
    P.pos[0] = a;
    P.pos[1] = b;
    P.pos[2] = c;
    P.nv = 3;
    P.nout = 0;
    for (int pl = 2; pl < 6; pl++) {  // at_least_partially_visible, :641-660
        float fa = plane_f(fr, pl, a), fb = plane_f(fr, pl, b), fc = plane_f(fr, pl, c);
        if (fa > 0.0f && fb > 0.0f && fc > 0.0f) continue;
        if (fa <= 0.0f && fb <= 0.0f && fc <= 0.0f) return;
    }
    uint8_t cur[4][3], nxt[4][3];
    int n = 1;
    cur[0][0] = 0;
    cur[0][1] = 1;
    cur[0][2] = 2;
    for (int d = 0; d < 2; d++) {  // near, then far
        int nn = 0;
        for (int i = 0; i < n; i++) {
            uint8_t ia = cur[i][0], ib = cur[i][1], ic = cur[i][2];
            float fa = plane_f(fr, d, P.pos[ia]), fb = plane_f(fr, d, P.pos[ib]), fc = plane_f(fr, d, P.pos[ic]);
            if (fa > 0.0f && fb > 0.0f && fc > 0.0f) {
                nxt[nn][0] = ia;
                nxt[nn][1] = ib;
                nxt[nn][2] = ic;
                nn++;
                continue;
            }
            if (fa <= 0.0f && fb <= 0.0f && fc <= 0.0f) continue;
            float tf;
            uint8_t ti;
            if (fM(fa, fc) >= 0.0f) {  // swap(b,c) then swap(a,b), :691-700
                tf = fb; fb = fc; fc = tf;
                ti = ib; ib = ic; ic = ti;
                tf = fa; fa = fb; fb = tf;
                ti = ia; ia = ib; ib = ti;
            } else if (fM(fb, fc) >= 0.0f) {  // swap(a,c) then swap(a,b), :701-711
                tf = fa; fa = fc; fc = tf;
                ti = ia; ia = ic; ic = ti;
                tf = fa; fa = fb; fb = tf;
                ti = ia; ia = ib; ib = ti;
            }
            V3 n3 = {fr.plane[d][0], fr.plane[d][1], fr.plane[d][2]};
            float t_a = fS(fD(plane_f(fr, d, P.pos[ia]), vdot(n3, vsub(P.pos[ia], P.pos[ic]))), EPS);
            int na = P.nv++;
            P.p[na] = ia;
            P.q[na] = ic;
            P.t[na] = t_a;
            P.pos[na] = vadd(P.pos[ia], vmul(vsub(P.pos[ic], P.pos[ia]), t_a));
            float t_b = fS(fD(plane_f(fr, d, P.pos[ib]), vdot(n3, vsub(P.pos[ib], P.pos[ic]))), EPS);
            int nb = P.nv++;
            P.p[nb] = ib;
            P.q[nb] = ic;
            P.t[nb] = t_b;
            P.pos[nb] = vadd(P.pos[ib], vmul(vsub(P.pos[ic], P.pos[ib]), t_b));
            if (fc <= 0.0f) {
                nxt[nn][0] = ia; nxt[nn][1] = (uint8_t)na; nxt[nn][2] = (uint8_t)nb; nn++;
                nxt[nn][0] = ia; nxt[nn][1] = ib; nxt[nn][2] = (uint8_t)nb; nn++;
            } else {
                nxt[nn][0] = ic; nxt[nn][1] = (uint8_t)na; nxt[nn][2] = (uint8_t)nb; nn++;
            }
        }
        for (int i = 0; i < nn; i++)
            for (int k = 0; k < 3; k++) cur[i][k] = nxt[i][k];
        n = nn;
    }
    for (int i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) P.out[i][k] = cur[i][k];
    P.nout = n;
}

// Values of one attribute field at the three vertices of clip output `o`
// (VertexAttributes add/sub/mul act field by field, canvas.rs:242-291).
__device__ void clip_field(const ClipProg& P, int o, float f0, float f1, float f2, float out[3]) {
    float v[9];
    v[0] = f0;
    v[1] = f1;
    v[2] = f2;
    for (int k = 3; k < P.nv; k++) v[k] = fA(v[P.p[k]], fM(fS(v[P.q[k]], v[P.p[k]]), P.t[k]));
    for (int i = 0; i < 3; i++) out[i] = v[P.out[o][i]];
}

// A triangle ready for rasterization.
struct RTri {
    float ax, ay, bx, by, cx, cy;
    float da, db, dc;
    uint32_t seq;
    uint32_t xlo, ylo, xhi, yhi;
    uint32_t frame;
};

// Screen centres and depths of clip output `o` (vertex ids < 3 reuse the vertex pass).
__device__ __noinline__ void clip_output_tri(const DgFrameDev& fr, const ClipProg& P, int o, const float4 r[3],
                                             RTri& t) {
    float cxs[3], cys[3];
    for (int i = 0; i < 3; i++) {
        int id = P.out[o][i];
        if (id < 3) {
            cxs[i] = r[id].x;
            cys[i] = r[id].y;
        } else {
            project_snap(fr, P.pos[id], cxs[i], cys[i]);
        }
    }
    float d[3];
    clip_field(P, o, r[0].z, r[1].z, r[2].z, d);
    t.ax = cxs[0]; t.ay = cys[0];
    t.bx = cxs[1]; t.by = cys[1];
    t.cx = cxs[2]; t.cy = cys[2];
    t.da = d[0]; t.db = d[1]; t.dc = d[2];
}

__device__ __forceinline__ uint32_t seg_of_tri(const DgJobDev& job, uint32_t g) {
    return last_le(job.nsegs, g, [&](uint32_t i) { return job.segs[i].tri_begin; });
}

// Light and halfway vectors of job vertex v for every light (scene/mod.rs:920-925).
// Only vertices of triangles that survive culling and clipping need them, so
// they are computed after the setup pass for the vertices it marked.
__device__ __forceinline__ void shade_vertex(const DgJobDev& job, uint32_t v) {
    const uint32_t si = last_le(job.nsegs, v, [&](uint32_t i) { return job.segs[i].vtx_begin; });
    const DgSegDev& sg = job.segs[si];
    const DgFrameDev& fr = job.frames[sg.frame];
    const float4 p4 = __ldg(sg.pos + (v - sg.vtx_begin));
    const V3 p = {p4.x, p4.y, p4.z};
    const V3 cam = {fr.cam[0], fr.cam[1], fr.cam[2]};
    const V3 eye = vnormalized(vsub(p, cam));
    for (uint32_t l = 0; l < fr.nlights; l++) {
        V3 L = {fr.light[l][0], fr.light[l][1], fr.light[l][2]};
        V3 lt = vnormalized(vsub(p, L));
        V3 h = vnormalized(vadd(lt, eye));
        float4* dst = job.vshade + ((uint64_t)v * job.shade_stride + l) * 2;
        dst[0] = make_float4(lt.x, lt.y, lt.z, h.x);
        dst[1] = make_float4(h.y, h.z, 0.0f, 0.0f);
    }
}

// ================================================================ kernels
__global__ void __launch_bounds__(256) k_vertex(const DgJobDev job) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < job.total_vtx; v += stride) {
        uint32_t si = last_le(job.nsegs, v, [&](uint32_t i) { return job.segs[i].vtx_begin; });
        const DgSegDev& sg = job.segs[si];
        const DgFrameDev& fr = job.frames[sg.frame];
        float4 p4 = __ldg(sg.pos + (v - sg.vtx_begin));
        V3 p = {p4.x, p4.y, p4.z};
        V3 cam = {fr.cam[0], fr.cam[1], fr.cam[2]};
        float depth = vnorm(vsub(p, cam));  // eye distance, scene/mod.rs:924
        float cx, cy;
        project_snap(fr, p, cx, cy);
        uint32_t mask = 0;
#pragma unroll
        for (int pl = 0; pl < 6; pl++) {
            float f = plane_f(fr, pl, p);
            if (f > 0.0f) mask |= 1u << pl;
            if (f <= 0.0f) mask |= 1u << (8 + pl);
        }
        job.vrec[v] = make_float4(cx, cy, depth, __uint_as_float(mask));
    }
}

// Rasterizes the triangles held by the lanes of a warp: the pixels of all
// bounding boxes are numbered with an inclusive warp scan and processed 32 at
// a time, each lane fetching its triangle's edge constants from the owner lane.
__device__ __forceinline__ void warp_flat_raster(const DgJobDev& job, const RTri& t, const EdgeSet& e, uint32_t npx) {
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t incl = npx;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(FULL, incl, o);
        if (lane >= (uint32_t)o) incl += v;
    }
    const uint32_t total = __shfl_sync(FULL, incl, 31);
    const uint32_t excl = incl - npx;
    const uint32_t w = t.xhi - t.xlo + 1u;
    for (uint32_t base = 0; base < total; base += 32u) {
        uint32_t j = base + lane;
        int lo = 0, hi = 31;
#pragma unroll
        for (int it = 0; it < 5; it++) {
            int mid = (lo + hi) >> 1;
            uint32_t v = __shfl_sync(FULL, incl, mid);
            if (v > j)
                hi = mid;
            else
                lo = mid + 1;
        }
        const int owner = lo;
        EdgeSet oe;
#pragma unroll
        for (int k = 0; k < 3; k++) {
            oe.A[k] = __shfl_sync(FULL, e.A[k], owner);
            oe.B[k] = __shfl_sync(FULL, e.B[k], owner);
            oe.C[k] = __shfl_sync(FULL, e.C[k], owner);
            oe.D[k] = __shfl_sync(FULL, e.D[k], owner);
            oe.den[k] = __shfl_sync(FULL, e.den[k], owner);
        }
        oe.tie = __shfl_sync(FULL, e.tie, owner);
        float da = __shfl_sync(FULL, t.da, owner);
        float db = __shfl_sync(FULL, t.db, owner);
        float dc = __shfl_sync(FULL, t.dc, owner);
        uint32_t seq = __shfl_sync(FULL, t.seq, owner);
        uint32_t xlo = __shfl_sync(FULL, t.xlo, owner);
        uint32_t ylo = __shfl_sync(FULL, t.ylo, owner);
        uint32_t ow = __shfl_sync(FULL, w, owner);
        uint32_t ofr = __shfl_sync(FULL, t.frame, owner);
        uint32_t oex = __shfl_sync(FULL, excl, owner);
        if (j < total) {
            uint32_t k = j - oex;
            uint32_t yy = k / ow;
            uint32_t xx = k - yy * ow;
            raster_pixel(oe, da, db, dc, seq, xlo + xx, ylo + yy, job.frames[ofr]);
        }
    }
}

// Kernels launched with programmatic dependent launch start before the previous
// kernel of the stream has finished; this waits until it has completed and its
// memory operations are visible.
__device__ __forceinline__ void wait_previous_kernel() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

__global__ void __launch_bounds__(256) k_setup_raster(const DgJobDev job) {
    wait_previous_kernel();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; base < job.total_tri; base += stride) {
        const uint32_t g = base + lane;
        int nout = 0;
        uint32_t si = 0, t = 0;
        uint4 tp = make_uint4(0, 0, 0, 0);
        float4 r[3];
        bool clipped = false;
        if (g < job.total_tri) {
            si = seg_of_tri(job, g);
            const DgSegDev& sg = job.segs[si];
            const DgFrameDev& fr = job.frames[sg.frame];
            t = g - sg.tri_begin;
            tp = __ldg(sg.tri_pos + t);
            // The lateral trivial reject (Triangle::clip_against_planes, scene/mod.rs:59-66) and
            // the back-face test (:1016-1027) are both pure predicates, so testing the cheap one
            // first gives the same surviving set: the plane-sign masks of the vertex records
            // reject most off-screen triangles before their positions are gathered.
            r[0] = __ldg(job.vrec + sg.vtx_begin + tp.x);
            r[1] = __ldg(job.vrec + sg.vtx_begin + tp.y);
            r[2] = __ldg(job.vrec + sg.vtx_begin + tp.z);
            const uint32_t m = __float_as_uint(r[0].w) & __float_as_uint(r[1].w) & __float_as_uint(r[2].w);
            if (((m >> 8) & 0x3Cu) == 0u) {  // no lateral plane has all three f <= 0
                float4 pa = __ldg(sg.pos + tp.x), pb = __ldg(sg.pos + tp.y), pc = __ldg(sg.pos + tp.z);
                V3 a = {pa.x, pa.y, pa.z}, b = {pb.x, pb.y, pb.z}, c = {pc.x, pc.y, pc.z};
                // back-face culling: Triangle::calc_normal, get_center; skip when (cam - centre) . n <= 0
                V3 n = vcross(vsub(b, a), vsub(c, b));
                V3 zero = {0.0f, 0.0f, 0.0f};
                V3 ctr = vdiv(vadd(vadd(vadd(zero, a), b), c), 3.0f);
                V3 cam = {fr.cam[0], fr.cam[1], fr.cam[2]};
                if (!(vdot(vsub(cam, ctr), n) <= 0.0f)) {
                    if ((m & 0x3u) == 0x3u) {
                        nout = 1;  // inside near and far: the triangle passes unchanged
                    } else {
                        ClipProg P;
                        build_clip(fr, a, b, c, P);
                        nout = P.nout;
                        clipped = true;
                    }
                    if (nout > 0) {  // its vertices need light/halfway vectors for shading
                        const uint32_t vv[3] = {sg.vtx_begin + tp.x, sg.vtx_begin + tp.y, sg.vtx_begin + tp.z};
                        for (int k = 0; k < 3; k++) atomicOr(job.vmark + (vv[k] >> 5), 1u << (vv[k] & 31u));
                    }
                }
            }
        }
        for (int rr = 0;; rr++) {
            bool has = rr < nout;
            if (__ballot_sync(FULL, has) == 0u) break;
            RTri tr;
            EdgeSet e;
            uint32_t npx = 0;
            uint32_t nu = 0;     // work units to queue (0: not queued)
            uint64_t qpx = 0;    // bounding-box pixels of the queued triangle
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
                    float4 pa = __ldg(sg.pos + tp.x), pb = __ldg(sg.pos + tp.y), pc = __ldg(sg.pos + tp.z);
                    ClipProg P;
                    build_clip(fr, V3{pa.x, pa.y, pa.z}, V3{pb.x, pb.y, pb.z}, V3{pc.x, pc.y, pc.z}, P);
                    clip_output_tri(fr, P, rr, r, tr);
                }
                bool nan = isnan(tr.ax) || isnan(tr.ay) || isnan(tr.bx) || isnan(tr.by) || isnan(tr.cx) ||
                           isnan(tr.cy);
                if (!nan) {  // any NaN centre makes every barycentric NaN: nothing is covered
                    bbox_axis(tr.ax, tr.bx, tr.cx, fr.width, tr.xlo, tr.xhi);
                    bbox_axis(tr.ay, tr.by, tr.cy, fr.height, tr.ylo, tr.yhi);
                    make_edges(tr.ax, tr.ay, tr.bx, tr.by, tr.cx, tr.cy, e);
                    uint64_t px = (uint64_t)(tr.xhi - tr.xlo + 1u) * (uint64_t)(tr.yhi - tr.ylo + 1u);
                    if (px <= job.small_max_px) {
                        npx = (uint32_t)px;
                    } else {
                        qpx = px;
                        nu = (uint32_t)((px + DG_UNIT_PX - 1u) / DG_UNIT_PX);
                    }
                }
            }
            // Queue this round's large triangles with one 64-bit atomic per warp: it hands out
            // the record slots and their first work units together, so work-unit bases ascend
            // with the slot (the queue pass binary-searches them).
            const unsigned qmask = __ballot_sync(FULL, nu != 0u);
            if (qmask) {
                uint32_t incl = nu;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    uint32_t v = __shfl_up_sync(FULL, incl, o);
                    if (lane >= (uint32_t)o) incl += v;
                }
                const uint32_t total_units = __shfl_sync(FULL, incl, 31);
                const int leader = __ffs(qmask) - 1;
                unsigned long long old = 0;
                if ((int)lane == leader)
                    old = atomicAdd(job.queue_counter,
                                    ((unsigned long long)__popc(qmask) << DG_PACK_SHIFT) | total_units);
                old = __shfl_sync(FULL, old, leader);
                if (nu != 0u) {
                    const uint64_t rec = (old >> DG_PACK_SHIFT) + __popc(qmask & ((1u << lane) - 1u));
                    const uint64_t ubase = (old & ((1ull << DG_PACK_SHIFT) - 1ull)) + (incl - nu);
                    // A record whose units would pass 2^32 is stored with no units (base
                    // saturated, so bases stay ascending) and rasterized by this lane.
                    const bool fits = ubase + nu <= 0xFFFFFFFFull;
                    if (rec < job.queue_cap) {
                        DgQueueRec q;
                        q.ax = tr.ax; q.ay = tr.ay; q.bx = tr.bx; q.by = tr.by; q.cx = tr.cx; q.cy = tr.cy;
                        q.da = tr.da; q.db = tr.db; q.dc = tr.dc;
                        q.seq = tr.seq;
                        q.frame = tr.frame;
                        q.xlo = tr.xlo;
                        q.ylo = tr.ylo;
                        q.w = tr.xhi - tr.xlo + 1u;
                        q.npx = (uint32_t)qpx;
                        q.nunits = fits ? nu : 0u;
                        job.queue[rec] = q;
                        job.queue_base[rec] = fits ? (uint32_t)ubase : 0xFFFFFFFFu;
                    }
                    if (!(rec < job.queue_cap && fits)) {
                        // queue full: this lane rasterizes the box itself
                        atomicAdd(job.stats + 1, 1ull);
                        const DgFrameDev& fr = job.frames[tr.frame];
                        for (uint32_t y = tr.ylo; y <= tr.yhi; y++)
                            for (uint32_t x = tr.xlo; x <= tr.xhi; x++)
                                raster_pixel(e, tr.da, tr.db, tr.dc, tr.seq, x, y, fr);
                    }
                }
            }
            warp_flat_raster(job, tr, e, npx);
        }
    }
}

// The raster queue: the bounding-box pixels of every queued triangle, numbered
// row-major in units of DG_UNIT_PX and spread over all warps. A warp keeps its
// current record (and edge constants) while consecutive units belong to it.
__global__ void __launch_bounds__(256) k_queue_raster(const DgJobDev job) {
    wait_previous_kernel();
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t nwarps = (gridDim.x * blockDim.x) >> 5;
    // Prologue: light/halfway vectors of the vertices the setup pass marked, one
    // mark word (32 vertices) per warp; the words are cleared for the next job.
    const uint32_t nwords = (job.total_vtx + 31u) >> 5;
    for (uint32_t w = warp; w < nwords; w += nwarps) {
        const uint32_t bits = __ldcg(job.vmark + w);
        if (bits == 0u) continue;
        if (((bits >> lane) & 1u) && (w << 5) + lane < job.total_vtx) shade_vertex(job, (w << 5) + lane);
        if (lane == 0) job.vmark[w] = 0u;
    }
    const unsigned long long cnt = __ldcg(job.queue_counter);
    const uint64_t nrec64 = cnt >> DG_PACK_SHIFT;
    const uint32_t nrec = (uint32_t)(nrec64 < job.queue_cap ? nrec64 : job.queue_cap);
    const uint64_t nu64 = cnt & ((1ull << DG_PACK_SHIFT) - 1ull);
    const uint32_t nunits = (uint32_t)(nu64 < 0xFFFFFFFFull ? nu64 : 0xFFFFFFFFull);
    if (nrec == 0) return;
    uint32_t cur_base = 1u, cur_end = 0u;
    DgQueueRec q;
    EdgeSet e;
    float rcp_w = 0.0f;
    // Each warp takes a contiguous range of units, so consecutive units usually
    // belong to the same record and the cached record and edge constants are reused.
    const uint32_t per = (nunits + nwarps - 1u) / nwarps;
    const uint32_t u0 = warp * per;
    const uint32_t u1 = min(nunits, u0 + per);
    for (uint32_t u = u0; u < u1; u++) {
        if (!(u >= cur_base && u < cur_end)) {
            uint32_t ri = last_le(nrec, u, [&](uint32_t i) { return __ldg(job.queue_base + i); });
            q = job.queue[ri];
            cur_base = __ldg(job.queue_base + ri);
            cur_end = cur_base + q.nunits;
            if (!(u >= cur_base && u < cur_end)) continue;  // unit of a record that did not fit the queue
            make_edges(q.ax, q.ay, q.bx, q.by, q.cx, q.cy, e);
            rcp_w = __frcp_rn((float)q.w);
        }
        const uint32_t k = (u - cur_base) * DG_UNIT_PX + lane;
        if (k < q.npx) {
            // k / w from a float reciprocal, corrected to the exact quotient
            uint32_t yy = (uint32_t)__fmul_rz((float)k, rcp_w);
            while ((uint64_t)yy * q.w > k) yy--;
            while ((uint64_t)(yy + 1u) * q.w <= k) yy++;
            const uint32_t xx = k - yy * q.w;
            raster_pixel(e, q.da, q.db, q.dc, q.seq, q.xlo + xx, q.ylo + yy, job.frames[q.frame]);
        }
    }
}

// Texel fetch of TextureMap::get_rgb_slice (scene/mod.rs:154-168) with the
// reference's wrapping usize arithmetic; false where the reference's slice
// index would panic.
__device__ __forceinline__ bool tex_rgb(const DgTexDev& tx, float u, float v, uint32_t& rgb) {
    uint64_t ui = as_usize(floorf(fM(u, fS(tx.fw, 1.0f))));
    uint64_t vi = (uint64_t)tx.height - 1ull - as_usize(floorf(fM(v, fS(tx.fh, 1.0f))));
    uint64_t off = (vi * (uint64_t)tx.width + ui) * (uint64_t)tx.comps;
    if (tx.len < 3ull || off > tx.len - 3ull) return false;
    uint64_t w = off >> 2;
    uint32_t lo = __ldg(tx.words + w), hi = __ldg(tx.words + w + 1);
    rgb = __funnelshift_r(lo, hi, (uint32_t)(off & 3ull) * 8u);
    return true;
}

// Shades the winning fragment of pixel (x, y): canvas.rs:682-741.
__device__ uint32_t shade_pixel(const DgJobDev& job, const DgFrameDev& fr, uint32_t seq, uint32_t x, uint32_t y,
                                const float* inv255, float& depth_out, int& errc) {
    errc = DG_OK;
    const uint32_t tl = seq >> 2, o = seq & 3u;
    uint32_t si =
        fr.seg_begin + last_le(fr.seg_count, tl, [&](uint32_t i) { return job.segs[fr.seg_begin + i].seq_base; });
    const DgSegDev& sg = job.segs[si];
    const uint32_t t = tl - sg.seq_base;
    if (t >= sg.ntri) {  // a key that no triangle of this frame can have produced
        errc = DG_E_CUDA;
        return 0u;
    }
    const uint4 tp = __ldg(sg.tri_pos + t);
    const uint4 tuv = __ldg(sg.tri_uv + t);
    const uint4 tnr = __ldg(sg.tri_nrm + t);
    const uint32_t vi[3] = {tp.x, tp.y, tp.z};
    const uint32_t ui[3] = {tuv.x, tuv.y, tuv.z};
    const uint32_t ni[3] = {tnr.x, tnr.y, tnr.z};
    float4 r[3];
    for (int k = 0; k < 3; k++) r[k] = __ldg(job.vrec + sg.vtx_begin + vi[k]);
    uint32_t gt = __float_as_uint(r[0].w) & __float_as_uint(r[1].w) & __float_as_uint(r[2].w);
    const bool clipped = (gt & 0x3u) != 0x3u;
    ClipProg P;
    RTri tr;
    if (!clipped) {
        if (o != 0u) {
            errc = DG_E_CUDA;
            return 0u;
        }
        tr.ax = r[0].x; tr.ay = r[0].y; tr.bx = r[1].x; tr.by = r[1].y; tr.cx = r[2].x; tr.cy = r[2].y;
        tr.da = r[0].z; tr.db = r[1].z; tr.dc = r[2].z;
    } else {
        float4 pa = __ldg(sg.pos + vi[0]), pb = __ldg(sg.pos + vi[1]), pc = __ldg(sg.pos + vi[2]);
        build_clip(fr, V3{pa.x, pa.y, pa.z}, V3{pb.x, pb.y, pb.z}, V3{pc.x, pc.y, pc.z}, P);
        if ((int)o >= P.nout) {
            errc = DG_E_CUDA;
            return 0u;
        }
        clip_output_tri(fr, P, (int)o, r, tr);
    }
    EdgeSet e;
    make_edges(tr.ax, tr.ay, tr.bx, tr.by, tr.cx, tr.cy, e);
    float al = 0.0f, be = 0.0f, ga = 0.0f;
    covered(e, (float)x, (float)y, al, be, ga);
    depth_out = interp(al, be, ga, tr.da, tr.db, tr.dc);

    // per-vertex field values of the output triangle
    auto field = [&](float f0, float f1, float f2) -> float {
        float v3[3];
        if (!clipped) {
            v3[0] = f0; v3[1] = f1; v3[2] = f2;
        } else {
            clip_field(P, (int)o, f0, f1, f2, v3);
        }
        return interp(al, be, ga, v3[0], v3[1], v3[2]);
    };
    float2 uv[3];
    float4 nr[3];
    for (int k = 0; k < 3; k++) {
        uv[k] = __ldg(sg.uv + ui[k]);
        nr[k] = __ldg(sg.nrm + ni[k]);
    }
    const float pu = field(uv[0].x, uv[1].x, uv[2].x);
    const float pv = field(uv[0].y, uv[1].y, uv[2].y);
    const V3 pn = {field(nr[0].x, nr[1].x, nr[2].x), field(nr[0].y, nr[1].y, nr[2].y),
                   field(nr[0].z, nr[1].z, nr[2].z)};
    const DgMatDev& mat = sg.mats[tp.w];
    uint32_t kd_rgb = 0, ka_rgb = 0;
    if (!tex_rgb(job.tex[mat.map_kd], pu, pv, kd_rgb) || !tex_rgb(job.tex[mat.map_ka], pu, pv, ka_rgb)) {
        errc = DG_E_TEXTURE_RANGE;
        return 0u;
    }
    // Pixel::normalized_as_vec3 (canvas.rs:81-87): byte / 255.0, looked up in a
    // table of the 256 correctly rounded quotients
    const V3 diffuse = {inv255[kd_rgb & 0xFFu], inv255[(kd_rgb >> 8) & 0xFFu], inv255[(kd_rgb >> 16) & 0xFFu]};
    const V3 ambient = {inv255[ka_rgb & 0xFFu], inv255[(ka_rgb >> 8) & 0xFFu], inv255[(ka_rgb >> 16) & 0xFFu]};
    const V3 c_l = {mat.ks[0], mat.ks[1], mat.ks[2]};
    const V3 c_r = {fM(diffuse.x, mat.kd[0]), fM(diffuse.y, mat.kd[1]), fM(diffuse.z, mat.kd[2])};
    const V3 c_a = {fM(ambient.x, mat.ka[0]), fM(ambient.y, mat.ka[1]), fM(ambient.z, mat.ka[2])};
    V3 inner = c_a;
    for (uint32_t l = 0; l < fr.nlights; l++) {
        float4 s0[3];
        for (int k = 0; k < 3; k++) s0[k] = __ldg(job.vshade + ((uint64_t)(sg.vtx_begin + vi[k]) * job.shade_stride + l) * 2);
        V3 pl = {field(s0[0].x, s0[1].x, s0[2].x), field(s0[0].y, s0[1].y, s0[2].y), field(s0[0].z, s0[1].z, s0[2].z)};
        float ln = vdot(pl, pn);
        float mx = ln > 0.0f ? ln : 0.0f;  // 0.0_f32.max(x): NaN -> 0
        inner = vadd(inner, vmul(c_l, fS(1.0f, mx)));
    }
    V3 col = {fM(c_r.x, inner.x), fM(c_r.y, inner.y), fM(c_r.z, inner.z)};
    for (uint32_t l = 0; l < fr.nlights; l++) {
        float4 s0[3], s1[3];
        for (int k = 0; k < 3; k++) {
            const float4* src = job.vshade + ((uint64_t)(sg.vtx_begin + vi[k]) * job.shade_stride + l) * 2;
            s0[k] = __ldg(src);
            s1[k] = __ldg(src + 1);
        }
        V3 ph = {field(s0[0].w, s0[1].w, s0[2].w), field(s1[0].x, s1[1].x, s1[2].x), field(s1[0].y, s1[1].y, s1[2].y)};
        col = vadd(col, vmul(c_l, powi(vdot(ph, pn), fr.exponent)));
    }
    // Pixel::from_normalized_vec3 (canvas.rs:89-92), stored as b,g,r,255
    V3 sc = vmul(col, 255.0f);
    uint32_t R = as_u8(sc.x), G = as_u8(sc.y), B = as_u8(sc.z);
    return B | (G << 8) | (R << 16) | (255u << 24);
}

__global__ void __launch_bounds__(256) k_resolve(const DgJobDev job) {
    __shared__ float inv255[256];
    inv255[threadIdx.x] = fD((float)threadIdx.x, 255.0f);  // independent of the previous kernel
    wait_previous_kernel();
    __syncthreads();
    const uint32_t tile = blockIdx.x;
    const uint32_t fi = last_le(job.nframes, tile, [&](uint32_t i) { return job.frames[i].tile_begin; });
    const DgFrameDev& fr = job.frames[fi];
    const uint32_t lt = tile - fr.tile_begin;
    const uint32_t ty = lt / fr.tiles_x, tx = lt - ty * fr.tiles_x;
    const uint32_t x = tx * DG_TILE_W + (threadIdx.x & (DG_TILE_W - 1u));
    const uint32_t y = ty * DG_TILE_H + threadIdx.x / DG_TILE_W;
    const bool in = x < fr.width && y < fr.height;
    bool hit = false;
    if (in) {
        const uint64_t i = (uint64_t)y * fr.width + x;
        const uint64_t ci = (uint64_t)(fr.height - 1u - y) * fr.width + x;
        const uint64_t key = __ldcg(reinterpret_cast<const unsigned long long*>(fr.vis) + i);
        if (key == DG_VIS_EMPTY) {
            fr.depth[i] = fr.clear_depth;
            fr.colour[ci] = AZUL_BB;
        } else {
            hit = true;
            fr.vis[i] = DG_VIS_EMPTY;
            float d = 0.0f;
            int errc;
            uint32_t c = shade_pixel(job, fr, (uint32_t)key, x, y, inv255, d, errc);
            if (errc != DG_OK) {
                atomicOr(job.err, 1u << errc);
                c = AZUL_BB;
            }
            fr.depth[i] = d;
            fr.colour[ci] = c;
        }
    }
    unsigned m = __ballot_sync(FULL, hit);
    if ((threadIdx.x & 31u) == 0u && m) atomicAdd(job.stats, (unsigned long long)__popc(m));
}

__global__ void k_fill(uint32_t* colour, float* depth, uint64_t n, uint32_t cv, float dv, int fc, int fd) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
        if (fc) colour[i] = cv;
        if (fd) depth[i] = dv;
    }
}

__global__ void k_vis_reset(uint64_t* vis, uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        vis[i] = DG_VIS_EMPTY;
}

inline unsigned grid_for(uint64_t n, unsigned cap) {
    uint64_t g = (n + 255) / 256;
    if (g < 1) g = 1;
    return (unsigned)(g < cap ? g : cap);
}

}  // namespace

cudaError_t dg_launch_vertex(const DgJobDev& job, cudaStream_t s) {
    if (job.total_vtx == 0) return cudaSuccess;
    k_vertex<<<grid_for(job.total_vtx, 1u << 20), 256, 0, s>>>(job);
    return cudaGetLastError();
}

// Programmatic dependent launch: the kernel may be scheduled while the previous
// kernel of the stream drains; it calls wait_previous_kernel() before reading
// anything that kernel wrote.
cudaError_t launch_dependent(void (*kern)(DgJobDev), unsigned grid, unsigned block, const DgJobDev& job,
                             cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, job);
}

cudaError_t dg_launch_setup_raster(const DgJobDev& job, unsigned max_blocks, cudaStream_t s) {
    if (job.total_tri == 0) return cudaSuccess;
    return launch_dependent(k_setup_raster, grid_for(job.total_tri, max_blocks < 1u ? 1u : max_blocks), 256, job, s);
}

cudaError_t dg_launch_queue_raster(const DgJobDev& job, unsigned blocks, cudaStream_t s) {
    if (job.total_tri == 0) return cudaSuccess;
    return launch_dependent(k_queue_raster, blocks < 1u ? 1u : blocks, 256, job, s);
}

cudaError_t dg_launch_resolve(const DgJobDev& job, cudaStream_t s) {
    if (job.total_tiles == 0) return cudaSuccess;
    return launch_dependent(k_resolve, job.total_tiles, 256, job, s);
}

cudaError_t dg_launch_fill(uint32_t* colour, float* depth, uint64_t n, uint32_t colour_value, float depth_value,
                           int fill_colour, int fill_depth, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_fill<<<grid_for(n, 4096u), 256, 0, s>>>(colour, depth, n, colour_value, depth_value, fill_colour, fill_depth);
    return cudaGetLastError();
}

cudaError_t dg_launch_vis_reset(uint64_t* vis, uint64_t n, cudaStream_t s) {
    if (n == 0) return cudaSuccess;
    k_vis_reset<<<grid_for(n, 4096u), 256, 0, s>>>(vis, n);
    return cudaGetLastError();
}
