// dg_device.cuh -- device-side building blocks shared by the kernels of the
// GB300 rasterizer (dg_kernels.cu: the opaque pipeline; dg_transparent.cu: the
// transparent pass): exact f32 arithmetic in the reference's evaluation order,
// camera-space plane tests, projection and snapping, edge functions and the
// coverage test, the clip program, triangle records, texel fetch and shading.
//
// Every expression uses __fadd_rn/__fsub_rn/__fmul_rn/__fdiv_rn/__fsqrt_rn in
// the reference's evaluation order (no contraction), Rust's saturating
// float->int casts, and wrapping usize arithmetic for texel offsets.
#pragma once

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

// a / b rounded to nearest from y = RN(1/b), by Markstein's method (P. Markstein,
// "Computation of elementary functions on the IBM RISC System/6000 processor",
// IBM J. Res. Develop. 34(1), 1990): q0 = RN(a*y) is within two ulps of a/b; one
// residual step q1 = RN(q0 + RN(a - b*q0)*y) makes it faithful, after which the
// residual a - b*q1 is exact (an FMA) and RN(q1 + (a - b*q1)*y) is RN(a/b).
// Callers guarantee the steps neither overflow nor underflow: b integer-valued
// in [1, 2^100), a integer-valued with |a| < 2^100, so a nonzero quotient is at
// least 2^-100 and every nonzero residual at least 2^-123. A zero a returns a*y,
// which is the zero of the same sign that a / b gives.
__device__ __forceinline__ float div_rcp(float a, float b, float y) {
    const float q0 = __fmul_rn(a, y);
    const float r0 = __fmaf_rn(-q0, b, a);
    const float q1 = __fmaf_rn(r0, y, q0);
    const float r1 = __fmaf_rn(-q1, b, a);
    const float q2 = __fmaf_rn(r1, y, q1);
    return a == 0.0f ? q0 : q2;
}

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

// The clip-space w of world position p: the fourth row of M * (p, 1), the
// divisor of the projection above (scene/mod.rs:1047-1050).
__device__ __forceinline__ float proj_w(const DgFrameDev& fr, V3 p) {
    return fA(fA(fA(fA(0.0f, fM(fr.M[3][0], p.x)), fM(fr.M[3][1], p.y)), fM(fr.M[3][2], p.z)), fM(fr.M[3][3], 1.0f));
}

// Extension (no counterpart in the reference): perspective-correct weights.
// From the reference's screen-space barycentrics and iw = (1/w_a, 1/w_b, 1/w_c):
// pa = alpha * iw_a, pb = beta * iw_b, pc = gama * iw_c, s = (pa + pb) + pc,
// and the weights become pa / s, pb / s, pc / s.
__device__ __forceinline__ void persp_weights(float& al, float& be, float& ga, float4 iw) {
    const float pa = fM(al, iw.x), pb = fM(be, iw.y), pc = fM(ga, iw.z);
    const float s = fA(fA(pa, pb), pc);
    al = fD(pa, s);
    be = fD(pb, s);
    ga = fD(pc, s);
}
__device__ __forceinline__ float4 inv_w3(const DgFrameDev& fr, V3 a, V3 b, V3 c) {
    return make_float4(fD(1.0f, proj_w(fr, a)), fD(1.0f, proj_w(fr, b)), fD(1.0f, proj_w(fr, c)), 0.0f);
}

// A vertex as the raster setup uses it: snapped screen centre, eye distance
// (scene/mod.rs:924) and the plane-sign mask of k_vertex, for a job vertex at
// world position p.
__device__ __forceinline__ float4 vertex_screen(const DgFrameDev& fr, float4 p4, uint32_t mask) {
    const V3 p = {p4.x, p4.y, p4.z};
    const V3 cam = {fr.cam[0], fr.cam[1], fr.cam[2]};
    const float depth = vnorm(vsub(p, cam));
    float cx, cy;
    project_snap(fr, p, cx, cy);
    return make_float4(cx, cy, depth, __uint_as_float(mask));
}

// The three vertex records (vertex_screen of each, written by k_vertex) of
// triangle tp of segment sg.
__device__ __forceinline__ void triangle_vertices(const DgJobDev& job, const DgSegDev& sg, const DgFrameDev& fr,
                                                  uint4 tp, float4 r[3]) {
    (void)fr;
    if (!DG_IN_RANGE(tp.x < sg.nv && tp.y < sg.nv && tp.z < sg.nv, job.err)) {
        r[0] = r[1] = r[2] = make_float4(NAN, NAN, NAN, 0.0f);  // no plane bit: the triangle is dropped
        return;
    }
    r[0] = __ldg(job.vrec + sg.vtx_begin + tp.x);
    r[1] = __ldg(job.vrec + sg.vtx_begin + tp.y);
    r[2] = __ldg(job.vrec + sg.vtx_begin + tp.z);
}

// ------------------------------------------------------------ edge set
// f_xy(x, y) = (((p.y - q.y) * x + (q.x - p.x) * y) + p.x * q.y) - q.x * p.y
// (canvas.rs:597-616) with the per-edge constants precomputed; the per-pixel
// result is the same IEEE value.
using EdgeSet = DgEdges;
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
    // Normalization: an edge whose f_alpha (den) has its sign bit set is negated
    // as a whole (A, B, C, D and den). Round-to-nearest is symmetric in sign, so
    // the negated constants give exactly -f at every pixel, and f/den, the tie
    // product den * f(-1,-1) and every result derived from them are
    // bit-identical; only the signs that the coverage test compares change.
    bool fast = true;
#pragma unroll
    for (int k = 0; k < 3; k++) {
        if (signbit(e.den[k])) {
            e.A[k] = -e.A[k];
            e.B[k] = -e.B[k];
            e.C[k] = -e.C[k];
            e.D[k] = -e.D[k];
            e.den[k] = -e.den[k];
        }
        fast = fast && e.den[k] > 0.0f && e.den[k] < INFINITY;
    }
    if (fast) e.tie |= DG_EDGE_FAST;
}

// Whether the barycentric divisions of an edge set may use div_rcp: every den
// is finite, > 0 and below 2^100 (DG_EDGE_FAST makes them integer-valued and so
// >= 1), |A|, |B| < 2^64 and |C|, |D| < 2^98, so that the edge value at any
// pixel (coordinates below 2^32) stays below 2^100 in magnitude.
__device__ __forceinline__ bool edge_rcp_ok(const EdgeSet& e) {
    bool ok = (e.tie & DG_EDGE_FAST) != 0u;
#pragma unroll
    for (int k = 0; k < 3; k++)
        ok = ok && e.den[k] < 0x1p100f && fabsf(e.A[k]) < 0x1p64f && fabsf(e.B[k]) < 0x1p64f &&
             fabsf(e.C[k]) < 0x1p98f && fabsf(e.D[k]) < 0x1p98f;
    return ok;
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

// canvas.rs:673-681: the barycentric coverage test with the (-1,-1) tie rule,
// for a pixel whose edge values n0..n2 passed prereject.
__device__ __forceinline__ bool covered_divide(const EdgeSet& e, float n0, float n1, float n2, float& al, float& be,
                                               float& ga) {
    al = fD(n0, e.den[0]);
    be = fD(n1, e.den[1]);
    ga = fD(n2, e.den[2]);
    if (!(al >= 0.0f && be >= 0.0f && ga >= 0.0f)) return false;
    return (al > 0.0f || (e.tie & 1u)) && (be > 0.0f || (e.tie & 2u)) && (ga > 0.0f || (e.tie & 4u));
}
// The coverage test of an edge set with DG_EDGE_FAST (every den finite and
// > 0 after normalization), without division: alpha = n0 / den0 is >= 0 exactly
// when n0 >= 0 (NaN fails both), and > 0 exactly when n0 > 0 (an integer-valued
// n0 >= 1 over a finite den cannot underflow to zero); likewise beta, gama.
__device__ __forceinline__ bool covered_signs(uint32_t tie, float n0, float n1, float n2) {
    return (n0 > 0.0f || (n0 == 0.0f && (tie & 1u))) && (n1 > 0.0f || (n1 == 0.0f && (tie & 2u))) &&
           (n2 > 0.0f || (n2 == 0.0f && (tie & 4u)));
}
__device__ __forceinline__ bool covered(const EdgeSet& e, float x, float y, float& al, float& be, float& ga) {
    const float n0 = edge_eval(e, 0, x, y);
    const float n1 = edge_eval(e, 1, x, y);
    const float n2 = edge_eval(e, 2, x, y);
    if (e.tie & DG_EDGE_FAST) {
        if (!covered_signs(e.tie, n0, n1, n2)) return false;
        al = fD(n0, e.den[0]);
        be = fD(n1, e.den[1]);
        ga = fD(n2, e.den[2]);
        return true;
    }
    if (prereject(n0, e.den[0]) || prereject(n1, e.den[1]) || prereject(n2, e.den[2])) return false;
    return covered_divide(e, n0, n1, n2, al, be, ga);
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

// Light and halfway vectors of a vertex at world position p for light l
// (scene/mod.rs:920-925); eye_n = normalize(p - camera).
__device__ __forceinline__ void light_halfway(const DgFrameDev& fr, V3 p, V3 eye_n, uint32_t l, V3& lt, V3& h) {
    const V3 L = {fr.light[l][0], fr.light[l][1], fr.light[l][2]};
    lt = vnormalized(vsub(p, L));
    h = vnormalized(vadd(lt, eye_n));
}

// Writes row `row` of the light/halfway table: per light l, float4s 2l and 2l+1
// hold (lt.x, lt.y, lt.z, h.x) and (h.y, h.z, 0, 0).
__device__ __forceinline__ void put_shade(const DgJobDev& job, uint32_t row, uint32_t l, V3 lt, V3 h) {
    float4* dst = job.vshade + ((uint64_t)row * job.shade_stride + l) * 2;
    dst[0] = make_float4(lt.x, lt.y, lt.z, h.x);
    dst[1] = make_float4(h.y, h.z, 0.0f, 0.0f);
}

// Light and halfway vectors of job vertex v for every light. Only vertices of
// triangles that survive culling and clipping need them, so they are computed
// after the setup pass for the vertices it marked.
__device__ __forceinline__ void shade_vertex(const DgJobDev& job, uint32_t v) {
    const uint32_t si = last_le(job.nsegs, v, [&](uint32_t i) { return job.segs[i].vtx_begin; });
    const DgSegDev& sg = job.segs[si];
    const DgFrameDev& fr = job.frames[sg.frame];
    const float4 p4 = __ldg(sg.pos + (v - sg.vtx_begin));
    const V3 p = {p4.x, p4.y, p4.z};
    const V3 cam = {fr.cam[0], fr.cam[1], fr.cam[2]};
    const V3 eye = vnormalized(vsub(p, cam));
    for (uint32_t l = 0; l < fr.nlights; l++) {
        V3 lt, h;
        light_halfway(fr, p, eye, l, lt, h);
        put_shade(job, v, l, lt, h);
    }
}

// Rows of the light/halfway table for the new vertices (ids 3 .. nv-1) of a
// clipped triangle: the three input vertices' vectors are computed here (the
// same operations as shade_vertex, so the same values) and carried through the
// clip program field by field. Row of vertex k: rowbase + (k - 3).
__device__ __noinline__ void clip_shade_rows(const DgJobDev& job, const DgFrameDev& fr, const ClipProg& P,
                                             uint32_t rowbase) {
    const V3 cam = {fr.cam[0], fr.cam[1], fr.cam[2]};
    V3 eye[3];
    for (int i = 0; i < 3; i++) eye[i] = vnormalized(vsub(P.pos[i], cam));
    for (uint32_t l = 0; l < fr.nlights; l++) {
        float f[6][9];
        for (int i = 0; i < 3; i++) {
            V3 lt, h;
            light_halfway(fr, P.pos[i], eye[i], l, lt, h);
            f[0][i] = lt.x; f[1][i] = lt.y; f[2][i] = lt.z;
            f[3][i] = h.x; f[4][i] = h.y; f[5][i] = h.z;
        }
        for (int k = 3; k < P.nv; k++)
            for (int c = 0; c < 6; c++) f[c][k] = fA(f[c][P.p[k]], fM(fS(f[c][P.q[k]], f[c][P.p[k]]), P.t[k]));
        for (int k = 3; k < P.nv; k++)
            put_shade(job, rowbase + (uint32_t)(k - 3), l, V3{f[0][k], f[1][k], f[2][k]},
                      V3{f[3][k], f[4][k], f[5][k]});
    }
}

__device__ __forceinline__ void store_edges(DgTriRec* r, const EdgeSet& e) {
    float4* d = reinterpret_cast<float4*>(r);
    d[0] = make_float4(e.A[0], e.A[1], e.A[2], e.B[0]);
    d[1] = make_float4(e.B[1], e.B[2], e.C[0], e.C[1]);
    d[2] = make_float4(e.C[2], e.D[0], e.D[1], e.D[2]);
    d[3] = make_float4(e.den[0], e.den[1], e.den[2], __uint_as_float(e.tie));
}
__device__ __forceinline__ void load_edges(const DgTriRec* r, EdgeSet& e) {
    const float4* s = reinterpret_cast<const float4*>(r);
    const float4 a = __ldg(s), b = __ldg(s + 1), c = __ldg(s + 2), d = __ldg(s + 3);
    e.A[0] = a.x; e.A[1] = a.y; e.A[2] = a.z; e.B[0] = a.w;
    e.B[1] = b.x; e.B[2] = b.y; e.C[0] = b.z; e.C[1] = b.w;
    e.C[2] = c.x; e.D[0] = c.y; e.D[1] = c.z; e.D[2] = c.w;
    e.den[0] = d.x; e.den[1] = d.y; e.den[2] = d.z; e.tie = __float_as_uint(d.w);
}

// Material words of a triangle record: ka, kd, ks and the two texture indices
// spread over the w slots of words 4-10 and word 11.
__device__ __forceinline__ void mat_words(const DgSegDev& sg, uint32_t mi, float w[9], uint4& last, const DgJobDev& job) {
    if (mi >= sg.nmats) {  // never produced by the host API; flagged and shaded as zero material
        atomicOr(job.err, 1u << DG_E_CUDA);
        mi = 0;
    }
    const float4* mq = reinterpret_cast<const float4*>(sg.mats + mi);
    const float4 m0 = __ldg(mq), m1 = __ldg(mq + 1), m2 = __ldg(mq + 2);  // ka, kd, ks, alpha, map_ka, map_kd
    w[0] = m0.x; w[1] = m0.y; w[2] = m0.z;  // ka
    w[3] = m0.w; w[4] = m1.x; w[5] = m1.y;  // kd
    w[6] = m1.z;                            // ks.x
    last = make_uint4(__float_as_uint(m1.w), __float_as_uint(m2.x), __float_as_uint(m2.z), __float_as_uint(m2.w));
}

// Triangle record of an unclipped triangle (its vertices are the mesh's).
// Wout (frames with DG_FRAME_PERSPECTIVE, else null): receives inv_w3 of the
// triangle's vertices.
__device__ __forceinline__ void write_record(const DgJobDev& job, DgTriRec* R, const DgSegDev& sg, uint4 tp, uint4 tuv,
                                             uint4 tnr, const EdgeSet& e, const float4 r[3], const DgFrameDev& fr,
                                             float4* Wout) {
    store_edges(R, e);
    if (Wout) {
        const float4 pa = __ldg(sg.pos + tp.x), pb = __ldg(sg.pos + tp.y), pc = __ldg(sg.pos + tp.z);
        *Wout = inv_w3(fr, V3{pa.x, pa.y, pa.z}, V3{pb.x, pb.y, pb.z}, V3{pc.x, pc.y, pc.z});
    }
    const float2 u0 = __ldg(sg.uv + tuv.x), u1 = __ldg(sg.uv + tuv.y), u2 = __ldg(sg.uv + tuv.z);
    const float4 n0 = __ldg(sg.nrm + tnr.x), n1 = __ldg(sg.nrm + tnr.y), n2 = __ldg(sg.nrm + tnr.z);
    float mw[9];
    uint4 last;
    mat_words(sg, tp.w, mw, last, job);
    float4* d = reinterpret_cast<float4*>(R);
    d[4] = make_float4(r[0].z, r[1].z, r[2].z, mw[0]);
    d[5] = make_float4(u0.x, u1.x, u2.x, mw[1]);
    d[6] = make_float4(u0.y, u1.y, u2.y, mw[2]);
    d[7] = make_float4(n0.x, n1.x, n2.x, mw[3]);
    d[8] = make_float4(n0.y, n1.y, n2.y, mw[4]);
    d[9] = make_float4(n0.z, n1.z, n2.z, mw[5]);
    reinterpret_cast<uint4*>(R)[10] =
        make_uint4(sg.vtx_begin + tp.x, sg.vtx_begin + tp.y, sg.vtx_begin + tp.z, __float_as_uint(mw[6]));
    reinterpret_cast<uint4*>(R)[11] = last;
}

// Triangle record of clip output o: attribute fields through the clip program;
// the light/halfway rows of new vertex k are rowbase + (k - 3).
__device__ __noinline__ void write_clip_record(const DgJobDev& job, DgTriRec* R, const DgSegDev& sg, uint4 tp,
                                               uint4 tuv, uint4 tnr, const EdgeSet& e, const RTri& tr,
                                               const ClipProg& P, int o, uint32_t rowbase, const DgFrameDev& fr,
                                               float4* Wout) {
    store_edges(R, e);
    if (Wout) *Wout = inv_w3(fr, P.pos[P.out[o][0]], P.pos[P.out[o][1]], P.pos[P.out[o][2]]);
    const float2 u0 = __ldg(sg.uv + tuv.x), u1 = __ldg(sg.uv + tuv.y), u2 = __ldg(sg.uv + tuv.z);
    const float4 n0 = __ldg(sg.nrm + tnr.x), n1 = __ldg(sg.nrm + tnr.y), n2 = __ldg(sg.nrm + tnr.z);
    float mw[9];
    uint4 last;
    mat_words(sg, tp.w, mw, last, job);
    float f[3];
    float4* d = reinterpret_cast<float4*>(R);
    d[4] = make_float4(tr.da, tr.db, tr.dc, mw[0]);
    clip_field(P, o, u0.x, u1.x, u2.x, f);
    d[5] = make_float4(f[0], f[1], f[2], mw[1]);
    clip_field(P, o, u0.y, u1.y, u2.y, f);
    d[6] = make_float4(f[0], f[1], f[2], mw[2]);
    clip_field(P, o, n0.x, n1.x, n2.x, f);
    d[7] = make_float4(f[0], f[1], f[2], mw[3]);
    clip_field(P, o, n0.y, n1.y, n2.y, f);
    d[8] = make_float4(f[0], f[1], f[2], mw[4]);
    clip_field(P, o, n0.z, n1.z, n2.z, f);
    d[9] = make_float4(f[0], f[1], f[2], mw[5]);
    const uint32_t vi[3] = {tp.x, tp.y, tp.z};
    uint32_t rows[3];
    for (int i = 0; i < 3; i++) {
        const int id = P.out[o][i];
        rows[i] = id < 3 ? sg.vtx_begin + vi[id] : rowbase + (uint32_t)(id - 3);
    }
    reinterpret_cast<uint4*>(R)[10] = make_uint4(rows[0], rows[1], rows[2], __float_as_uint(mw[6]));
    reinterpret_cast<uint4*>(R)[11] = last;
}


// Kernels launched with programmatic dependent launch start before the previous
// kernel of the stream has finished; this waits until it has completed and its
// memory operations are visible.
// Lets the next kernel of the stream (one launched by launch_dependent) be
// scheduled as soon as every block of this grid has started. That kernel still
// waits in wait_previous_kernel() until this grid has completed and its writes
// are visible, so the early start only overlaps its launch and prologue.
__device__ __forceinline__ void allow_next_kernel() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
// Waits until the previous kernel of the stream has completed and its writes are
// visible (a no-op after a plain launch); lets the next kernel be scheduled first.
__device__ __forceinline__ void wait_previous_kernel() {
    allow_next_kernel();
    asm volatile("griddepcontrol.wait;" ::: "memory");
}

// Rasterizes a triangle's clipped bounding box on the calling lane alone, row
// by row (the pixel position advances without division).
__device__ __forceinline__ void raster_box(const EdgeSet& e, float da, float db, float dc, uint32_t seq, uint32_t xlo,
                                           uint32_t ylo, uint32_t w, uint32_t h, const DgFrameDev& fr) {
    unsigned long long* vis = reinterpret_cast<unsigned long long*>(fr.vis);
    const float clear_depth = fr.clear_depth;
    const uint32_t width = fr.width;
    uint32_t x = xlo, y = ylo;
    const uint32_t xe = xlo + w;
    const uint64_t n = (uint64_t)w * h;
    if ((e.tie & DG_EDGE_FAST) && n <= 64u) {
        // Two passes: the division-free sign test of every box pixel into a mask,
        // then the covered pixels alone (divisions, depth, keyed minimum), so that
        // a lane's expensive steps are not interleaved with its uncovered pixels.
        uint64_t mask = 0;
        for (uint32_t k = 0; k < (uint32_t)n; k++) {
            const float xf = (float)x, yf = (float)y;
            if (covered_signs(e.tie, edge_eval(e, 0, xf, yf), edge_eval(e, 1, xf, yf), edge_eval(e, 2, xf, yf)))
                mask |= 1ull << k;
            if (++x == xe) {
                x = xlo;
                y++;
            }
        }
        if (!mask) return;
        const bool rcp = edge_rcp_ok(e);
        const float y0 = rcp ? __frcp_rn(e.den[0]) : 0.0f, y1 = rcp ? __frcp_rn(e.den[1]) : 0.0f,
                    y2 = rcp ? __frcp_rn(e.den[2]) : 0.0f;
        // k / w for k < 64 and w <= 64: k * ceil(2^16 / w) >> 16 errs by less than
        // 64 / 2^16 < 1 / w, which cannot carry past the next multiple of 1 / w
        const uint32_t inv_w = (65536u + w - 1u) / w;
        while (mask) {
            const uint32_t k = (uint32_t)__ffsll((long long)mask) - 1u;
            mask &= mask - 1ull;
            const uint32_t dy = (k * inv_w) >> 16, px = xlo + (k - dy * w), py = ylo + dy;
            const float xf = (float)px, yf = (float)py;
            const float n0 = edge_eval(e, 0, xf, yf), n1 = edge_eval(e, 1, xf, yf), n2 = edge_eval(e, 2, xf, yf);
            float al, be, ga;
            if (rcp) {
                al = div_rcp(n0, e.den[0], y0);
                be = div_rcp(n1, e.den[1], y1);
                ga = div_rcp(n2, e.den[2], y2);
            } else {
                al = fD(n0, e.den[0]);
                be = fD(n1, e.den[1]);
                ga = fD(n2, e.den[2]);
            }
            const float depth = interp(al, be, ga, da, db, dc);
            if (depth < clear_depth) atomicMin(vis + (uint64_t)py * width + px, depth_key(depth, seq));
        }
        return;
    }
    for (uint64_t k = 0; k < n; k++) {
        float al, be, ga;
        if (covered(e, (float)x, (float)y, al, be, ga)) {
            const float depth = interp(al, be, ga, da, db, dc);
            if (depth < clear_depth) atomicMin(vis + (uint64_t)y * width + x, depth_key(depth, seq));
        }
        if (++x == xe) {
            x = xlo;
            y++;
        }
    }
}

// Texel fetch of TextureMap::get_rgb_slice (scene/mod.rs:154-168) with the
// reference's wrapping usize arithmetic; false where the reference's slice
// index would panic.
__device__ __forceinline__ bool tex_rgb(const DgTexDev& tx, float u, float v, uint32_t& rgb) {
    const float fu = floorf(fM(u, fS(tx.fw, 1.0f)));
    const float fv = floorf(fM(v, fS(tx.fh, 1.0f)));
    uint64_t off;
    if (tx.small != 0u && fu >= 0.0f && fu < tx.fw && fv >= 0.0f && fv < tx.fh) {
        // both indices inside the map: the wrapping usize arithmetic below reduces
        // to this 32-bit one (the offset is below len < 2^32)
        off = ((tx.height - 1u - (uint32_t)fv) * tx.width + (uint32_t)fu) * tx.comps;
    } else {
        const uint64_t ui = as_usize(fu);
        const uint64_t vi = (uint64_t)tx.height - 1ull - as_usize(fv);
        off = (vi * (uint64_t)tx.width + ui) * (uint64_t)tx.comps;
    }
    if (tx.len < 3ull || off > tx.len - 3ull) return false;
    const uint64_t w = off >> 2;
    const uint32_t sh = (uint32_t)(off & 3ull) * 8u;
    const uint32_t lo = __ldg(tx.words + w);
    // the three bytes span two words only when the offset is not word aligned
    rgb = sh <= 8u ? (lo >> sh) : __funnelshift_r(lo, __ldg(tx.words + w + 1), sh);
    return true;
}

// Three image bytes at byte offset off (off <= len - 3) as the low 24 bits.
__device__ __forceinline__ uint32_t tex_bytes3(const DgTexDev& tx, uint64_t off) {
    const uint64_t w = off >> 2;
    const uint32_t sh = (uint32_t)(off & 3ull) * 8u;
    const uint32_t lo = __ldg(tx.words + w);
    return sh <= 8u ? (lo >> sh) : __funnelshift_r(lo, __ldg(tx.words + w + 1), sh);
}

// Extension (no counterpart in the reference, which samples the nearest texel):
// bilinear fetch. x = u * (W - 1), y = v * (H - 1) as in get_rgb_slice; the base
// texel (floor x, floor y) has the nearest texel's wrapping offset; its
// neighbours are the next column (when it exists, else the same column) and the
// next row up (the previous row in memory, when it exists, else the same row).
// Per channel, with c = byte / 255, ax = x - floor x, ay = y - floor y:
// t0 = c00 (1 - ax) + c01 ax, t1 = c10 (1 - ax) + c11 ax, c = t0 (1 - ay) + t1 ay.
// False (the texture-range error) when any of the four offsets is past the image.
__device__ __noinline__ bool tex_bilinear(const DgTexDev& tx, float u, float v, const float* inv255, V3& out) {
    const float x = fM(u, fS(tx.fw, 1.0f)), y = fM(v, fS(tx.fh, 1.0f));
    const float fx = floorf(x), fy = floorf(y);
    const float ax = fS(x, fx), ay = fS(y, fy);
    const uint64_t ui = as_usize(fx);
    const uint64_t vi = (uint64_t)tx.height - 1ull - as_usize(fy);
    const uint64_t o00 = (vi * (uint64_t)tx.width + ui) * (uint64_t)tx.comps;
    const uint64_t dx = (ui + 1ull < (uint64_t)tx.width) ? (uint64_t)tx.comps : 0ull;
    const uint64_t dy = (vi >= 1ull && vi < (uint64_t)tx.height) ? (uint64_t)tx.width * tx.comps : 0ull;
    const uint64_t off[4] = {o00, o00 + dx, o00 - dy, o00 - dy + dx};
    uint32_t c[4];
    for (int k = 0; k < 4; k++) {
        if (tx.len < 3ull || off[k] > tx.len - 3ull) return false;
        c[k] = tex_bytes3(tx, off[k]);
    }
    const float bx = fS(1.0f, ax), by = fS(1.0f, ay);
    float ch[3];
    for (int i = 0; i < 3; i++) {
        const uint32_t sh = 8u * (uint32_t)i;
        const float c00 = inv255[(c[0] >> sh) & 0xFFu], c01 = inv255[(c[1] >> sh) & 0xFFu];
        const float c10 = inv255[(c[2] >> sh) & 0xFFu], c11 = inv255[(c[3] >> sh) & 0xFFu];
        const float t0 = fA(fM(c00, bx), fM(c01, ax));
        const float t1 = fA(fM(c10, bx), fM(c11, ax));
        ch[i] = fA(fM(t0, by), fM(t1, ay));
    }
    out = V3{ch[0], ch[1], ch[2]};
    return true;
}

// A triangle's material as the shading formula uses it.
struct MatVals {
    V3 ka, kd, ks;
    uint32_t map_ka, map_kd;
};

// Texture descriptors the shade pass keeps in shared memory (the rest are read
// from the job's table).
#define DG_SMEM_TEX 32u

// Shading of canvas.rs:713-741 from the interpolated texture coordinates,
// normal and per-light vectors: lv(l, lt, h) gives the interpolated light and
// halfway vectors of light l. EXT: the texture maps may use the bilinear
// extension (false compiles the reference's nearest fetch alone, which keeps
// the extension's out-of-line call and its register spills off that path).
template <bool EXT, class LV>
__device__ __forceinline__ uint32_t shade_colour(const DgJobDev& job, const DgTexDev* stex, const DgFrameDev& fr,
                                                 const MatVals& m, float pu, float pv, V3 pn, const float* inv255,
                                                 int& errc, LV lv) {
    const uint32_t nst = job.ntex < DG_SMEM_TEX ? job.ntex : DG_SMEM_TEX;
    // descriptors by value: shared-memory loads for the first DG_SMEM_TEX maps
    auto tex_desc = [&](uint32_t i) -> DgTexDev {
        if (i < nst) return stex[i];
        DgTexDev t;
        const uint4* g = reinterpret_cast<const uint4*>(job.tex + i);
        uint4* d = reinterpret_cast<uint4*>(&t);
        d[0] = __ldg(g);
        d[1] = __ldg(g + 1);
        d[2] = __ldg(g + 2);
        return t;
    };
    const DgTexDev tkd = tex_desc(m.map_kd);
    const DgTexDev tka = m.map_ka == m.map_kd ? tkd : tex_desc(m.map_ka);
    // Pixel::normalized_as_vec3 (canvas.rs:81-87): byte / 255.0, looked up in a
    // table of the 256 correctly rounded quotients; or the bilinear extension
    auto sample = [&](const DgTexDev& t, V3& out) -> bool {
        if (EXT && t.filter == DG_FILTER_BILINEAR) return tex_bilinear(t, pu, pv, inv255, out);
        uint32_t rgb = 0;
        if (!tex_rgb(t, pu, pv, rgb)) return false;
        out = V3{inv255[rgb & 0xFFu], inv255[(rgb >> 8) & 0xFFu], inv255[(rgb >> 16) & 0xFFu]};
        return true;
    };
    V3 diffuse, ambient;
    if (!sample(tkd, diffuse)) {
        errc = DG_E_TEXTURE_RANGE;
        return 0u;
    }
    if (m.map_ka == m.map_kd) {
        ambient = diffuse;  // the same map at the same coordinates
    } else if (!sample(tka, ambient)) {
        errc = DG_E_TEXTURE_RANGE;
        return 0u;
    }
    const V3 c_l = m.ks;
    const V3 c_r = {fM(diffuse.x, m.kd.x), fM(diffuse.y, m.kd.y), fM(diffuse.z, m.kd.z)};
    const V3 c_a = {fM(ambient.x, m.ka.x), fM(ambient.y, m.ka.y), fM(ambient.z, m.ka.z)};
    const uint32_t nl = fr.nlights;
    // The per-light H.N dots are taken in the first loop (one read of each light's
    // vectors) and used in the second, in the reference's order of operations.
    float hn[DG_MAXL];
    V3 inner = c_a;
#pragma unroll
    for (uint32_t l = 0; l < DG_MAXL; l++) {
        if (l < nl) {
            V3 lt, h;
            lv(l, lt, h);
            const float ln = vdot(lt, pn);
            const float mx = ln > 0.0f ? ln : 0.0f;  // 0.0_f32.max(x): NaN -> 0
            inner = vadd(inner, vmul(c_l, fS(1.0f, mx)));
            hn[l] = vdot(h, pn);
        }
    }
    V3 col = {fM(c_r.x, inner.x), fM(c_r.y, inner.y), fM(c_r.z, inner.z)};
    const int32_t ex = fr.exponent;
#pragma unroll
    for (uint32_t l = 0; l < DG_MAXL; l++)
        if (l < nl) col = vadd(col, vmul(c_l, powi(hn[l], ex)));
    // Pixel::from_normalized_vec3 (canvas.rs:89-92), stored as b,g,r,255
    const V3 sc = vmul(col, 255.0f);
    const uint32_t R = as_u8(sc.x), G = as_u8(sc.y), B = as_u8(sc.z);
    return B | (G << 8) | (R << 16) | (255u << 24);
}

// Row `row` of the light/halfway table for light l: (lt.x, lt.y, lt.z, h.x), (h.y, h.z, -, -).
__device__ __forceinline__ const float4* shade_row(const DgJobDev& job, uint32_t row, uint32_t l) {
    return job.vshade + ((uint64_t)row * job.shade_stride + l) * 2;
}

// Shades the winning fragment of pixel (x, y) from its triangle record:
// canvas.rs:682-741.
// World position of job vertex v (the segment that holds it, then its position).
__device__ __forceinline__ V3 job_vertex(const DgJobDev& job, uint32_t v) {
    const uint32_t si = last_le(job.nsegs, v, [&](uint32_t i) { return job.segs[i].vtx_begin; });
    const DgSegDev& sg = job.segs[si];
    const float4 p4 = __ldg(sg.pos + (v - sg.vtx_begin));
    return V3{p4.x, p4.y, p4.z};
}

// Wp (frames with DG_FRAME_PERSPECTIVE, else null): the record's inv_w3. EXT
// as for shade_colour (false: the reference's interpolation and fetch only).
// LAZY: the record may carry DG_TRI_LAZY, and then the light/halfway vectors of
// its three vertices are computed here from their positions (shade_vertex's
// operations) instead of read from job.vshade.
template <bool EXT, bool LAZY>
__device__ __forceinline__ uint32_t shade_from_record(const DgJobDev& job, const DgFrameDev& fr, const DgTriRec* R,
                                                      uint32_t x, uint32_t y, const float* inv255,
                                                      const DgTexDev* stex, float& depth_out, int& errc,
                                                      const float4* Wp) {
    errc = DG_OK;
    EdgeSet e;
    load_edges(R, e);
    const float4* q = reinterpret_cast<const float4*>(R);
    const float4 dd = __ldg(q + 4), fu = __ldg(q + 5), fv = __ldg(q + 6);
    const float4 fx = __ldg(q + 7), fy = __ldg(q + 8), fz = __ldg(q + 9);
    const uint4 rows = __ldg(reinterpret_cast<const uint4*>(R) + 10);
    const uint4 last = __ldg(reinterpret_cast<const uint4*>(R) + 11);
    const float xf = (float)x, yf = (float)y;
    float al = fD(edge_eval(e, 0, xf, yf), e.den[0]);
    float be = fD(edge_eval(e, 1, xf, yf), e.den[1]);
    float ga = fD(edge_eval(e, 2, xf, yf), e.den[2]);
    depth_out = interp(al, be, ga, dd.x, dd.y, dd.z);
    if (EXT && Wp) persp_weights(al, be, ga, __ldg(Wp));  // coverage and depth keep the screen-space weights
    const float pu = interp(al, be, ga, fu.x, fu.y, fu.z);
    const float pv = interp(al, be, ga, fv.x, fv.y, fv.z);
    const V3 pn = {interp(al, be, ga, fx.x, fx.y, fx.z), interp(al, be, ga, fy.x, fy.y, fy.z),
                   interp(al, be, ga, fz.x, fz.y, fz.z)};
    MatVals m;
    m.ka = V3{dd.w, fu.w, fv.w};
    m.kd = V3{fx.w, fy.w, fz.w};
    m.ks = V3{__uint_as_float(rows.w), __uint_as_float(last.x), __uint_as_float(last.y)};
    m.map_ka = last.z;
    m.map_kd = last.w;
    const bool lazy = LAZY && (e.tie & DG_TRI_LAZY) != 0u;
    auto lv = [&](uint32_t l, V3& lt, V3& h) {
        float4 a, b, c, a1, b1, c1;
        if (LAZY && lazy) {
            // each vertex again per light (positions are cached loads): nothing is
            // held across the lights, which keeps the registers of the common path
            const V3 cam = {fr.cam[0], fr.cam[1], fr.cam[2]};
            auto vtx = [&](uint32_t v, float4& o0, float4& o1) {
                const V3 p = job_vertex(job, v);
                V3 t, hh;
                light_halfway(fr, p, vnormalized(vsub(p, cam)), l, t, hh);
                o0 = make_float4(t.x, t.y, t.z, hh.x);
                o1 = make_float4(hh.y, hh.z, 0.0f, 0.0f);
            };
            vtx(rows.x, a, a1);
            vtx(rows.y, b, b1);
            vtx(rows.z, c, c1);
        } else {
            if (DG_CHECKED) {
                const uint32_t nrow = job.total_vtx + job.vrow_extra + 6u * job.ntt;
                if (!DG_IN_RANGE(rows.x < nrow && rows.y < nrow && rows.z < nrow, job.err)) {
                    lt = h = V3{0.0f, 0.0f, 0.0f};
                    return;
                }
            }
            const float4* pa = shade_row(job, rows.x, l);
            const float4* pb = shade_row(job, rows.y, l);
            const float4* pc = shade_row(job, rows.z, l);
            a = __ldg(pa), b = __ldg(pb), c = __ldg(pc);
            a1 = __ldg(pa + 1), b1 = __ldg(pb + 1), c1 = __ldg(pc + 1);
        }
        lt = V3{interp(al, be, ga, a.x, b.x, c.x), interp(al, be, ga, a.y, b.y, c.y),
                interp(al, be, ga, a.z, b.z, c.z)};
        h = V3{interp(al, be, ga, a.w, b.w, c.w), interp(al, be, ga, a1.x, b1.x, c1.x),
               interp(al, be, ga, a1.y, b1.y, c1.y)};
    };
    return shade_colour<EXT>(job, stex, fr, m, pu, pv, pn, inv255, errc, lv);
}

// Shades the winning fragment of pixel (x, y) from its key alone (the triangle
// has no record: the record buffers were full): the triangle is set up and
// clipped again here.
__device__ __noinline__ uint32_t shade_without_record(const DgJobDev& job, const DgFrameDev& fr, uint32_t seq,
                                                      uint32_t x, uint32_t y, const float* inv255,
                                                      const DgTexDev* stex, float& depth_out, int& errc) {
    errc = DG_OK;
    const uint32_t tl = seq >> 2, o = seq & 3u;
    const uint32_t si =
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
    triangle_vertices(job, sg, fr, tp, r);
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
    const float xf = (float)x, yf = (float)y;
    float al = fD(edge_eval(e, 0, xf, yf), e.den[0]);
    float be = fD(edge_eval(e, 1, xf, yf), e.den[1]);
    float ga = fD(edge_eval(e, 2, xf, yf), e.den[2]);
    depth_out = interp(al, be, ga, tr.da, tr.db, tr.dc);
    if (fr.flags & DG_FRAME_PERSPECTIVE) {
        float4 iw;
        if (!clipped) {
            const float4 pa = __ldg(sg.pos + vi[0]), pb = __ldg(sg.pos + vi[1]), pc = __ldg(sg.pos + vi[2]);
            iw = inv_w3(fr, V3{pa.x, pa.y, pa.z}, V3{pb.x, pb.y, pb.z}, V3{pc.x, pc.y, pc.z});
        } else {
            iw = inv_w3(fr, P.pos[P.out[o][0]], P.pos[P.out[o][1]], P.pos[P.out[o][2]]);
        }
        persp_weights(al, be, ga, iw);
    }

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
    if (tp.w >= sg.nmats) {
        errc = DG_E_CUDA;
        return 0u;
    }
    const DgMatDev& md = sg.mats[tp.w];
    MatVals m;
    m.ka = V3{md.ka[0], md.ka[1], md.ka[2]};
    m.kd = V3{md.kd[0], md.kd[1], md.kd[2]};
    m.ks = V3{md.ks[0], md.ks[1], md.ks[2]};
    m.map_ka = md.map_ka;
    m.map_kd = md.map_kd;
    // Clip vertices' light/halfway vectors come from the input vertices' rows
    // through the clip program (clip_shade_rows computes the same values).
    auto comp = [&](uint32_t l, int c) {
        auto at = [&](int k) {
            return __ldg(reinterpret_cast<const float*>(shade_row(job, sg.vtx_begin + vi[k], l)) + c);
        };
        return field(at(0), at(1), at(2));
    };
    auto lv = [&](uint32_t l, V3& lt, V3& h) {
        lt = V3{comp(l, 0), comp(l, 1), comp(l, 2)};
        h = V3{comp(l, 3), comp(l, 4), comp(l, 5)};
    };
    return shade_colour<true>(job, stex, fr, m, pu, pv, pn, inv255, errc, lv);
}

inline unsigned grid_for(uint64_t n, unsigned cap) {
    uint64_t g = (n + 255) / 256;
    if (g < 1) g = 1;
    return (unsigned)(g < cap ? g : cap);
}

// Programmatic dependent launch: the kernel may be scheduled while the previous
// kernel of the stream drains; it calls wait_previous_kernel() before reading
// anything that kernel wrote.
template <class Arg>
cudaError_t launch_dependent(void (*kern)(Arg), unsigned grid, unsigned block, const Arg& arg, cudaStream_t s) {
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
    return cudaLaunchKernelEx(&cfg, kern, arg);
}

}  // namespace
