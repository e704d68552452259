// dg_api.cu -- host side of the GB300 rasterizer: the C ABI declared in
// include/draw_gpu.h, resource management in HBM, the per-frame host setup of
// Scene::render (camera basis, transformation matrix, view planes) and the
// launch sequence of one render job.
//
// Host floating point follows the reference's Rust semantics: this file is
// compiled with -ffp-contract=off, so every expression below rounds each
// operation to f32 in source order.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "dg_host.h"

namespace dgh {

namespace {

HM4 hm_zero() {
    HM4 r;
    std::memset(&r, 0, sizeof(r));
    return r;
}
HM4 hm_mul(const HM4& a, const HM4& b) {  // linalg.rs:328-344, accumulator starts at 0.0
    HM4 c = hm_zero();
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) {
            float acc = 0.0f;
            for (int k = 0; k < 4; k++) acc = acc + a.m[i][k] * b.m[k][j];
            c.m[i][j] = acc;
        }
    return c;
}
void hm_vec(const HM4& a, const float v[4], float out[4]) {  // linalg.rs:346-360
    for (int i = 0; i < 4; i++) {
        float acc = 0.0f;
        for (int j = 0; j < 4; j++) acc = acc + a.m[i][j] * v[j];
        out[i] = acc;
    }
}

const float kRadsPerDeg = 3.14159265358979323846f / 180.0f;  // f32::to_radians

dg_status camera_basis(const Camera& c, HM4& b) {  // scene/mod.rs:415-428
    if (!(hnorm(c.u) > 0.0f && hnorm(c.v) > 0.0f && hnorm(c.w) > 0.0f)) return DG_E_CAMERA;
    b = hm_zero();
    const HV3 cols[3] = {c.u, c.v, c.w};
    for (int j = 0; j < 3; j++) {
        b.m[0][j] = cols[j].x;
        b.m[1][j] = cols[j].y;
        b.m[2][j] = cols[j].z;
    }
    b.m[3][3] = 1.0f;
    return DG_OK;
}

}  // namespace

dg_status camera_init(Camera& c, HV3 pos, HV3 dir, float ratio, float near_, float far_, float fov_x) {
    // Camera::new, scene/mod.rs:297-357
    float rad = fov_x * kRadsPerDeg;
    float right = std::fabs(near_) * std::tan(rad / 2.0f);
    float left = -right;
    float top = (1.0f / ratio) * right;
    float bottom = -top;
    if (!(fov_x < 180.0f) || !(near_ < 0.0f) || !(near_ > far_) || !(right > left) || !(top > bottom))
        return DG_E_CAMERA;
    c.position = pos;
    c.direction = hnormalized(dir);
    c.up = h3(0.0f, 1.0f, 0.0f);
    c.top = top;
    c.bottom = bottom;
    c.right = right;
    c.left = left;
    c.near_ = near_;
    c.far_ = far_;
    c.u = c.v = c.w = h3(0.0f, 0.0f, 0.0f);
    return DG_OK;
}

void camera_update_basis(Camera& c) {  // scene/mod.rs:438-451
    HV3 g = c.direction;
    HV3 w = hmul(hdiv(g, hnorm(g)), -1.0f);
    HV3 txw = hcross(c.up, w);
    HV3 u = hdiv(txw, hnorm(txw));
    HV3 v = hcross(w, u);
    c.u = hnormalized(u);
    c.v = hnormalized(v);
    c.w = hnormalized(w);
}

dg_status camera_op(Scene& s, int32_t op, const float* a) {
    Camera& cam = s.cam;
    switch (op) {
        case 0: cam.position = hadd(cam.position, hmul(cam.up, a[0])); break;   // move_up :381-383
        case 1: cam.position = hadd(cam.position, hmul(cam.up, -a[0])); break;  // move_down :385-387
        case 2: cam.position = hadd(cam.position, hmul(cam.u, -a[0])); break;   // move_left :389-391
        case 3: cam.position = hadd(cam.position, hmul(cam.u, a[0])); break;    // move_right :393-395
        case 4: cam.position = hadd(cam.position, hmul(hnormalized(hcross(cam.up, cam.u)), a[0])); break;  // :397-400
        case 5: cam.position = hadd(cam.position, hmul(hnormalized(hcross(cam.u, cam.up)), a[0])); break;  // :402-405
        case 6: {  // rotate_origin: Matrix4::rotate_y(theta.to_radians()) * v.as_vec4(), :407-413
            float th = a[0] * kRadsPerDeg;
            float sn = std::sin(th), cs = std::cos(th);
            HM4 r = hm_zero();
            r.m[0][0] = cs; r.m[0][2] = sn; r.m[1][1] = 1.0f; r.m[2][0] = -sn; r.m[2][2] = cs; r.m[3][3] = 1.0f;
            float p[4] = {cam.position.x, cam.position.y, cam.position.z, 1.0f}, po[4];
            float d[4] = {cam.direction.x, cam.direction.y, cam.direction.z, 1.0f}, dout[4];
            hm_vec(r, p, po);
            hm_vec(r, d, dout);
            cam.position = h3(po[0], po[1], po[2]);
            cam.direction = h3(dout[0], dout[1], dout[2]);
            break;
        }
        case 7: cam.position = h3(a[0], a[1], a[2]); break;  // set_pos :377-379
        case 8: {                                             // Scene::move_camera_direction :803-813
            int32_t dx = (int32_t)a[0], dy = (int32_t)a[1];
            if (!((int64_t)dx < (int64_t)s.width) || !((int64_t)dy < (int64_t)s.height)) return DG_E_INVALID;
            float fx = (float)dx / (float)s.width, fy = (float)dy / (float)s.height;
            cam.direction = hnormalized(hadd(hadd(cam.direction, hmul(cam.u, fx)), hmul(cam.v, fy)));  // :430-432
            camera_update_basis(cam);
            break;
        }
        default: return DG_E_INVALID;
    }
    return DG_OK;
}

dg_status frame_setup(Scene& s, float M[4][4], float planes[6][4]) {
    Camera& c = s.cam;
    const float nx = (float)s.width, ny = (float)s.height;
    const float n = c.near_, f = c.far_, r = c.right, l = c.left, t = c.top, b = c.bottom;
    // Camera::gen_matrix, scene/mod.rs:453-479
    HM4 tr = hm_zero();
    tr.m[0][0] = tr.m[1][1] = tr.m[2][2] = tr.m[3][3] = 1.0f;
    tr.m[0][3] = -c.position.x;
    tr.m[1][3] = -c.position.y;
    tr.m[2][3] = -c.position.z;
    camera_update_basis(c);
    HM4 basis;
    dg_status e = camera_basis(c, basis);
    if (e) return e;
    HM4 bt = basis;
    for (int i = 0; i < 4; i++)
        for (int j = 0; j < 4; j++) bt.m[i][j] = basis.m[j][i];
    HM4 view = hm_mul(bt, tr);
    HM4 persp = hm_zero();
    persp.m[0][0] = n;
    persp.m[1][1] = n;
    persp.m[2][2] = n + f;
    persp.m[2][3] = -(n * f);
    persp.m[3][2] = 1.0f;
    HM4 orth = hm_zero();
    orth.m[0][0] = 2.0f / (r - l);
    orth.m[0][3] = -(r + l) / (r - l);
    orth.m[1][1] = 2.0f / (t - b);
    orth.m[1][3] = -(t + b) / (t - b);
    orth.m[2][2] = 2.0f / (n - f);
    orth.m[2][3] = -(n + f) / (n - f);
    orth.m[3][3] = 1.0f;
    HM4 vp = hm_zero();
    vp.m[0][0] = nx / 2.0f;
    vp.m[0][3] = (nx - 1.0f) / 2.0f;
    vp.m[1][1] = ny / 2.0f;
    vp.m[1][3] = (ny - 1.0f) / 2.0f;
    vp.m[2][2] = 1.0f;
    vp.m[3][3] = 1.0f;
    HM4 full = hm_mul(hm_mul(hm_mul(vp, orth), persp), view);
    std::memcpy(M, full.m, sizeof(full.m));

    // Camera::gen_view_planes, scene/mod.rs:481-593
    camera_update_basis(c);
    e = camera_basis(c, basis);
    if (e) return e;
    auto world = [&](float x, float y, float z) {
        float in[4] = {x, y, z, 1.0f}, out[4];
        hm_vec(basis, in, out);
        return hadd(h3(out[0] / out[3], out[1] / out[3], out[2] / out[3]), c.position);
    };
    HV3 urn = world(r, t, n), uln = world(l, t, n), lrn = world(r, b, n), lln = world(l, b, n);
    float xc = (l + r) / 2.0f, yc = (b + t) / 2.0f;
    HV3 ucf = world(xc, (f * t) / n, f), lcf = world(xc, (f * b) / n, f);
    HV3 rcf = world((f * r) / n, yc, f), lfc = world((f * l) / n, yc, f);
    HV3 vis = hdiv(hadd(urn, lcf), 2.0f);
    const HV3 pts[6][3] = {{urn, lrn, lln}, {lfc, rcf, ucf}, {rcf, urn, lrn},
                           {lfc, lln, uln}, {ucf, uln, urn}, {lcf, lln, lrn}};
    for (int p = 0; p < 6; p++) {  // ViewPlane::new, scene/mod.rs:603-632
        HV3 pv = hsub(pts[p][1], pts[p][0]);
        HV3 qv = hsub(pts[p][2], pts[p][1]);
        HV3 nn = hcross(pv, qv);
        float k = -hdot(nn, pts[p][0]);
        float tv = hdot(nn, vis) + k;
        if (tv < 0.0f) {
            nn = hcross(qv, pv);
            k = -hdot(nn, pts[p][0]);
            tv = hdot(nn, vis) + k;
            if (!(tv > 0.0f)) return DG_E_CAMERA;
        }
        planes[p][0] = nn.x;
        planes[p][1] = nn.y;
        planes[p][2] = nn.z;
        planes[p][3] = k;
    }
    return DG_OK;
}

}  // namespace dgh

using namespace dgh;

namespace {

dg_status cuda_ok(cudaError_t e) { return e == cudaSuccess ? DG_OK : DG_E_CUDA; }
#define DG_CUDA(x)                                                         \
    do {                                                                   \
        cudaError_t _e = (x);                                              \
        if (_e != cudaSuccess) {                                           \
            return _e == cudaErrorMemoryAllocation ? DG_E_OOM : DG_E_CUDA; \
        }                                                                  \
    } while (0)

template <class T>
dg_status dalloc(T** p, size_t n) {
    *p = nullptr;
    if (n == 0) n = 1;
    cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? DG_E_OOM : DG_E_CUDA;
    }
    return DG_OK;
}
template <class T>
void dfree(T*& p) {
    if (p) cudaFree((void*)p);
    p = nullptr;
}

dg_status tex_upload(const uint8_t* img, uint64_t len, uint32_t w, uint32_t h, uint32_t comps, TexMap& out) {
    uint64_t nwords = (len + 3) / 4 + 1;
    std::vector<uint32_t> words(nwords, 0u);
    if (len) std::memcpy(words.data(), img, len);
    dg_status e = dalloc(&out.d_words, nwords);
    if (e) return e;
    DG_CUDA(cudaMemcpy(out.d_words, words.data(), nwords * 4, cudaMemcpyHostToDevice));
    out.len = len;
    out.w = w;
    out.h = h;
    out.comps = comps;
    return DG_OK;
}

// Grows a slot scratch buffer (synchronizing only that slot's stream).
template <class T>
dg_status grow(JobSlot& s, T** p, size_t* cap, size_t need) {
    if (*cap >= need && *p) return DG_OK;
    DG_CUDA(cudaStreamSynchronize(s.stream));
    if (*p) s.scratch_bytes -= *cap * sizeof(T);
    dfree(*p);
    size_t n = std::max(need, (size_t)(*cap * 3 / 2));
    dg_status e = dalloc(p, n);
    if (e) {
        *cap = 0;
        return e;
    }
    *cap = n;
    s.scratch_bytes += n * sizeof(T);
    return DG_OK;
}

void free_object(Object& o) {
    dfree(o.d_pos); dfree(o.d_nrm); dfree(o.d_uv);
    dfree(o.d_tri_pos); dfree(o.d_tri_uv); dfree(o.d_tri_nrm); dfree(o.d_mats);
    for (int b = 0; b < 2; b++)
        for (int k = 0; k < 3; k++) dfree(o.d_tt[b][k]);
}

Scene* get_scene(dg_ctx* c, int32_t id) {
    if (!c || id < 0 || (size_t)id >= c->scenes.size()) return nullptr;
    return &c->scenes[id];
}
// Every operation on a canvas looks it up here, so a pending asynchronous read
// is ordered before whatever the context stream does to the canvas next.
Canvas* get_canvas(dg_ctx* c, int32_t id) {
    if (!c || id < 0 || (size_t)id >= c->canvases.size() || !c->canvases[id].alive) return nullptr;
    Canvas* v = &c->canvases[id];
    if (v->read_pending) {
        cudaStreamWaitEvent(c->main.stream, v->ev_read, 0);
        v->read_pending = false;
    }
    return v;
}
void free_canvas(Canvas& v) {
    dfree(v.d_colour); dfree(v.d_depth); dfree(v.d_vis); dfree(v.d_cells);
    if (v.ev_rendered) cudaEventDestroy(v.ev_rendered);
    if (v.ev_read) cudaEventDestroy(v.ev_read);
    if (v.h_err) cudaFreeHost(v.h_err);
    v.h_err = nullptr;
    v.ev_rendered = v.ev_read = nullptr;
    v.read_pending = false;
}
Object* get_object(dg_ctx* c, int32_t id) {
    if (!c || id < 0 || (size_t)id >= c->objects.size() || !c->objects[id].alive) return nullptr;
    return &c->objects[id];
}

}  // namespace

namespace dgh {

dg_status resolve_frames(dg_ctx* c, const int32_t* scenes, const int32_t* canvases, uint32_t n,
                         std::vector<Scene*>& sc, std::vector<FrameTarget>& tg) {
    sc.resize(n);
    tg.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        Scene* s = get_scene(c, scenes[i]);
        Canvas* cv = get_canvas(c, canvases[i]);
        if (!s || !cv) return DG_E_INVALID;
        if (!cv->depth_init) return DG_E_DEPTH_UNINIT;
        sc[i] = s;
        tg[i] = FrameTarget{cv->d_colour, cv->d_depth, cv->d_vis,   cv->w,      cv->h,
                            cv->depth_max, cv->off_x, cv->off_y, cv->d_cells, ++cv->epoch};
    }
    return DG_OK;
}

// dg_scene_render / dg_render_batch: resolves ids, then launches on the context slot.
dg_status render_job(dg_ctx* c, const int32_t* scenes, const int32_t* canvases, uint32_t n) {
    if (n == 0) return DG_OK;
    std::vector<Scene*> sc;
    std::vector<FrameTarget> tg;
    dg_status e = resolve_frames(c, scenes, canvases, n, sc, tg);
    if (e) return e;
    // An object with transparent meshes advances its painter's order once per
    // render of it, and a canvas holds one frame's visibility keys: frames that
    // render such an object or a canvas again start a new job.
    uint32_t first = 0;
    std::vector<int32_t> seen, seen_canvas;
    for (uint32_t i = 0; i < n; i++) {
        bool repeat = std::find(seen_canvas.begin(), seen_canvas.end(), canvases[i]) != seen_canvas.end();
        for (int32_t oid : sc[i]->objects)
            if (oid >= 0 && (size_t)oid < c->objects.size() && c->objects[oid].nt &&
                std::find(seen.begin(), seen.end(), oid) != seen.end())
                repeat = true;
        if (repeat) {
            e = launch_frames(c, c->main, sc.data() + first, tg.data() + first, i - first);
            if (e) return e;
            first = i;
            seen.clear();
            seen_canvas.clear();
        }
        for (int32_t oid : sc[i]->objects)
            if (oid >= 0 && (size_t)oid < c->objects.size() && c->objects[oid].nt) seen.push_back(oid);
        seen_canvas.push_back(canvases[i]);
    }
    return launch_frames(c, c->main, sc.data() + first, tg.data() + first, n - first);
}

}  // namespace dgh

namespace dgh {

dg_status set_device(dg_ctx* c) {
    if (c->device < 0) return DG_E_CUDA;  // host-only context: no device work
    return cuda_ok(cudaSetDevice(c->device));
}

dg_status slot_init(dg_ctx* c, JobSlot& s, cudaStream_t stream) {
    (void)c;
    s.stream = stream;
    for (int i = 0; i < JobSlot::kStage; i++) DG_CUDA(cudaEventCreateWithFlags(&s.stage_ev[i], cudaEventDisableTiming));
    for (int i = 0; i <= DG_NKERNELS; i++) DG_CUDA(cudaEventCreate(&s.ev[i]));
    dg_status e = dalloc(&s.d_counters, DG_NCOUNTERS);
    if (e) return e;
    e = dalloc(&s.d_err, 1);
    if (e) return e;
    DG_CUDA(cudaMemset(s.d_err, 0, 4));
    return DG_OK;
}

void slot_free(JobSlot& s) {
    if (s.stream) cudaStreamSynchronize(s.stream);
    dfree(s.d_vmask);
    dfree(s.d_vrec);
    dfree(s.d_vshade);
    dfree(s.d_vmark);
    dfree(s.d_queue);
    dfree(s.d_small);
    for (int k = 0; k < 2; k++) {
        dfree(s.d_tkey[k]); dfree(s.d_tval[k]); dfree(s.d_fkey[k]); dfree(s.d_fval[k]);
    }
    dfree(s.d_ttrec); dfree(s.d_tbox); dfree(s.d_tmeta); dfree(s.d_talpha); dfree(s.d_tcnt); dfree(s.d_tscan);
    dfree(s.d_hist);
    s.tsort_cap = s.tout_cap = s.frag_cap = s.hist_cap = 0;
    dfree(s.d_items);
    dfree(s.d_surv);
    dfree(s.d_rec_of);
    dfree(s.d_trec);
    dfree(s.d_trec_w);
    dfree(s.d_ttrec_w);
    s.trec_w_cap = s.ttrec_w_cap = 0;
    dfree(s.d_counters);
    dfree(s.d_err);
    for (int i = 0; i < JobSlot::kStage; i++) {
        if (s.h_stage[i]) cudaFreeHost(s.h_stage[i]);
        s.h_stage[i] = nullptr;
        dfree(s.d_stage[i]);
        if (s.stage_ev[i]) cudaEventDestroy(s.stage_ev[i]);
        s.stage_ev[i] = nullptr;
    }
    for (int i = 0; i <= DG_NKERNELS; i++) {
        if (s.ev[i]) cudaEventDestroy(s.ev[i]);
        s.ev[i] = nullptr;
    }
    s.scratch_bytes = 0;
}

dg_status slot_take_errors(JobSlot& s) {
    uint32_t err = 0;
    DG_CUDA(cudaMemcpy(&err, s.d_err, 4, cudaMemcpyDeviceToHost));
    if (!err) return DG_OK;
    uint32_t zero = 0;
    DG_CUDA(cudaMemcpy(s.d_err, &zero, 4, cudaMemcpyHostToDevice));
    for (int b = 1; b < 32; b++)
        if (err & (1u << b)) return (dg_status)b;
    return DG_E_CUDA;
}

dg_status sync_tex_table(dg_ctx* c, cudaStream_t stream) {
    if (!c->tex_dirty) return DG_OK;
    std::vector<DgTexDev> t(c->tex.size());
    for (size_t i = 0; i < c->tex.size(); i++) {
        t[i].words = c->tex[i].d_words;
        t[i].len = c->tex[i].len;
        t[i].width = c->tex[i].w;
        t[i].height = c->tex[i].h;
        t[i].comps = c->tex[i].comps;
        t[i].fw = (float)c->tex[i].w;
        t[i].fh = (float)c->tex[i].h;
        t[i].small = dg_tex_small(c->tex[i].len, c->tex[i].w, c->tex[i].h);
        t[i].filter = c->tex[i].filter;
        t[i].pad = 0;
    }
    DG_CUDA(cudaStreamSynchronize(stream));
    if (c->d_tex_cap < t.size()) {
        DG_CUDA(cudaDeviceSynchronize());  // the old table may still be read by other streams
        dfree(c->d_tex);
        size_t cap = std::max<size_t>(16, t.size() * 2);
        dg_status e = dalloc(&c->d_tex, cap);
        if (e) return e;
        c->d_tex_cap = cap;
    }
    DG_CUDA(cudaMemcpy(c->d_tex, t.data(), t.size() * sizeof(DgTexDev), cudaMemcpyHostToDevice));
    c->tex_dirty = false;
    return DG_OK;
}

// Queue capacity: one record per input triangle (clip outputs beyond it, and
// anything past 2^24 records, are rasterized in place by their warp).
size_t queue_records(uint64_t total_tri) {
    return std::min<size_t>(std::max<size_t>(1u << 16, (size_t)total_tri), (1u << 24) - 1);
}

// Triangle records: one per cull survivor plus room for clip outputs (the
// resolve pass shades the pixels of triangles without a record the long way).
size_t trec_records(uint64_t total_tri) { return (size_t)std::min<uint64_t>(dg_trec_cap(total_tri), 0xFFFFFFF0ull); }

uint64_t slot_scratch_after(const JobSlot& s, uint64_t V, uint64_t T, uint32_t L, uint64_t P) {
    auto cap_after = [](size_t cap, const void* p, size_t need) -> size_t {
        return (cap >= need && p) ? cap : std::max(need, cap * 3 / 2);
    };
    if (L == 0) L = 1;
    const size_t vmask = cap_after(s.vmask_cap, s.d_vmask, std::max<uint64_t>(V, 1));
    const size_t vrec = cap_after(s.vrec_cap, s.d_vrec, std::max<uint64_t>(V, 1));
    const size_t vshade = cap_after(s.vshade_cap, s.d_vshade, (V + dg_vrow_extra(T)) * L * 2);
    const size_t vmark = cap_after(s.vmark_cap, s.d_vmark, std::max<uint64_t>(V, 1));
    const size_t q = cap_after(s.queue_cap, s.d_queue, queue_records(T));
    const size_t sm = cap_after(s.small_cap, s.d_small, queue_records(T));
    const size_t qb = cap_after(s.items_cap, s.d_items, dg_items_cap(q));
    const size_t sv = cap_after(s.surv_cap, s.d_surv, std::max<uint64_t>(T, 1));
    const size_t ro = cap_after(s.rec_of_cap, s.d_rec_of, std::max<uint64_t>(T, 1));
    const size_t tr = cap_after(s.trec_cap, s.d_trec, trec_records(T));
    return vmask * sizeof(uint16_t) + vrec * sizeof(float4) + vshade * sizeof(float4) + vmark * sizeof(uint8_t) + (q + sm) * sizeof(DgQueueRec) +
           qb * sizeof(uint2) + (sv + ro) * sizeof(uint32_t) + tr * sizeof(DgTriRec);
}

dg_status build_job(dg_ctx* c, JobSlot& S, Scene* const* scenes, const FrameTarget* targets, uint32_t n,
                    JobBuild& B) {
    dg_status e = set_device(c);
    if (e) return e;
    std::vector<DgFrameDev>& frames = B.frames;
    std::vector<DgSegDev>& segs = B.segs;
    frames.assign(n, DgFrameDev{});
    segs.clear();
    uint64_t total_vtx = 0, total_tri = 0, total_tiles = 0, total_px = 0;
    uint64_t ntt = 0, tmesh_total = 0, max_frame_tt = 0;
    uint32_t stride = 1;
    bool any_persp = false, any_lazy = false;
    B.transparent_objects.clear();
    // Resolve tile height: the tile_rows knob, or (0) the tallest of 32, 16 and 8
    // rows whose tiles fill the resolve pass's resident blocks (4 per SM), else 8.
    // A tile's threads shade its covered pixels one after another (up to 4 each
    // at 32 rows), so a job of few tiles finishes sooner with shorter ones; a
    // job that fills the GPU gains nothing from them and pays their overhead.
    // Measured: 256x256 frames 57 -> 41 us (8 rows), 512x512 71 -> 51 us (8 rows),
    // 800x600 47 -> 40 us (16 rows), 1920x1080 best at 32 rows.
    uint32_t th = S.tile_rows;
    if (th == 0) {
        const uint64_t slots = 4ull * (uint64_t)(c->nsm > 0 ? c->nsm : 1);
        th = 8;
        for (uint32_t cand : {32u, 16u}) {
            uint64_t tiles = 0;
            for (uint32_t i = 0; i < n; i++)
                tiles += ((targets[i].w + DG_TILE_W - 1) / DG_TILE_W) * ((targets[i].h + cand - 1) / cand);
            if (tiles >= slots) {
                th = cand;
                break;
            }
        }
    }
    for (uint32_t i = 0; i < n; i++) {
        Scene& s = *scenes[i];  // frame_setup updates the camera basis, as Scene::render does
        const FrameTarget& tg = targets[i];
        for (int32_t oid : s.objects)
            if (oid < 0 || (size_t)oid >= c->objects.size() || !c->objects[oid].alive) return DG_E_INVALID;
        // An object with transparent meshes is sorted once per render of it and
        // keeps the order: a job renders it at most once.
        for (int32_t oid : s.objects)
            if (c->objects[oid].nt) {
                if (std::find(B.transparent_objects.begin(), B.transparent_objects.end(), oid) !=
                    B.transparent_objects.end())
                    return DG_E_LIMIT;
                B.transparent_objects.push_back(oid);
            }
        DgFrameDev& f = frames[i];
        std::memset(&f, 0, sizeof(f));
        e = frame_setup(s, f.M, f.plane);
        if (e) return e;
        f.cam[0] = s.cam.position.x;
        f.cam[1] = s.cam.position.y;
        f.cam[2] = s.cam.position.z;
        f.clear_depth = tg.clear_depth;
        f.nlights = (uint32_t)s.lights.size();
        for (size_t l = 0; l < s.lights.size(); l++) {
            f.light[l][0] = s.lights[l].x;
            f.light[l][1] = s.lights[l].y;
            f.light[l][2] = s.lights[l].z;
        }
        stride = std::max(stride, f.nlights);
        f.exponent = s.exponent;
        f.flags = s.interpolation == DG_INTERP_PERSPECTIVE ? DG_FRAME_PERSPECTIVE : 0u;
        any_persp = any_persp || f.flags != 0u;
        {
            // At least as many opaque triangles as pixels, and a light/halfway table
            // (32 bytes per vertex and light) beyond the L2: the small triangles'
            // vertices get no rows, and their shading computes the vectors for the
            // pixels they win. Measured: the 3840x2160 frame of 10M micro triangles and
            // 4 lights gains 5% (most of its triangles win no pixel); a 256x256 frame of
            // a 300k-triangle mesh and 1 light (a 5 MB table) lost 14%, so it keeps rows.
            uint64_t frame_tris = 0, frame_vtx = 0;
            for (int32_t oid : s.objects) {
                frame_tris += c->objects[oid].ntri_opaque;
                frame_vtx += c->objects[oid].nv;
            }
            if (frame_tris >= tg.w * tg.h && frame_vtx * s.lights.size() * 32u >= (128ull << 20)) {
                f.flags |= DG_FRAME_LAZY;
                any_lazy = true;
            }
            f.small_max_px = S.small_max_px != DG_SMALL_MAX_PX_AUTO ? S.small_max_px
                             : frame_tris >= tg.w * tg.h             ? DG_SMALL_MAX_PX_MICRO
                                                                     : DG_SMALL_MAX_PX;
        }
        f.off_x = tg.off_x;
        f.off_y = tg.off_y;
        f.width = (uint32_t)tg.w;
        f.height = (uint32_t)tg.h;
        f.vis = tg.vis;
        f.cells = tg.cells;
        f.epoch = tg.epoch;
        f.colour = tg.colour;
        f.depth = tg.depth;
        f.seg_begin = (uint32_t)segs.size();
        f.tile_begin = (uint32_t)total_tiles;
        f.tiles_x = (uint32_t)((tg.w + DG_TILE_W - 1) / DG_TILE_W);
        total_tiles += (uint64_t)f.tiles_x * ((tg.h + th - 1) / th);
        f.pix_begin = (uint32_t)total_px;
        total_px += tg.w * tg.h;
        if (total_px >= 0x80000000ull) return DG_E_LIMIT;  // job-wide pixel indices use 31 bits
        f.tt_begin = (uint32_t)ntt;
        const uint64_t frame_tt0 = ntt;
        uint64_t seq = 0;
        for (int32_t oid : s.objects) {
            Object& o = c->objects[oid];
            DgSegDev sg;
            std::memset(&sg, 0, sizeof(sg));
            sg.frame = i;
            sg.tri_begin = (uint32_t)total_tri;
            sg.vtx_begin = (uint32_t)total_vtx;
            sg.seq_base = (uint32_t)seq;
            sg.ntri = o.ntri_opaque;
            sg.nv = o.nv;
            sg.nmats = o.nmats;
            sg.pos = o.d_pos;
            sg.nrm = o.d_nrm;
            sg.uv = o.d_uv;
            sg.tri_pos = o.d_tri_pos;
            sg.tri_uv = o.d_tri_uv;
            sg.tri_nrm = o.d_tri_nrm;
            sg.mats = o.d_mats;
            sg.t_begin = (uint32_t)ntt;
            sg.nt = o.nt;
            sg.tmesh_base = (uint32_t)tmesh_total;
            sg.obj_rank = (uint32_t)(segs.size() - f.seg_begin);
            for (int k = 0; k < 3; k++) {
                sg.tsrc[k] = o.d_tt[o.tcur][k];
                sg.tdst[k] = o.d_tt[1 - o.tcur][k];
            }
            segs.push_back(sg);
            total_tri += o.ntri_opaque;
            total_vtx += o.nv;
            seq += o.ntri_opaque;
            ntt += o.nt;
            if (o.nt) tmesh_total += o.tmesh_off.size() - 1;
        }
        if (seq >= (1ull << 30)) return DG_E_LIMIT;
        max_frame_tt = std::max(max_frame_tt, ntt - frame_tt0);
        f.seg_count = (uint32_t)(segs.size() - f.seg_begin);
    }
    if (total_tri >= 0xFFFFFFFFull || total_vtx >= 0xFFFFFFFFull || total_tiles >= 0x7FFFFFFFull) return DG_E_LIMIT;
    if (ntt >= (1ull << 29) || tmesh_total >= (1ull << 24)) return DG_E_LIMIT;  // transparent keys and outputs
    if (segs.empty()) {  // keep a valid segment table
        DgSegDev sg;
        std::memset(&sg, 0, sizeof(sg));
        segs.push_back(sg);
    }
    e = sync_tex_table(c, S.stream);
    if (e) return e;
    e = grow(S, &S.d_vmask, &S.vmask_cap, std::max<uint64_t>(total_vtx, 1));
    if (e) return e;
    e = grow(S, &S.d_vrec, &S.vrec_cap, std::max<uint64_t>(total_vtx, 1));
    if (e) return e;
    const uint64_t vrow_extra = dg_vrow_extra(total_tri);
    // rows: job vertices, clip vertices of opaque triangles, 6 per transparent triangle
    e = grow(S, &S.d_vshade, &S.vshade_cap, (total_vtx + vrow_extra + 6 * ntt) * stride * 2);
    if (e) return e;
    const uint64_t fcap = std::min<uint64_t>(2 * total_px + 65536, 0x7FFFFFFFull);
    if (ntt) {
        const uint64_t nout = 4 * ntt;
        if (S.tsort_cap < ntt) {
            DG_CUDA(cudaStreamSynchronize(S.stream));
            for (int k = 0; k < 2; k++) {
                dfree(S.d_tkey[k]);
                dfree(S.d_tval[k]);
            }
            S.tsort_cap = 0;
            for (int k = 0; k < 2; k++) {
                if ((e = dalloc(&S.d_tkey[k], ntt)) || (e = dalloc(&S.d_tval[k], ntt))) return e;
            }
            S.tsort_cap = ntt;
        }
        if (S.tout_cap < nout) {
            DG_CUDA(cudaStreamSynchronize(S.stream));
            dfree(S.d_ttrec); dfree(S.d_tbox); dfree(S.d_tmeta); dfree(S.d_talpha); dfree(S.d_tcnt); dfree(S.d_tscan);
            S.tout_cap = 0;
            if ((e = dalloc(&S.d_ttrec, nout)) || (e = dalloc(&S.d_tbox, nout)) || (e = dalloc(&S.d_tmeta, nout)) ||
                (e = dalloc(&S.d_talpha, nout)) || (e = dalloc(&S.d_tcnt, nout)) || (e = dalloc(&S.d_tscan, nout + 1)))
                return e;
            S.tout_cap = nout;
        }
        if (S.frag_cap < fcap) {
            DG_CUDA(cudaStreamSynchronize(S.stream));
            for (int k = 0; k < 2; k++) {
                dfree(S.d_fkey[k]);
                dfree(S.d_fval[k]);
            }
            S.frag_cap = 0;
            for (int k = 0; k < 2; k++) {
                if ((e = dalloc(&S.d_fkey[k], fcap)) || (e = dalloc(&S.d_fval[k], fcap))) return e;
            }
            S.frag_cap = fcap;
        }
        const uint64_t tiles = (std::max(ntt, fcap) + DG_SORT_TILE - 1) / DG_SORT_TILE;
        e = grow(S, &S.d_hist, &S.hist_cap, 256 * tiles);
        if (e) return e;
    }
    e = grow(S, &S.d_surv, &S.surv_cap, std::max<uint64_t>(total_tri, 1));
    if (e) return e;
    e = grow(S, &S.d_rec_of, &S.rec_of_cap, std::max<uint64_t>(total_tri, 1));
    if (e) return e;
    e = grow(S, &S.d_trec, &S.trec_cap, trec_records(total_tri));
    if (e) return e;
    if (any_persp) {
        e = grow(S, &S.d_trec_w, &S.trec_w_cap, S.trec_cap);
        if (e) return e;
        if (ntt) {
            e = grow(S, &S.d_ttrec_w, &S.ttrec_w_cap, 4 * ntt);
            if (e) return e;
        }
    }
    const size_t want_mark = std::max<uint64_t>(total_vtx, 1);
    if (S.vmark_cap < want_mark) {
        e = grow(S, &S.d_vmark, &S.vmark_cap, want_mark);
        if (e) return e;
        DG_CUDA(cudaMemsetAsync(S.d_vmark, 0, S.vmark_cap * sizeof(uint8_t), S.stream));
    }
    const size_t want_queue = queue_records(total_tri);
    if (S.queue_cap < want_queue) {
        e = grow(S, &S.d_queue, &S.queue_cap, want_queue);
        if (e) return e;
        e = grow(S, &S.d_items, &S.items_cap, dg_items_cap(S.queue_cap));
        if (e) return e;
    }
    if (S.small_cap < want_queue) {
        e = grow(S, &S.d_small, &S.small_cap, want_queue);
        if (e) return e;
    }

    B.fbytes = frames.size() * sizeof(DgFrameDev);
    B.sbytes = segs.size() * sizeof(DgSegDev);
    DgJobDev& job = B.job;
    std::memset(&job, 0, sizeof(job));
    job.nframes = n;
    job.nsegs = (uint32_t)segs.size();
    job.total_vtx = (uint32_t)total_vtx;
    job.total_tri = (uint32_t)total_tri;
    job.total_tiles = (uint32_t)total_tiles;
    job.shade_stride = stride;
    job.vmask = S.d_vmask;
    job.vrec = S.d_vrec;
    job.vshade = S.d_vshade;
    job.vrow_extra = (uint32_t)vrow_extra;
    job.vmark = S.d_vmark;
    job.surv = S.d_surv;
    job.rec_of = S.d_rec_of;
    job.trec = S.d_trec;
    job.trec_w = any_persp ? S.d_trec_w : nullptr;
    job.ext = any_persp ? 1u : 0u;
    job.lazy = any_lazy ? 1u : 0u;
    for (const TexMap& t : c->tex)
        if (t.filter != DG_FILTER_NEAREST) job.ext = 1u;
    job.ttrec_w = any_persp && ntt ? S.d_ttrec_w : nullptr;
    job.trec_cap = (uint32_t)std::min<size_t>(S.trec_cap, 0xFFFFFFF0ull);
    if (S.record_limit) job.trec_cap = std::min(job.trec_cap, S.record_limit);
    job.queue = S.d_queue;
    job.small = S.d_small;
    job.small_cap = (uint32_t)std::min<size_t>(S.small_cap, 0xFFFFFFF0ull);
    job.items = S.d_items;
    job.items_cap = (uint32_t)std::min<size_t>(S.items_cap, 0xFFFFFFF0ull);
    job.queue_cap = (uint32_t)std::min<size_t>(S.queue_cap, (1u << 24) - 1);
    job.item_units = S.item_units;
    job.cnt = S.d_counters;
    job.total_px = (uint32_t)total_px;
    job.tile_rows = th;
    job.tex = c->d_tex;
    job.ntex = (uint32_t)c->tex.size();
    job.err = S.d_err;
    B.launches = (total_vtx ? 1 : 0) + (total_tri ? 3 : 0) + (total_tiles ? 1 : 0);
    B.cfg.tplan = DgTransparentPlan{};
    if (ntt) {
        job.ntt = (uint32_t)ntt;
        job.fcap = (uint32_t)fcap;
        for (int k = 0; k < 2; k++) {
            job.tkey[k] = S.d_tkey[k];
            job.tval[k] = S.d_tval[k];
            job.fkey[k] = S.d_fkey[k];
            job.fval[k] = S.d_fval[k];
        }
        job.ttrec = S.d_ttrec;
        job.tbox = S.d_tbox;
        job.tmeta = S.d_tmeta;
        job.talpha = S.d_talpha;
        job.tcnt = S.d_tcnt;
        job.tscan = S.d_tscan;
        job.sort_hist = S.d_hist;
        job.hist_tiles = (uint32_t)(S.hist_cap / 256);
        // radix digits: the painter's keys are (mesh << 32 | distance key), the
        // fragment keys (pixel << 32 | frame-local transparent key)
        auto bits = [](uint64_t v) {
            uint32_t b = 0;
            while (v) {
                b++;
                v >>= 1;
            }
            return b;
        };
        DgTransparentPlan& p = B.cfg.tplan;
        auto add = [](uint32_t* sh, uint32_t& np, uint32_t lo, uint32_t nbits) {
            for (uint32_t b = 0; b < nbits; b += 8) sh[np++] = lo + b;
        };
        add(p.tsort_shift, p.n_tsort, 0, 32);
        add(p.tsort_shift, p.n_tsort, 32, bits(tmesh_total - 1));
        if (p.n_tsort & 1u) p.tsort_shift[p.n_tsort++] = 56;  // even pass count: the result lands in buffer 0
        add(p.fsort_shift, p.n_fsort, 0, bits(4 * max_frame_tt - 1));
        add(p.fsort_shift, p.n_fsort, 32, bits(total_px - 1));
        if (p.n_fsort & 1u) p.fsort_shift[p.n_fsort++] = 56;
        p.blocks = (unsigned)c->nsm * 8u;
        B.launches += 3 * (p.n_tsort + p.n_fsort) + 6;
    }
    B.cfg.vertex_blocks = (unsigned)c->nsm * DG_VERTEX_BLOCKS_PER_SM;
    B.cfg.cull_blocks = (unsigned)c->nsm * S.cull_blocks_per_sm;
    B.cfg.setup_blocks = (unsigned)c->nsm * S.setup_blocks_per_sm;
    B.cfg.queue_blocks = (unsigned)c->nsm * S.queue_blocks_per_sm;
    B.total_vtx = total_vtx;
    B.total_tri = total_tri;
    return DG_OK;
}

dg_status enqueue_job(JobBuild& B, JobSlot& S, void* d_stage, cudaStream_t stream, bool timing) {
    B.job.frames = (const DgFrameDev*)d_stage;
    B.job.segs = (const DgSegDev*)((uint8_t*)d_stage + B.fbytes);
    if (!B.job.total_vtx)  // otherwise the first kernel zeroes them
        DG_CUDA(cudaMemsetAsync(S.d_counters, 0, DG_NCOUNTERS * sizeof(unsigned long long), stream));
    DG_CUDA(dg_launch_job(B.job, B.cfg, stream, timing ? S.ev : nullptr));
    return DG_OK;
}

void advance_transparent(dg_ctx* c, const JobBuild& b) {
    for (int32_t oid : b.transparent_objects) c->objects[oid].tcur ^= 1;
}

dg_status launch_frames(dg_ctx* c, JobSlot& S, Scene* const* scenes, const FrameTarget* targets, uint32_t n) {
    if (n == 0) return DG_OK;
    JobBuild B;
    dg_status e = build_job(c, S, scenes, targets, n, B);
    if (e) return e;
    // job descriptor upload through a pinned staging slot
    const size_t need = B.fbytes + B.sbytes;
    const int k = S.stage;
    S.stage = (S.stage + 1) % JobSlot::kStage;
    DG_CUDA(cudaEventSynchronize(S.stage_ev[k]));
    if (S.stage_cap[k] < need) {
        if (S.h_stage[k]) cudaFreeHost(S.h_stage[k]);
        dfree(S.d_stage[k]);
        S.h_stage[k] = nullptr;
        S.stage_cap[k] = 0;
        size_t cap = std::max<size_t>(need * 2, 64 * 1024);
        DG_CUDA(cudaMallocHost(&S.h_stage[k], cap));
        e = dalloc((uint8_t**)&S.d_stage[k], cap);
        if (e) return e;
        S.stage_cap[k] = cap;
    }
    // A small job's descriptors go to the device as a kernel parameter (k_vertex
    // writes them to the staging buffer); larger ones are copied.
    DgInlineDesc inl;
    const bool inline_desc = B.frames.size() == 1 && B.segs.size() <= DG_INLINE_SEGS && B.total_vtx > 0;
    if (inline_desc) {
        std::memset(&inl, 0, sizeof(inl));
        inl.frame = B.frames[0];
        for (size_t i = 0; i < B.segs.size(); i++) inl.segs[i] = B.segs[i];
        inl.nsegs = (uint32_t)B.segs.size();
        B.cfg.inl = &inl;
    } else {
        std::memcpy(S.h_stage[k], B.frames.data(), B.fbytes);
        std::memcpy((uint8_t*)S.h_stage[k] + B.fbytes, B.segs.data(), B.sbytes);
        DG_CUDA(cudaMemcpyAsync(S.d_stage[k], S.h_stage[k], need, cudaMemcpyHostToDevice, S.stream));
    }
    DG_CUDA(cudaEventRecord(S.stage_ev[k], S.stream));
    S.last_vtx = B.total_vtx;
    S.last_tri = B.total_tri;
    S.last_h2d = need;
    S.last_launches = B.launches;
    S.last_tile_rows = B.job.tile_rows;
    S.last_small_max_px = B.frames.empty() ? 0 : B.frames[0].small_max_px;
    e = enqueue_job(B, S, S.d_stage[k], S.stream, S.timing);
    if (e) return e;
    advance_transparent(c, B);
    if (S.timing) S.ev_valid = true;
    return DG_OK;
}

}  // namespace dgh

// Camera::new followed by the per-frame host setup of Scene::render, for callers
// that hold no dg_ctx; uses only stack storage.
dg_status dg_host_frame_setup(uint64_t width, uint64_t height, const float pos[3], const float dir[3], float ratio,
                              float near_, float far_, float fov_x_deg, float M[4][4], float planes[6][4]) {
    if (width == 0 || height == 0 || !pos || !dir) return DG_E_INVALID;
    Scene s;
    s.width = width;
    s.height = height;
    s.exponent = 2;
    dg_status e = camera_init(s.cam, h3(pos[0], pos[1], pos[2]), h3(dir[0], dir[1], dir[2]), ratio, near_, far_,
                              fov_x_deg);
    if (e) return e;
    return frame_setup(s, M, planes);
}

extern "C" {

const char* dg_status_string(dg_status s) {
    switch (s) {
        case DG_OK: return "ok";
        case DG_E_INVALID: return "invalid argument";
        case DG_E_INDEX: return "mesh index out of range";
        case DG_E_TEXTURE_RANGE: return "texel offset outside the texture map";
        case DG_E_CAMERA: return "camera or view-plane assertion failed";
        case DG_E_DEPTH_UNINIT: return "canvas depth buffer not initialized";
        case DG_E_CUDA: return "CUDA error";
        case DG_E_OOM: return "out of device memory";
        case DG_E_LIMIT: return "size or feature beyond a documented limit";
        case DG_E_TIMEOUT: return "bounded wait timed out";
        case DG_E_CANCELLED: return "request cancelled";
        default: return "unknown status";
    }
}

dg_status dg_ctx_create(int32_t device, dg_ctx** out) {
    if (!out) return DG_E_INVALID;
    *out = nullptr;
    if (device == -1) {  // host-only context: scenes and cameras work, device calls return DG_E_CUDA
        dg_ctx* h = new (std::nothrow) dg_ctx();
        if (!h) return DG_E_OOM;
        h->device = -1;
        *out = h;
        return DG_OK;
    }
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
        cudaGetLastError();
        return DG_E_CUDA;
    }
    std::unique_ptr<dg_ctx> c(new (std::nothrow) dg_ctx());
    if (!c) return DG_E_OOM;
    c->device = device;
    DG_CUDA(cudaSetDevice(device));
    DG_CUDA(cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, device));
    DG_CUDA(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
    dg_status e = slot_init(c.get(), c->main, c->own_stream);
    if (e) return e;
    TexMap white;
    const uint8_t px[3] = {255, 255, 255};  // TextureMap::default, scene/mod.rs:128-135
    e = tex_upload(px, 3, 1, 1, 3, white);
    if (e) return e;
    c->tex.push_back(white);
    *out = c.release();
    return DG_OK;
}

dg_status dg_ctx_destroy(dg_ctx* c) {
    if (!c) return DG_E_INVALID;
    if (c->device < 0) {
        delete c;
        return DG_OK;
    }
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    for (auto& t : c->tex) dfree(t.d_words);
    for (auto& o : c->objects) free_object(o);
    for (auto& v : c->canvases) free_canvas(v);
    if (c->copy_stream) cudaStreamDestroy(c->copy_stream);
    dfree(c->d_tex);
    slot_free(c->main);
    {
        OverlaySlot& O = c->overlay;
        dfree(O.d_rec); dfree(O.d_box); dfree(O.d_scan); dfree(O.d_hist); dfree(O.d_cnt); dfree(O.d_rgba);
        for (int k = 0; k < 2; k++) {
            dfree(O.d_fkey[k]);
            dfree(O.d_fval[k]);
        }
    }
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
    return DG_OK;
}

dg_status dg_ctx_synchronize(dg_ctx* c) {
    if (!c) return DG_E_INVALID;
    dg_status e = set_device(c);
    if (e) return e;
    DG_CUDA(cudaStreamSynchronize(c->main.stream));
    return slot_take_errors(c->main);
}

dg_status dg_ctx_set_stream(dg_ctx* c, void* stream) {
    if (!c) return DG_E_INVALID;
    if (c->device < 0) return DG_E_CUDA;
    DG_CUDA(cudaStreamSynchronize(c->main.stream));
    c->main.stream = stream ? (cudaStream_t)stream : c->own_stream;
    return DG_OK;
}

void* dg_ctx_stream(dg_ctx* c) { return c ? (void*)c->main.stream : nullptr; }

dg_status dg_ctx_set_timing(dg_ctx* c, int32_t enable) {
    if (!c) return DG_E_INVALID;
    c->main.timing = enable != 0;
    c->main.ev_valid = false;
    return DG_OK;
}

dg_status dg_timeline_read(dg_ctx* c, uint64_t* out, int32_t n) {
    if (!c || !out || n < 0) return DG_E_INVALID;
    dg_status e = set_device(c);
    if (e) return e;
    unsigned long long h[DG_NKERNELS * 4];
    cudaError_t ce = cudaSuccess;
    if (!dg_timeline_copy(h, c->main.stream, &ce)) return DG_E_INVALID;  // not a DRAW_TIMELINE build
    if (ce != cudaSuccess) {
        cudaGetLastError();
        return DG_E_CUDA;
    }
    for (int i = 0; i < n && i < DG_NKERNELS * 4; i++) out[i] = h[i] == ~0ull ? 0u : h[i];
    return DG_OK;
}

dg_status dg_ctx_kernel_times(dg_ctx* c, float* ms, int32_t n) {
    if (!c || !ms || n < 0) return DG_E_INVALID;
    if (c->device < 0) return DG_E_CUDA;
    if (!c->main.ev_valid) return DG_E_INVALID;
    DG_CUDA(cudaEventSynchronize(c->main.ev[DG_NKERNELS]));
    for (int i = 0; i < n && i < DG_NKERNELS; i++)
        DG_CUDA(cudaEventElapsedTime(&ms[i], c->main.ev[i], c->main.ev[i + 1]));
    return DG_OK;
}

dg_status dg_ctx_set_tuning(dg_ctx* c, const dg_tuning* t) {
    if (!c || !t) return DG_E_INVALID;
    auto bad = [](uint32_t b) { return b < 1 || b > 64; };
    if ((t->small_max_px > 4096 && t->small_max_px != DG_SMALL_MAX_PX_AUTO) || bad(t->setup_blocks_per_sm) ||
        bad(t->queue_blocks_per_sm) ||
        bad(t->cull_blocks_per_sm) || (t->tile_rows != 0 && t->tile_rows != 8 && t->tile_rows != 16 && t->tile_rows != 32) ||
        t->item_units < 1 || t->item_units > 256)
        return DG_E_INVALID;
    c->main.small_max_px = t->small_max_px;
    c->main.setup_blocks_per_sm = t->setup_blocks_per_sm;
    c->main.queue_blocks_per_sm = t->queue_blocks_per_sm;
    c->main.cull_blocks_per_sm = t->cull_blocks_per_sm;
    c->main.record_limit = t->record_limit;
    c->main.tile_rows = t->tile_rows;
    c->main.item_units = t->item_units;
    return DG_OK;
}

dg_status dg_ctx_get_tuning(dg_ctx* c, dg_tuning* t) {
    if (!c || !t) return DG_E_INVALID;
    t->small_max_px = c->main.small_max_px;
    t->setup_blocks_per_sm = c->main.setup_blocks_per_sm;
    t->queue_blocks_per_sm = c->main.queue_blocks_per_sm;
    t->cull_blocks_per_sm = c->main.cull_blocks_per_sm;
    t->record_limit = c->main.record_limit;
    t->tile_rows = c->main.tile_rows;
    t->item_units = c->main.item_units;
    return DG_OK;
}

dg_status dg_ctx_last_stats(dg_ctx* c, uint64_t* out, int32_t n) {
    if (!c || !out || n < 0) return DG_E_INVALID;
    if (c->device < 0) return DG_E_CUDA;
    JobSlot& S = c->main;
    DG_CUDA(cudaStreamSynchronize(S.stream));
    unsigned long long h[DG_NCOUNTERS];
    DG_CUDA(cudaMemcpy(h, S.d_counters, sizeof(h), cudaMemcpyDeviceToHost));
    const uint64_t v[14] = {S.last_vtx,
                            S.last_tri,
                            h[DG_CNT_QUEUE] >> DG_PACK_SHIFT,
                            h[DG_CNT_UNITS],
                            h[DG_CNT_COVERED],
                            h[DG_CNT_INPLACE],
                            S.last_h2d,
                            S.last_launches,
                            h[DG_CNT_SURV],
                            h[DG_CNT_TREC],
                            h[DG_CNT_VROW],
                            h[DG_CNT_SMALL],
                            S.last_tile_rows,
                            S.last_small_max_px};
    for (int i = 0; i < n && i < 14; i++) out[i] = v[i];
    return DG_OK;
}

dg_status dg_texmap_create(dg_ctx* c, const uint8_t* img, uint64_t len, uint64_t w, uint64_t h, uint64_t comps,
                           int32_t* out_id) {
    if (!c || !out_id || (len && !img)) return DG_E_INVALID;
    // scene/mod.rs:114-115
    if (comps == 0 || len % comps != 0 || len / comps != w * h) return DG_E_INVALID;
    if (w > 0xFFFFFFFFull || h > 0xFFFFFFFFull || comps > 0xFFFFFFFFull) return DG_E_LIMIT;
    dg_status e = set_device(c);
    if (e) return e;
    TexMap t;
    e = tex_upload(img, len, (uint32_t)w, (uint32_t)h, (uint32_t)comps, t);
    if (e) return e;
    c->tex.push_back(t);
    c->tex_dirty = true;
    *out_id = (int32_t)c->tex.size() - 2;  // user ids start at 0; [0] is the default map
    return DG_OK;
}

dg_status dg_object_create(dg_ctx* c, const float* vertices, uint64_t nv, const float* normals, uint64_t nn,
                           const float* uvs, uint64_t nuv, const dg_mesh_desc* meshes, uint64_t nmesh,
                           const dg_material* mats, uint64_t nmat, int32_t* out_id) {
    if (!c || !out_id) return DG_E_INVALID;
    if ((nv && !vertices) || (nn && !normals) || (nuv && !uvs) || (nmesh && !meshes) || (nmat && !mats))
        return DG_E_INVALID;
    if (nv >= 0xFFFFFFFFull || nn >= 0xFFFFFFFFull || nuv >= 0xFFFFFFFFull) return DG_E_LIMIT;
    dg_status e = set_device(c);
    if (e) return e;
    std::vector<DgMatDev> dm(nmat);
    for (uint64_t i = 0; i < nmat; i++) {
        for (int k = 0; k < 3; k++) {
            dm[i].ka[k] = mats[i].ka[k];
            dm[i].kd[k] = mats[i].kd[k];
            dm[i].ks[k] = mats[i].ks[k];
        }
        dm[i].alpha = mats[i].alpha;
        int32_t ids[2] = {mats[i].map_ka, mats[i].map_kd};
        uint32_t tix[2];
        for (int k = 0; k < 2; k++) {
            if (ids[k] < -1 || ids[k] + 1 >= (int64_t)c->tex.size()) return DG_E_INVALID;
            tix[k] = (uint32_t)(ids[k] + 1);
        }
        dm[i].map_ka = tix[0];
        dm[i].map_kd = tix[1];
    }
    Object o;
    std::vector<uint4> tpos, tuv, tnrm;
    std::vector<uint4> xpos, xuv, xnrm;  // transparent meshes
    o.tmesh_off.push_back(0u);
    uint64_t total = 0;
    for (uint64_t m = 0; m < nmesh; m++) {
        if (meshes[m].ntri && !meshes[m].tris) return DG_E_INVALID;
        // object.rs:46-53: textures[texture_idx] panics when out of range
        if (meshes[m].texture_idx < 0 || (uint64_t)meshes[m].texture_idx >= nmat) return DG_E_INVALID;
        total += meshes[m].ntri;
        for (uint64_t t = 0; t < meshes[m].ntri; t++) {
            const uint32_t* q = meshes[m].tris + 9 * t;
            for (int k = 0; k < 3; k++)  // mesh.rs:46-48
                if (q[k] >= nv || q[3 + k] >= nuv || q[6 + k] >= nn) return DG_E_INDEX;
        }
    }
    if (total >= (1ull << 30)) return DG_E_LIMIT;
    for (uint64_t m = 0; m < nmesh; m++) {
        const dg_mesh_desc& md = meshes[m];
        bool transparent = mats[md.texture_idx].alpha < 1.0f;
        if (transparent) {
            const uint32_t mesh = (uint32_t)(o.tmesh_off.size() - 1);
            for (uint64_t t = 0; t < md.ntri; t++) {
                const uint32_t* q = md.tris + 9 * t;
                xpos.push_back(make_uint4(q[0], q[1], q[2], (uint32_t)md.texture_idx));
                xuv.push_back(make_uint4(q[3], q[4], q[5], mesh));
                xnrm.push_back(make_uint4(q[6], q[7], q[8], 0u));
            }
            o.tmesh_off.push_back((uint32_t)xpos.size());
            continue;
        }
        for (uint64_t t = 0; t < md.ntri; t++) {
            const uint32_t* q = md.tris + 9 * t;
            tpos.push_back(make_uint4(q[0], q[1], q[2], (uint32_t)md.texture_idx));
            tuv.push_back(make_uint4(q[3], q[4], q[5], 0u));
            tnrm.push_back(make_uint4(q[6], q[7], q[8], 0u));
        }
    }
    std::vector<float4> p4(nv), n4(nn);
    std::vector<float2> u2(nuv);
    for (uint64_t i = 0; i < nv; i++) p4[i] = make_float4(vertices[3 * i], vertices[3 * i + 1], vertices[3 * i + 2], 1.0f);
    for (uint64_t i = 0; i < nn; i++) n4[i] = make_float4(normals[3 * i], normals[3 * i + 1], normals[3 * i + 2], 0.0f);
    for (uint64_t i = 0; i < nuv; i++) u2[i] = make_float2(uvs[3 * i], uvs[3 * i + 1]);
    o.nv = (uint32_t)nv;
    o.nt = (uint32_t)xpos.size();
    o.nn = (uint32_t)nn;
    o.nuv = (uint32_t)nuv;
    o.ntri_opaque = (uint32_t)tpos.size();
    o.nmats = (uint32_t)nmat;
    auto up = [&](auto** dst, const auto& src) -> dg_status {
        dg_status ee = dalloc(dst, src.size());
        if (ee) return ee;
        if (!src.empty())
            DG_CUDA(cudaMemcpy(*dst, src.data(), src.size() * sizeof(src[0]), cudaMemcpyHostToDevice));
        return DG_OK;
    };
    if ((e = up(&o.d_pos, p4)) || (e = up(&o.d_nrm, n4)) || (e = up(&o.d_uv, u2)) || (e = up(&o.d_tri_pos, tpos)) ||
        (e = up(&o.d_tri_uv, tuv)) || (e = up(&o.d_tri_nrm, tnrm)) || (e = up(&o.d_mats, dm)) ||
        (e = up(&o.d_tt[0][0], xpos)) || (e = up(&o.d_tt[0][1], xuv)) || (e = up(&o.d_tt[0][2], xnrm)) ||
        (e = dalloc(&o.d_tt[1][0], xpos.size())) || (e = dalloc(&o.d_tt[1][1], xpos.size())) ||
        (e = dalloc(&o.d_tt[1][2], xpos.size()))) {
        free_object(o);
        return e;
    }
    o.alive = true;
    c->objects.push_back(std::move(o));
    *out_id = (int32_t)c->objects.size() - 1;
    return DG_OK;
}

dg_status dg_object_destroy(dg_ctx* c, int32_t id) {
    Object* o = get_object(c, id);
    if (!o) return DG_E_INVALID;
    for (auto& s : c->scenes)
        for (int32_t x : s.objects)
            if (x == id) return DG_E_INVALID;  // still referenced by a scene
    cudaSetDevice(c->device);
    cudaDeviceSynchronize();
    free_object(*o);
    o->alive = false;
    return DG_OK;
}

dg_status dg_scene_create(dg_ctx* c, uint64_t width, uint64_t height, int32_t* out_id) {
    if (!c || !out_id || width == 0 || height == 0) return DG_E_INVALID;
    Scene s;
    s.width = width;
    s.height = height;
    HV3 pos = h3(0.0f, 0.0f, 150.0f);  // scene/mod.rs:763-769
    HV3 dir = hmul(pos, -1.0f);
    s.lights.push_back(h3(0.0f, 300.0f, 300.0f));
    s.exponent = 2;
    float ratio = (float)width / (float)height;
    dg_status e = camera_init(s.cam, pos, dir, ratio, -10.0f, -10.0f - 500.0f, 135.0f);
    if (e) return e;
    c->scenes.push_back(s);
    *out_id = (int32_t)c->scenes.size() - 1;
    return DG_OK;
}

dg_status dg_scene_add_obj(dg_ctx* c, int32_t scene, int32_t object, uint32_t* out_obj_id) {
    Scene* s = get_scene(c, scene);
    if (!s || !get_object(c, object)) return DG_E_INVALID;
    s->objects.push_back(object);
    if (out_obj_id) *out_obj_id = (uint32_t)s->objects.size() - 1;
    return DG_OK;
}

dg_status dg_scene_set_camera(dg_ctx* c, int32_t scene, const float pos[3], const float dir[3], float ratio,
                              float near_, float far_, float fov_x_deg) {
    Scene* s = get_scene(c, scene);
    if (!s || !pos || !dir) return DG_E_INVALID;
    return camera_init(s->cam, h3(pos[0], pos[1], pos[2]), h3(dir[0], dir[1], dir[2]), ratio, near_, far_, fov_x_deg);
}

dg_status dg_scene_camera_op(dg_ctx* c, int32_t scene, int32_t op, const float* a) {
    Scene* s = get_scene(c, scene);
    if (!s || !a) return DG_E_INVALID;
    return camera_op(*s, op, a);
}

dg_status dg_scene_get_camera(dg_ctx* c, int32_t scene, float pos[3], float dir[3]) {
    Scene* s = get_scene(c, scene);
    if (!s || !pos || !dir) return DG_E_INVALID;
    pos[0] = s->cam.position.x; pos[1] = s->cam.position.y; pos[2] = s->cam.position.z;
    dir[0] = s->cam.direction.x; dir[1] = s->cam.direction.y; dir[2] = s->cam.direction.z;
    return DG_OK;
}

dg_status dg_scene_set_lights(dg_ctx* c, int32_t scene, const float* pos, uint32_t n) {
    Scene* s = get_scene(c, scene);
    if (!s || !pos || n == 0 || n > DG_MAX_LIGHTS) return DG_E_INVALID;
    s->lights.clear();
    for (uint32_t i = 0; i < n; i++) s->lights.push_back(h3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
    return DG_OK;
}

dg_status dg_scene_set_interpolation(dg_ctx* c, int32_t scene, int32_t mode) {
    Scene* s = get_scene(c, scene);
    if (!s || (mode != DG_INTERP_AFFINE && mode != DG_INTERP_PERSPECTIVE)) return DG_E_INVALID;
    s->interpolation = mode;
    return DG_OK;
}

dg_status dg_texmap_set_filter(dg_ctx* c, int32_t texmap, int32_t filter) {
    if (!c || texmap < 0 || (size_t)texmap + 1 >= c->tex.size() ||
        (filter != DG_FILTER_NEAREST && filter != DG_FILTER_BILINEAR))
        return DG_E_INVALID;
    if (c->tex[(size_t)texmap + 1].filter != (uint32_t)filter) {
        c->tex[(size_t)texmap + 1].filter = (uint32_t)filter;
        c->tex_dirty = true;
    }
    return DG_OK;
}

dg_status dg_scene_set_exponent(dg_ctx* c, int32_t scene, int32_t exponent) {
    Scene* s = get_scene(c, scene);
    if (!s) return DG_E_INVALID;
    s->exponent = exponent;
    return DG_OK;
}

dg_status dg_scene_frame_setup(dg_ctx* c, int32_t scene, float M[16], float planes[24]) {
    Scene* s = get_scene(c, scene);
    if (!s || !M || !planes) return DG_E_INVALID;
    float m[4][4], p[6][4];
    dg_status e = frame_setup(*s, m, p);
    if (e) return e;
    std::memcpy(M, m, sizeof(m));
    std::memcpy(planes, p, sizeof(p));
    return DG_OK;
}

dg_status dg_object_transparent_tris(dg_ctx* c, int32_t object, uint32_t mesh, uint32_t* out, uint64_t cap,
                                     uint64_t* out_ntri) {
    Object* o = get_object(c, object);
    if (!o || (size_t)mesh + 1 >= o->tmesh_off.size()) return DG_E_INVALID;
    const uint32_t b = o->tmesh_off[mesh], n = o->tmesh_off[mesh + 1] - b;
    if (out_ntri) *out_ntri = n;
    if (!out || n == 0) return DG_OK;
    if (cap < 9ull * n) return DG_E_INVALID;
    dg_status e = set_device(c);
    if (e) return e;
    DG_CUDA(cudaStreamSynchronize(c->main.stream));
    std::vector<uint4> a[3];
    for (int k = 0; k < 3; k++) {
        a[k].resize(n);
        DG_CUDA(cudaMemcpy(a[k].data(), o->d_tt[o->tcur][k] + b, n * sizeof(uint4), cudaMemcpyDeviceToHost));
    }
    for (uint32_t t = 0; t < n; t++) {  // (position, uv, normal) index triples, as the mesh was given
        const uint4 p = a[0][t], u = a[1][t], q = a[2][t];
        const uint32_t row[9] = {p.x, p.y, p.z, u.x, u.y, u.z, q.x, q.y, q.z};
        std::memcpy(out + 9ull * t, row, sizeof(row));
    }
    return DG_OK;
}

dg_status dg_canvas_create(dg_ctx* c, uint64_t width, uint64_t height, int32_t* out_id) {
    if (!c || !out_id || width == 0 || height == 0) return DG_E_INVALID;
    if (width > 65535 || height > 65535) return DG_E_LIMIT;
    dg_status e = set_device(c);
    if (e) return e;
    Canvas v;
    uint64_t n = width * height;
    const uint64_t nc = dg_cell_count(width, height);
    if ((e = dalloc(&v.d_colour, n)) || (e = dalloc(&v.d_depth, n)) || (e = dalloc(&v.d_vis, n)) ||
        (e = dalloc(&v.d_cells, nc))) {
        dfree(v.d_colour); dfree(v.d_depth); dfree(v.d_vis); dfree(v.d_cells);
        return e;
    }
    v.w = width;
    v.h = height;
    DG_CUDA(cudaMemsetAsync(v.d_cells, 0, nc * sizeof(uint32_t), c->main.stream));
    // Canvas::new: black frame (canvas.rs:368), no depth buffer yet
    DG_CUDA(dg_launch_fill(v.d_colour, v.d_depth, n, 0xFF000000u, 0.0f, 1, 0, c->main.stream));
    DG_CUDA(dg_launch_vis_reset(v.d_vis, n, c->main.stream));
    v.alive = true;
    c->canvases.push_back(v);
    *out_id = (int32_t)c->canvases.size() - 1;
    return DG_OK;
}

dg_status dg_canvas_destroy(dg_ctx* c, int32_t id) {
    Canvas* v = get_canvas(c, id);
    if (!v) return DG_E_INVALID;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->main.stream);
    free_canvas(*v);
    v->alive = false;
    return DG_OK;
}

dg_status dg_canvas_init_depth(dg_ctx* c, int32_t id, float depth) {
    Canvas* v = get_canvas(c, id);
    if (!v) return DG_E_INVALID;
    dg_status e = set_device(c);
    if (e) return e;
    v->depth_max = depth;
    v->depth_init = true;
    DG_CUDA(dg_launch_fill(v->d_colour, v->d_depth, v->w * v->h, 0u, depth, 0, 1, c->main.stream));
    return DG_OK;
}

dg_status dg_canvas_apply_offset(dg_ctx* c, int32_t id, int32_t x, int32_t y) {
    Canvas* v = get_canvas(c, id);
    if (!v) return DG_E_INVALID;
    v->off_x = (float)x;
    v->off_y = (float)y;
    return DG_OK;
}

dg_status dg_canvas_resize(dg_ctx* c, int32_t id, uint64_t width, uint64_t height) {
    Canvas* v = get_canvas(c, id);
    if (!v || width == 0 || height == 0) return DG_E_INVALID;
    if (width > 65535 || height > 65535) return DG_E_LIMIT;
    dg_status e = set_device(c);
    if (e) return e;
    cudaStream_t st = c->main.stream;
    uint64_t n_old = v->w * v->h, n = width * height;
    // Vec::resize keeps the first min(old, new) pixels and pads with black (canvas.rs:390)
    uint32_t* col = nullptr;
    float* dep = nullptr;
    uint64_t* vis = nullptr;
    uint32_t* cells = nullptr;
    const uint64_t nc = dg_cell_count(width, height);
    if ((e = dalloc(&col, n)) || (e = dalloc(&dep, n)) || (e = dalloc(&vis, n)) || (e = dalloc(&cells, nc))) {
        dfree(col); dfree(dep); dfree(vis); dfree(cells);
        return e;
    }
    DG_CUDA(cudaMemsetAsync(cells, 0, nc * sizeof(uint32_t), st));
    DG_CUDA(dg_launch_fill(col, dep, n, 0xFF000000u, 0.0f, 1, 0, st));
    DG_CUDA(cudaMemcpyAsync(col, v->d_colour, std::min(n, n_old) * 4, cudaMemcpyDeviceToDevice, st));
    DG_CUDA(dg_launch_vis_reset(vis, n, st));
    DG_CUDA(cudaStreamSynchronize(st));
    dfree(v->d_colour); dfree(v->d_depth); dfree(v->d_vis); dfree(v->d_cells);
    v->d_colour = col;
    v->d_depth = dep;
    v->d_vis = vis;
    v->d_cells = cells;
    v->w = width;
    v->h = height;
    // init_depth(depth_max) (canvas.rs:392)
    v->depth_init = true;
    DG_CUDA(dg_launch_fill(v->d_colour, v->d_depth, n, 0u, v->depth_max, 0, 1, st));
    return DG_OK;
}

dg_status dg_canvas_clear(dg_ctx* c, int32_t id) {
    Canvas* v = get_canvas(c, id);
    if (!v) return DG_E_INVALID;
    dg_status e = set_device(c);
    if (e) return e;
    DG_CUDA(dg_launch_fill(v->d_colour, v->d_depth, v->w * v->h, 0xFF9BBAFFu, v->depth_max, 1, v->depth_init ? 1 : 0,
                           c->main.stream));
    return DG_OK;
}

dg_status dg_canvas_read(dg_ctx* c, int32_t id, uint8_t* bgra, float* depth) {
    Canvas* v = get_canvas(c, id);
    if (!v) return DG_E_INVALID;
    if (depth && !v->depth_init) return DG_E_DEPTH_UNINIT;
    dg_status e = set_device(c);
    if (e) return e;
    uint64_t n = v->w * v->h;
    cudaStream_t st = c->main.stream;
    if (bgra) DG_CUDA(cudaMemcpyAsync(bgra, v->d_colour, n * 4, cudaMemcpyDeviceToHost, st));
    if (depth) DG_CUDA(cudaMemcpyAsync(depth, v->d_depth, n * 4, cudaMemcpyDeviceToHost, st));
    DG_CUDA(cudaStreamSynchronize(st));
    return slot_take_errors(c->main);
}

dg_status dg_canvas_read_async(dg_ctx* c, int32_t id, uint8_t* bgra, float* depth) {
    Canvas* v = get_canvas(c, id);
    if (!v) return DG_E_INVALID;
    if (depth && !v->depth_init) return DG_E_DEPTH_UNINIT;
    dg_status e = set_device(c);
    if (e) return e;
    if (!c->copy_stream) DG_CUDA(cudaStreamCreateWithFlags(&c->copy_stream, cudaStreamNonBlocking));
    if (!v->ev_rendered) DG_CUDA(cudaEventCreateWithFlags(&v->ev_rendered, cudaEventDisableTiming));
    if (!v->ev_read) DG_CUDA(cudaEventCreateWithFlags(&v->ev_read, cudaEventDisableTiming));
    if (!v->h_err && cudaMallocHost((void**)&v->h_err, sizeof(uint32_t)) != cudaSuccess) return DG_E_OOM;
    const uint64_t n = v->w * v->h;
    DG_CUDA(cudaEventRecord(v->ev_rendered, c->main.stream));
    DG_CUDA(cudaStreamWaitEvent(c->copy_stream, v->ev_rendered, 0));
    if (bgra) DG_CUDA(cudaMemcpyAsync(bgra, v->d_colour, n * 4, cudaMemcpyDeviceToHost, c->copy_stream));
    if (depth) DG_CUDA(cudaMemcpyAsync(depth, v->d_depth, n * 4, cudaMemcpyDeviceToHost, c->copy_stream));
    // the error word of the frames before the copy, read with it (not cleared:
    // later frames may be running, and the next synchronous call reports it again)
    DG_CUDA(cudaMemcpyAsync(v->h_err, c->main.d_err, sizeof(uint32_t), cudaMemcpyDeviceToHost, c->copy_stream));
    DG_CUDA(cudaEventRecord(v->ev_read, c->copy_stream));
    v->read_pending = true;
    return DG_OK;
}

dg_status dg_canvas_read_wait(dg_ctx* c, int32_t id) {
    if (!c || id < 0 || (size_t)id >= c->canvases.size() || !c->canvases[id].alive) return DG_E_INVALID;
    Canvas* v = &c->canvases[id];
    dg_status e = set_device(c);
    if (e) return e;
    if (!v->ev_read) return DG_OK;  // never read asynchronously
    DG_CUDA(cudaEventSynchronize(v->ev_read));  // waits for this copy only, not for later ones
    const uint32_t err = v->h_err ? *v->h_err : 0u;
    for (int b = 1; b < 32; b++)
        if (err & (1u << b)) return (dg_status)b;
    return DG_OK;
}

dg_status dg_canvas_write(dg_ctx* c, int32_t id, const uint8_t* bgra, const float* depth) {
    Canvas* v = get_canvas(c, id);
    if (!v) return DG_E_INVALID;
    if (depth && !v->depth_init) return DG_E_DEPTH_UNINIT;
    dg_status e = set_device(c);
    if (e) return e;
    uint64_t n = v->w * v->h;
    cudaStream_t st = c->main.stream;
    if (bgra) DG_CUDA(cudaMemcpyAsync(v->d_colour, bgra, n * 4, cudaMemcpyHostToDevice, st));
    if (depth) DG_CUDA(cudaMemcpyAsync(v->d_depth, depth, n * 4, cudaMemcpyHostToDevice, st));
    DG_CUDA(cudaStreamSynchronize(st));
    return DG_OK;
}

dg_status dg_canvas_device_ptrs(dg_ctx* c, int32_t id, void** bgra, void** depth) {
    Canvas* v = get_canvas(c, id);
    if (!v) return DG_E_INVALID;
    if (bgra) *bgra = v->d_colour;
    if (depth) *depth = v->d_depth;
    return DG_OK;
}

namespace {

// Rust `as usize` from f32 (saturating, NaN -> 0), on the host.
uint64_t h_as_usize(float f) {
    if (!(f > 0.0f)) return 0ull;
    if (f >= 18446744073709551616.0f) return ~0ull;
    return (uint64_t)f;
}

// Rectangle (canvas.rs:293-351) in usize arithmetic.
struct HRect {
    uint64_t x, y, w, h;
    static HRect from_coords(uint64_t x0, uint64_t y0, uint64_t x1, uint64_t y1) {
        const uint64_t xa = std::min(x0, x1), ya = std::min(y0, y1), xb = std::max(x0, x1), yb = std::max(y0, y1);
        return HRect{xa, ya, xb - xa, yb - ya};
    }
    static HRect clip(const HRect& a, const HRect& b) {
        uint64_t x0 = std::max(a.x, b.x), y0 = std::max(a.y, b.y);
        uint64_t x1 = std::min(a.x + a.w, b.x + b.w), y1 = std::min(a.y + a.h, b.y + b.h);
        if (x0 > x1) x0 = x1 = 0;
        if (y0 > y1) y0 = y1 = 0;
        return from_coords(x0, y0, x1, y1);
    }
};

// The edge set of dg_device.cuh make_edges, on the host (the same f32
// operations; this file is compiled without contraction), as the 16 words of
// a triangle record: A[3], B[3], C[3], D[3], den[3], tie bits.
void host_edges(float ax, float ay, float bx, float by, float cx, float cy, float w[16]) {
    const float px[3] = {bx, cx, ax}, py[3] = {by, cy, ay};
    const float qx[3] = {cx, ax, bx}, qy[3] = {cy, ay, by};
    const float vx[3] = {ax, bx, cx}, vy[3] = {ay, by, cy};
    float A[3], B[3], C[3], D[3], den[3];
    uint32_t tie = 0;
    for (int k = 0; k < 3; k++) {
        A[k] = py[k] - qy[k];
        B[k] = qx[k] - px[k];
        C[k] = px[k] * qy[k];
        D[k] = qx[k] * py[k];
    }
    auto eval = [&](int k, float x, float y) { return ((A[k] * x + B[k] * y) + C[k]) - D[k]; };
    for (int k = 0; k < 3; k++) {
        den[k] = eval(k, vx[k], vy[k]);
        if (den[k] * eval(k, -1.0f, -1.0f) > 0.0f) tie |= 1u << k;
    }
    bool fast = true;
    for (int k = 0; k < 3; k++) {
        if (std::signbit(den[k])) {
            A[k] = -A[k];
            B[k] = -B[k];
            C[k] = -C[k];
            D[k] = -D[k];
            den[k] = -den[k];
        }
        fast = fast && den[k] > 0.0f && den[k] < INFINITY;
    }
    if (fast) tie |= DG_EDGE_FAST;
    const float words[16] = {A[0], A[1], A[2], B[0], B[1], B[2], C[0], C[1], C[2], D[0], D[1], D[2],
                             den[0], den[1], den[2], 0.0f};
    std::memcpy(w, words, sizeof(words));
    std::memcpy(w + 15, &tie, 4);
}

}  // namespace

dg_status dg_canvas_draw_triangles_2d(dg_ctx* c, int32_t canvas, const float* verts, uint32_t n, int32_t texmap,
                                      const uint64_t* clips) {
    Canvas* cv = get_canvas(c, canvas);
    if (!cv || (n && !verts)) return DG_E_INVALID;
    if (!cv->depth_init) return DG_E_DEPTH_UNINIT;
    if (texmap < -1 || texmap + 1 >= (int64_t)c->tex.size()) return DG_E_INVALID;
    if (n == 0) return DG_OK;
    dg_status e = set_device(c);
    if (e) return e;
    e = sync_tex_table(c, c->main.stream);
    if (e) return e;
    // host setup (canvas.rs:449-535): snapped centres, bounding box clipped to the
    // screen and the clipping rectangle, edges, attributes
    std::vector<DgTriRec> rec(n);
    std::vector<uint4> box(n);
    std::vector<unsigned long long> scan(n + 1);
    const HRect screen = HRect::from_coords(0, 0, cv->w - 1, cv->h - 1);
    unsigned long long total = 0;
    for (uint32_t t = 0; t < n; t++) {
        const float* v = verts + 24ull * t;
        float cx[3], cy[3], words[28];
        for (int k = 0; k < 3; k++) {  // pos_map_center, canvas.rs:896-904
            cx[k] = std::floor(v[8 * k] + 0.5f);
            cy[k] = std::floor(v[8 * k + 1] + 0.5f);
        }
        auto mn = [](float a, float b, float d) {  // NaN-skipping strict-< minimum
            float r = INFINITY;
            for (float x : {a, b, d})
                if (x < r) r = x;
            return r;
        };
        auto mx = [](float a, float b, float d) {
            float r = -INFINITY;
            for (float x : {a, b, d})
                if (x > r) r = x;
            return r;
        };
        const HRect drawable = HRect::clip(
            HRect::from_coords(h_as_usize(mn(cx[0], cx[1], cx[2])), h_as_usize(mn(cy[0], cy[1], cy[2])),
                               h_as_usize(mx(cx[0], cx[1], cx[2])), h_as_usize(mx(cy[0], cy[1], cy[2]))),
            screen);
        const HRect cr = clips ? HRect::from_coords(clips[4ull * t], clips[4ull * t + 1], clips[4ull * t + 2],
                                                    clips[4ull * t + 3])
                               : screen;
        const HRect valid = HRect::clip(cr, drawable);
        if (valid.x + valid.w >= cv->w || valid.y + valid.h >= cv->h) return DG_E_INVALID;  // outside the canvas
        host_edges(cx[0], cy[0], cx[1], cy[1], cx[2], cy[2], words);
        uint32_t col[3];
        for (int k = 0; k < 3; k++) {  // Color::Custom([r, g, b]).as_pixel(): b, g, r bytes
            const float* p = v + 8 * k;
            if (!(p[4] >= 0.0f && p[4] <= 255.0f && p[5] >= 0.0f && p[5] <= 255.0f && p[6] >= 0.0f && p[6] <= 255.0f))
                return DG_E_INVALID;
            col[k] = (uint32_t)(uint8_t)p[6] | ((uint32_t)(uint8_t)p[5] << 8) | ((uint32_t)(uint8_t)p[4] << 16);
        }
        const float w4[4] = {v[2], v[10], v[18], v[7]}, w5[4] = {v[3], v[11], v[19], v[15]};
        std::memcpy(words + 16, w4, 16);
        std::memcpy(words + 20, w5, 16);
        std::memcpy(words + 24, col, 12);
        std::memcpy(words + 27, &v[23], 4);
        std::memset(&rec[t], 0, sizeof(DgTriRec));
        std::memcpy(&rec[t], words, sizeof(words));
        const uint64_t bw = valid.w + 1, bh = valid.h + 1;
        box[t] = make_uint4((uint32_t)valid.x, (uint32_t)valid.y, (uint32_t)bw, 0u);
        scan[t] = total;
        total += bw * bh;
    }
    scan[n] = total;
    if (total >= 0x7FFFFFFFull) return DG_E_LIMIT;
    JobSlot& S = c->main;
    OverlaySlot& O = c->overlay;
    auto need = [&](auto** p, size_t* cap, size_t k) -> dg_status { return grow(S, p, cap, std::max<size_t>(k, 1)); };
    if ((e = need(&O.d_rec, &O.rec_cap, n)) || (e = need(&O.d_box, &O.box_cap, n)) ||
        (e = need(&O.d_scan, &O.scan_cap, n + 1)) || (e = need(&O.d_fkey[0], &O.frag_cap[0], total)) ||
        (e = need(&O.d_fkey[1], &O.frag_cap[1], total)) || (e = need(&O.d_fval[0], &O.frag_cap[2], total)) ||
        (e = need(&O.d_fval[1], &O.frag_cap[3], total)) ||
        (e = need(&O.d_hist, &O.hist_cap, 256 * ((total + DG_SORT_TILE - 1) / DG_SORT_TILE))) ||
        (e = need(&O.d_cnt, &O.cnt_cap, 1)))
        return e;
    DG_CUDA(cudaStreamSynchronize(S.stream));  // the scratch may still be read by the previous batch
    DG_CUDA(cudaMemcpyAsync(O.d_rec, rec.data(), n * sizeof(DgTriRec), cudaMemcpyHostToDevice, S.stream));
    DG_CUDA(cudaMemcpyAsync(O.d_box, box.data(), n * sizeof(uint4), cudaMemcpyHostToDevice, S.stream));
    DG_CUDA(cudaMemcpyAsync(O.d_scan, scan.data(), (n + 1) * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                            S.stream));
    DG_CUDA(cudaMemsetAsync(O.d_cnt, 0, sizeof(unsigned long long), S.stream));
    DgOverlayJob j;
    std::memset(&j, 0, sizeof(j));
    j.rec = O.d_rec;
    j.box = O.d_box;
    j.scan = O.d_scan;
    j.n = n;
    j.width = (uint32_t)cv->w;
    j.height = (uint32_t)cv->h;
    j.colour = cv->d_colour;
    j.depth = cv->d_depth;
    const TexMap& tm = c->tex[(size_t)(texmap + 1)];
    j.tex.words = tm.d_words;
    j.tex.len = tm.len;
    j.tex.width = tm.w;
    j.tex.height = tm.h;
    j.tex.comps = tm.comps;
    j.tex.fw = (float)tm.w;
    j.tex.fh = (float)tm.h;
    j.tex.small = dg_tex_small(tm.len, tm.w, tm.h);
    for (int k = 0; k < 2; k++) {
        j.fkey[k] = O.d_fkey[k];
        j.fval[k] = O.d_fval[k];
    }
    j.fcap = (uint32_t)total;
    j.hist = O.d_hist;
    j.cnt = O.d_cnt;
    j.err = S.d_err;
    auto bits = [](uint64_t v) {
        uint32_t b = 0;
        while (v) {
            b++;
            v >>= 1;
        }
        return b;
    };
    for (uint32_t b = 0; b < bits(n - 1); b += 8) j.sort_shift[j.n_sort++] = b;
    for (uint32_t b = 0; b < bits(cv->w * cv->h - 1); b += 8) j.sort_shift[j.n_sort++] = 32 + b;
    if (j.n_sort & 1u) j.sort_shift[j.n_sort++] = 56;  // even pass count: the result lands in buffer 0
    DG_CUDA(dg_launch_overlay(j, (unsigned)c->nsm * 8u, S.stream));
    return DG_OK;
}

dg_status dg_canvas_read_rgba(dg_ctx* c, int32_t id, uint8_t* rgba) {
    Canvas* cv = get_canvas(c, id);
    if (!cv || !rgba) return DG_E_INVALID;
    dg_status e = set_device(c);
    if (e) return e;
    const uint64_t n = cv->w * cv->h;
    JobSlot& S = c->main;
    e = grow(S, &c->overlay.d_rgba, &c->overlay.rgba_cap, std::max<uint64_t>(n, 1));
    if (e) return e;
    DG_CUDA(dg_launch_bgra_to_rgba(cv->d_colour, c->overlay.d_rgba, n, S.stream));
    DG_CUDA(cudaMemcpyAsync(rgba, c->overlay.d_rgba, n * 4, cudaMemcpyDeviceToHost, S.stream));
    DG_CUDA(cudaStreamSynchronize(S.stream));
    return slot_take_errors(S);
}

dg_status dg_canvas_size(dg_ctx* c, int32_t id, uint64_t* w, uint64_t* h) {
    Canvas* v = get_canvas(c, id);
    if (!v) return DG_E_INVALID;
    if (w) *w = v->w;
    if (h) *h = v->h;
    return DG_OK;
}

dg_status dg_scene_render(dg_ctx* c, int32_t scene, int32_t canvas) {
    if (!c) return DG_E_INVALID;
    return render_job(c, &scene, &canvas, 1);
}

dg_status dg_render_batch(dg_ctx* c, const int32_t* scenes, const int32_t* canvases, uint32_t n) {
    if (!c || (n && (!scenes || !canvases))) return DG_E_INVALID;
    return render_job(c, scenes, canvases, n);
}

}  // extern "C"
