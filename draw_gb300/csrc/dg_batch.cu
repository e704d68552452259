// dg_batch.cu -- the graph-replayed batched form of the draw call and the
// launch-shape autotuner.
//
// dg_batch: n (scene, canvas) frames rendered as one job whose launch sequence
// (descriptor upload, counter reset, the five pipeline kernels with their
// programmatic dependencies) is captured once in a CUDA graph and replayed by
// every dg_batch_render. Per-frame state that may change between replays
// (cameras, lights, exponent, clear depth, canvas offset) lives in the uploaded
// descriptors, which the host rewrites in a pinned staging buffer before each
// replay; two graphs with two staging buffers alternate, so the host prepares
// one replay while the previous one runs. Anything that changes the job's
// shape (the scenes' object lists, a canvas resize, new texture maps, the
// context's tuning) is detected from a signature and triggers a new capture.
//
// dg_autotune: coordinate descent over the dg_tuning knobs, each candidate
// timed with CUDA events on the context stream over the caller's frames.
// Knobs change only grid sizes and how work is split between passes, never the
// rendered result.
#include <algorithm>
#include <cstring>
#include <vector>

#include "dg_host.h"

using namespace dgh;

namespace {

#define DG_CUDA(x)                                                         \
    do {                                                                   \
        cudaError_t _e = (x);                                              \
        if (_e != cudaSuccess) {                                           \
            cudaGetLastError();                                            \
            return _e == cudaErrorMemoryAllocation ? DG_E_OOM : DG_E_CUDA; \
        }                                                                  \
    } while (0)

}  // namespace

struct dg_batch {
    dg_ctx* ctx = nullptr;
    std::vector<int32_t> scenes, canvases;
    JobSlot slot;                  // the batch's own scratch (its stream is the capture stream)
    cudaStream_t cap = nullptr;    // capture stream
    std::vector<uint64_t> sig;     // job shape the graphs were captured for
    cudaGraphExec_t exec[2] = {};
    void* h_stage[2] = {};
    void* d_stage[2] = {};
    size_t stage_cap = 0;
    cudaEvent_t done[2] = {};
    int next = 0;
    uint64_t captures = 0, replays = 0, launches = 0, h2d = 0;
};

namespace {

void drop_graphs(dg_batch* b) {
    for (int k = 0; k < 2; k++) {
        if (b->exec[k]) cudaGraphExecDestroy(b->exec[k]);
        b->exec[k] = nullptr;
    }
    b->sig.clear();
}

// Everything the captured kernels and their launch parameters depend on.
void signature(const dg_batch* b, const std::vector<Scene*>& sc, const std::vector<FrameTarget>& tg,
               std::vector<uint64_t>& sig) {
    const dg_ctx* c = b->ctx;
    sig.clear();
    sig.push_back(sc.size());
    for (size_t i = 0; i < sc.size(); i++) {
        sig.push_back((uint64_t)(uintptr_t)tg[i].colour);
        sig.push_back((uint64_t)(uintptr_t)tg[i].depth);
        sig.push_back((uint64_t)(uintptr_t)tg[i].vis);
        sig.push_back(tg[i].w);
        sig.push_back(tg[i].h);
        sig.push_back(sc[i]->lights.size());
        sig.push_back((uint64_t)(uint32_t)sc[i]->interpolation);
        sig.push_back(sc[i]->objects.size());
        for (int32_t oid : sc[i]->objects) {
            sig.push_back((uint64_t)(uint32_t)oid);
            if (oid >= 0 && (size_t)oid < c->objects.size()) {
                const Object& o = c->objects[oid];
                sig.push_back((uint64_t)(uintptr_t)o.d_pos);
                sig.push_back(o.ntri_opaque);
                sig.push_back(o.nv);
            }
        }
    }
    sig.push_back((uint64_t)(uintptr_t)c->d_tex);
    sig.push_back(c->tex.size());
    sig.push_back(c->tex_dirty ? 1u : 0u);
    const JobSlot& m = c->main;
    sig.push_back(m.small_max_px);
    sig.push_back(m.setup_blocks_per_sm);
    sig.push_back(m.queue_blocks_per_sm);
    sig.push_back(m.cull_blocks_per_sm);
    sig.push_back(m.tile_rows);
    sig.push_back(m.record_limit);
    sig.push_back(m.item_units);
}

dg_status capture(dg_batch* b, const std::vector<Scene*>& sc, const std::vector<FrameTarget>& tg, JobBuild& B) {
    dg_ctx* c = b->ctx;
    DG_CUDA(cudaStreamSynchronize(c->main.stream));  // earlier replays use the scratch and staging
    drop_graphs(b);
    JobSlot& S = b->slot;
    S.small_max_px = c->main.small_max_px;
    S.setup_blocks_per_sm = c->main.setup_blocks_per_sm;
    S.queue_blocks_per_sm = c->main.queue_blocks_per_sm;
    S.cull_blocks_per_sm = c->main.cull_blocks_per_sm;
    S.tile_rows = c->main.tile_rows;
    S.record_limit = c->main.record_limit;
    S.item_units = c->main.item_units;
    dg_status e = build_job(c, S, sc.data(), tg.data(), (uint32_t)sc.size(), B);
    if (e) return e;
    B.job.err = c->main.d_err;  // kernel errors surface at the context's next synchronizing call
    DG_CUDA(cudaStreamSynchronize(S.stream));  // scratch initialization issued by build_job
    const size_t need = B.fbytes + B.sbytes;
    if (b->stage_cap < need) {
        for (int k = 0; k < 2; k++) {
            if (b->h_stage[k]) cudaFreeHost(b->h_stage[k]);
            if (b->d_stage[k]) cudaFree(b->d_stage[k]);
            b->h_stage[k] = b->d_stage[k] = nullptr;
        }
        b->stage_cap = 0;
        for (int k = 0; k < 2; k++) {
            DG_CUDA(cudaMallocHost(&b->h_stage[k], need));
            DG_CUDA(cudaMalloc(&b->d_stage[k], need));
        }
        b->stage_cap = need;
    }
    for (int k = 0; k < 2; k++) {
        DG_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
        cudaError_t ce = cudaMemcpyAsync(b->d_stage[k], b->h_stage[k], need, cudaMemcpyHostToDevice, b->cap);
        dg_status le = ce == cudaSuccess ? enqueue_job(B, S, b->d_stage[k], b->cap, false) : DG_E_CUDA;
        cudaGraph_t g = nullptr;
        cudaError_t ee = cudaStreamEndCapture(b->cap, &g);
        if (le != DG_OK || ee != cudaSuccess || !g) {
            if (g) cudaGraphDestroy(g);
            cudaGetLastError();
            drop_graphs(b);
            return le != DG_OK ? le : DG_E_CUDA;
        }
        cudaError_t ie = cudaGraphInstantiate(&b->exec[k], g, 0);
        cudaGraphDestroy(g);
        if (ie != cudaSuccess) {
            cudaGetLastError();
            b->exec[k] = nullptr;
            drop_graphs(b);
            return DG_E_CUDA;
        }
    }
    b->captures++;
    b->launches = B.launches;
    b->h2d = need;
    return DG_OK;
}

// Median-free timing of one tuning: one warm-up render, then `reps` renders
// between two events on the context stream.
dg_status time_tuning(dg_ctx* c, const int32_t* scenes, const int32_t* canvases, uint32_t n, uint32_t reps,
                      cudaEvent_t e0, cudaEvent_t e1, float* ms) {
    dg_status e = render_job(c, scenes, canvases, n);
    if (e) return e;
    DG_CUDA(cudaEventRecord(e0, c->main.stream));
    for (uint32_t r = 0; r < reps; r++) {
        e = render_job(c, scenes, canvases, n);
        if (e) return e;
    }
    DG_CUDA(cudaEventRecord(e1, c->main.stream));
    DG_CUDA(cudaEventSynchronize(e1));
    e = slot_take_errors(c->main);
    if (e) return e;
    float t = 0.0f;
    DG_CUDA(cudaEventElapsedTime(&t, e0, e1));
    *ms = t / (float)reps;
    return DG_OK;
}

// One job renders each canvas at most once (a canvas holds one frame's visibility keys).
bool canvases_distinct(const int32_t* canvases, uint32_t n) {
    std::vector<int32_t> v(canvases, canvases + n);
    std::sort(v.begin(), v.end());
    return std::adjacent_find(v.begin(), v.end()) == v.end();
}

}  // namespace

extern "C" {

dg_status dg_batch_create(dg_ctx* c, const int32_t* scenes, const int32_t* canvases, uint32_t n, dg_batch** out) {
    if (!c || !out || n == 0 || !scenes || !canvases) return DG_E_INVALID;
    *out = nullptr;
    if (!canvases_distinct(canvases, n)) return DG_E_INVALID;
    if (c->device < 0) return DG_E_CUDA;
    std::vector<Scene*> sc;
    std::vector<FrameTarget> tg;
    dg_status e = resolve_frames(c, scenes, canvases, n, sc, tg);
    if (e) return e;
    e = set_device(c);
    if (e) return e;
    dg_batch* b = new (std::nothrow) dg_batch();
    if (!b) return DG_E_OOM;
    b->ctx = c;
    b->scenes.assign(scenes, scenes + n);
    b->canvases.assign(canvases, canvases + n);
    cudaError_t ce = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&b->done[0], cudaEventDisableTiming);
    if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&b->done[1], cudaEventDisableTiming);
    e = ce == cudaSuccess ? slot_init(c, b->slot, b->cap) : DG_E_CUDA;
    if (e) {
        cudaGetLastError();
        dg_batch_destroy(b);
        return e;
    }
    *out = b;
    return DG_OK;
}

dg_status dg_batch_render(dg_batch* b) {
    if (!b) return DG_E_INVALID;
    dg_ctx* c = b->ctx;
    const uint32_t n = (uint32_t)b->scenes.size();
    std::vector<Scene*> sc;
    std::vector<FrameTarget> tg;
    dg_status e = resolve_frames(c, b->scenes.data(), b->canvases.data(), n, sc, tg);
    if (e) return e;
    e = set_device(c);
    if (e) return e;
    e = sync_tex_table(c, c->main.stream);
    if (e) return e;
    std::vector<uint64_t> sig;
    signature(b, sc, tg, sig);
    JobBuild B;
    if (sig != b->sig || !b->exec[0]) {
        e = capture(b, sc, tg, B);
        if (e) return e;
        b->sig = sig;
    } else {
        e = build_job(c, b->slot, sc.data(), tg.data(), n, B);  // frame descriptors only: sizes are unchanged
        if (e) return e;
    }
    const int k = b->next;
    b->next ^= 1;
    DG_CUDA(cudaEventSynchronize(b->done[k]));  // the previous replay of graph k has read its staging
    std::memcpy(b->h_stage[k], B.frames.data(), B.fbytes);
    std::memcpy((uint8_t*)b->h_stage[k] + B.fbytes, B.segs.data(), B.sbytes);
    DG_CUDA(cudaGraphLaunch(b->exec[k], c->main.stream));
    DG_CUDA(cudaEventRecord(b->done[k], c->main.stream));
    advance_transparent(c, B);
    b->replays++;
    return DG_OK;
}

dg_status dg_batch_info(dg_batch* b, uint64_t* out, int32_t n) {
    if (!b || !out || n < 0) return DG_E_INVALID;
    const uint64_t v[5] = {b->scenes.size(), b->captures, b->replays, b->launches, b->h2d};
    for (int32_t i = 0; i < n && i < 5; i++) out[i] = v[i];
    return DG_OK;
}

dg_status dg_batch_destroy(dg_batch* b) {
    if (!b) return DG_E_INVALID;
    if (b->ctx && b->ctx->device >= 0) {
        cudaSetDevice(b->ctx->device);
        if (b->ctx->main.stream) cudaStreamSynchronize(b->ctx->main.stream);
    }
    drop_graphs(b);
    slot_free(b->slot);
    for (int k = 0; k < 2; k++) {
        if (b->h_stage[k]) cudaFreeHost(b->h_stage[k]);
        if (b->d_stage[k]) cudaFree(b->d_stage[k]);
        if (b->done[k]) cudaEventDestroy(b->done[k]);
    }
    if (b->cap) cudaStreamDestroy(b->cap);
    delete b;
    return DG_OK;
}

dg_status dg_autotune(dg_ctx* c, const int32_t* scenes, const int32_t* canvases, uint32_t n, uint32_t reps,
                      dg_tuning* best, float* best_ms) {
    if (!c || n == 0 || !scenes || !canvases || reps == 0 || reps > 1000) return DG_E_INVALID;
    if (!canvases_distinct(canvases, n)) return DG_E_INVALID;
    if (c->device < 0) return DG_E_CUDA;
    dg_status e = set_device(c);
    if (e) return e;
    std::vector<Scene*> sc;
    std::vector<FrameTarget> tg;
    e = resolve_frames(c, scenes, canvases, n, sc, tg);
    if (e) return e;
    dg_tuning cur;
    e = dg_ctx_get_tuning(c, &cur);
    if (e) return e;
    const dg_tuning start = cur;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    DG_CUDA(cudaEventCreate(&e0));
    if (cudaEventCreate(&e1) != cudaSuccess) {
        cudaEventDestroy(e0);
        return DG_E_CUDA;
    }
    // Candidate values per knob, searched one knob at a time (two sweeps).
    struct Knob {
        uint32_t dg_tuning::*field;
        std::vector<uint32_t> values;
    };
    const Knob knobs[] = {
        {&dg_tuning::small_max_px, {0, 4, 16, 64, 256}},
        {&dg_tuning::item_units, {2, 4, 8, 16, 32}},
        {&dg_tuning::queue_blocks_per_sm, {4, 8, 12, 16}},
        {&dg_tuning::setup_blocks_per_sm, {1, 2, 4, 8}},
        {&dg_tuning::cull_blocks_per_sm, {4, 8, 16, 32}},
        {&dg_tuning::tile_rows, {0, 8, 16, 32}},
    };
    float cur_ms = 0.0f;
    e = time_tuning(c, scenes, canvases, n, reps, e0, e1, &cur_ms);
    for (int sweep = 0; sweep < 2 && !e; sweep++) {
        for (const Knob& k : knobs) {
            const uint32_t keep = cur.*(k.field);
            uint32_t best_v = keep;
            for (uint32_t v : k.values) {
                if (v == keep) continue;
                dg_tuning t = cur;
                t.*(k.field) = v;
                if ((e = dg_ctx_set_tuning(c, &t)) != DG_OK) break;
                float ms = 0.0f;
                if ((e = time_tuning(c, scenes, canvases, n, reps, e0, e1, &ms)) != DG_OK) break;
                if (ms < cur_ms * 0.98f) {  // a change must win by 2% to count over timing noise
                    cur_ms = ms;
                    best_v = v;
                }
            }
            if (e) break;
            cur.*(k.field) = best_v;
            if ((e = dg_ctx_set_tuning(c, &cur)) != DG_OK) break;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e) {
        dg_ctx_set_tuning(c, &start);
        return e;
    }
    if (best) *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return DG_OK;
}

}  // extern "C"
