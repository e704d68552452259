// dg_server.cu -- a continuous-batching render server on one GPU.
//
// Clients submit render requests (a resident object, a frame size, a camera,
// lights) from any thread. Requests go to one of two lanes: large ones (at
// least 1920x1080 pixels or 1M triangles) and the rest, each lane with its own
// arrival-ordered queue and its own job slots (stream and scratch), so a small
// request never waits behind a large frame; a slot whose own lane is empty
// takes requests of the other lane. A scheduler thread admits pending
// requests of a lane in arrival order while the device-memory budget allows
// (each request holds colour, depth and visibility buffers; job-slot scratch
// counts too), packs up to max_batch of them (large lane: at most
// kLargeBatch) into one render job, and launches it on a free slot of the lane.
// Several batches are in flight at once, so requests that arrive while others
// run are admitted as soon as a slot and memory free up, and their work
// overlaps on the device. A host callback on the slot's stream stamps each
// request's completion time.
//
// Request buffers are pooled per frame size: a finished request's buffers go
// back to the pool (their visibility keys are all empty again: the resolve
// pass resets every key it reads), so a later request of that size takes them
// without an allocation or a clear. Pooled buffers count against the budget;
// when a request does not fit, pooled buffers of other sizes are released.
//
// Every request renders exactly as dg_scene_render would render it alone: a
// batch is the same kernels over more frames, with per-frame keys and buffers.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "dg_host.h"

using namespace dgh;

namespace {

double now_s() {
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

enum ReqState { kPending = 0, kRunning = 1, kDone = 2 };

constexpr int kLanes = 2;            // 0: small requests, 1: large ones
constexpr uint32_t kLargeBatch = 16;  // requests per batch in the large lane
constexpr uint64_t kLargePixels = 1920ull * 1080ull;
constexpr uint64_t kLargeTris = 1000000ull;

struct Request {
    uint64_t ticket = 0;
    Scene scene;
    FrameTarget tgt{};
    void* mem = nullptr;  // one buffer set: vis | colour | depth | cells
    uint64_t bytes = 0;
    uint64_t size_key = 0;  // (width << 32) | height: the buffer pool of the request's size
    int lane = 0;
    double t_submit = 0, t_start = 0, t_done = 0;
    int state = kPending;
    dg_status status = DG_OK;
    bool discard = false;
    bool fail_alloc = false;  // dg_server_inject_alloc_failure
};

struct Slot {
    JobSlot js;
    bool busy = false;
    int lane = 0;
    std::vector<Request*> batch;
    uint32_t* h_err = nullptr;  // pinned copy of the slot's error word
    struct dg_server* srv = nullptr;
};

}  // namespace

struct dg_server {
    dg_ctx* ctx = nullptr;
    uint64_t budget = 0;
    uint64_t used = 0;       // request buffers + slot scratch
    uint64_t peak_used = 0;
    uint64_t held_done = 0;  // buffers of finished requests not yet collected by dg_server_wait
    uint32_t max_batch = 1;
    std::vector<std::unique_ptr<Slot>> slots;
    std::deque<Request*> pending[kLanes];
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    // buffers back from finished requests, by frame size (counted in `used`)
    std::unordered_map<uint64_t, std::vector<void*>> pool;
    uint64_t pooled_bytes = 0;
    std::vector<void*> to_free;  // buffers the scheduler releases to the device
    std::vector<uint64_t> to_free_bytes;
    std::mutex mu;
    std::condition_variable cv_sched, cv_done;
    std::thread thr;
    bool stop = false;
    uint64_t next_ticket = 1;
    std::vector<double> latencies_ms;
    uint64_t batches = 0, frames = 0;
    uint64_t allocations = 0;  // buffer sets allocated (the others came from the pool)
    dg_status sticky = DG_OK;  // first launch error, reported by later calls
    cudaStream_t copy_stream = nullptr;
};

namespace {

uint64_t request_bytes(uint64_t w, uint64_t h) { return w * h * (4 + 4 + 8) + dg_cell_count(w, h) * 4; }

// A finished request's buffers go back to the pool of its size (lock held).
void pool_put(dg_server* s, Request* r) {
    s->pool[r->size_key].push_back(r->mem);
    s->pooled_bytes += r->bytes;
    r->mem = nullptr;
}

// Host callback at the end of a batch on its slot stream (no CUDA calls allowed here).
void CUDART_CB batch_done(void* arg) {
    Slot* sl = static_cast<Slot*>(arg);
    dg_server* s = sl->srv;
    const double t = now_s();
    std::lock_guard<std::mutex> lk(s->mu);
    dg_status st = DG_OK;
    for (int b = 1; b < 32; b++)
        if (*sl->h_err & (1u << b)) {
            st = (dg_status)b;
            break;
        }
    for (Request* r : sl->batch) {
        r->t_done = t;
        r->state = kDone;
        r->status = st;
        s->latencies_ms.push_back((r->t_done - r->t_submit) * 1e3);
        if (r->discard) {
            if (st == DG_OK) {
                pool_put(s, r);
            } else {  // keys may be left set: the buffers are released, not pooled
                s->to_free.push_back(r->mem);
                s->to_free_bytes.push_back(r->bytes);
                r->mem = nullptr;
            }
        } else {
            s->held_done += r->bytes;  // kept until the client collects the frame
        }
    }
    s->frames += sl->batch.size();
    sl->batch.clear();
    sl->busy = false;
    s->cv_sched.notify_all();
    s->cv_done.notify_all();
}

// Launches one batch on slot sl (called by the scheduler without the lock
// held). Each request takes a pooled buffer set of its size or allocates one
// (a fresh set has its visibility keys cleared once). A request whose
// allocation fails completes alone with DG_E_OOM; the others still render.
dg_status launch_batch(dg_server* s, Slot* sl, std::vector<Request*>& batch, uint64_t reserved) {
    cudaStream_t st = sl->js.stream;
    const uint64_t scratch_before = sl->js.scratch_bytes;
    // the admission reserved the predicted scratch growth; settle it against the actual one
    auto settle = [&]() {
        std::lock_guard<std::mutex> lk(s->mu);
        s->used = s->used - reserved + (sl->js.scratch_bytes - scratch_before);
        s->peak_used = std::max(s->peak_used, s->used);
    };
    std::vector<Request*> run;
    for (Request* r : batch) {
        const uint64_t n = r->scene.width * r->scene.height;
        if (!r->mem) {  // not from the pool: allocate and clear the keys
            if (r->fail_alloc || cudaMallocAsync(&r->mem, r->bytes, st) != cudaSuccess) {
                cudaGetLastError();
                r->mem = nullptr;
                std::lock_guard<std::mutex> lk(s->mu);
                s->used -= r->bytes;
                r->state = kDone;
                r->status = DG_E_OOM;
                r->t_done = now_s();
                s->latencies_ms.push_back((r->t_done - r->t_submit) * 1e3);
                s->cv_done.notify_all();
                continue;
            }
            {
                std::lock_guard<std::mutex> lk(s->mu);
                s->allocations++;
            }
            if (cudaMemsetAsync(r->mem, 0xFF, n * 8, st) != cudaSuccess) {
                cudaGetLastError();
                settle();
                return DG_E_CUDA;
            }
        }
        uint8_t* base = static_cast<uint8_t*>(r->mem);
        r->tgt.vis = reinterpret_cast<uint64_t*>(base);
        r->tgt.colour = reinterpret_cast<uint32_t*>(base + n * 8);
        r->tgt.depth = reinterpret_cast<float*>(base + n * 12);
        // the cells keep whatever the memory held: a word equal to this request's
        // ticket (unique among the server's requests) was written by this frame
        r->tgt.cells = reinterpret_cast<uint32_t*>(base + n * 16);
        r->tgt.epoch = (uint32_t)r->ticket;
        r->tgt.w = r->scene.width;
        r->tgt.h = r->scene.height;
        r->tgt.off_x = r->tgt.off_y = 0.0f;
        run.push_back(r);
    }
    batch.swap(run);
    if (batch.empty()) {
        settle();
        std::lock_guard<std::mutex> lk(s->mu);
        sl->busy = false;
        s->cv_sched.notify_all();
        return DG_OK;
    }
    std::vector<Scene*> sc(batch.size());
    std::vector<FrameTarget> tg(batch.size());
    for (size_t i = 0; i < batch.size(); i++) {
        sc[i] = &batch[i]->scene;
        tg[i] = batch[i]->tgt;
    }
    dg_status e = launch_frames(s->ctx, sl->js, sc.data(), tg.data(), (uint32_t)batch.size());
    settle();
    if (e) return e;
    if (cudaMemcpyAsync(sl->h_err, sl->js.d_err, 4, cudaMemcpyDeviceToHost, st) != cudaSuccess) return DG_E_CUDA;
    if (cudaMemsetAsync(sl->js.d_err, 0, 4, st) != cudaSuccess) return DG_E_CUDA;
    sl->batch = batch;
    if (cudaLaunchHostFunc(st, batch_done, sl) != cudaSuccess) return DG_E_CUDA;
    return DG_OK;
}

// The lane a request waits in (lane 0 when the server has no large-lane slot).
int lane_of(const dg_server* s, uint64_t pixels, uint64_t tris) {
    const bool large = pixels >= kLargePixels || tris >= kLargeTris;
    return (large && s->slots.size() > 1) ? 1 : 0;
}

void scheduler(dg_server* s) {
    cudaSetDevice(s->ctx->device);
    std::unique_lock<std::mutex> lk(s->mu);
    for (;;) {
        // release the buffers handed to the device
        if (!s->to_free.empty()) {
            std::vector<void*> fr;
            fr.swap(s->to_free);
            uint64_t b = 0;
            for (uint64_t x : s->to_free_bytes) b += x;
            s->to_free_bytes.clear();
            lk.unlock();
            for (void* p : fr) cudaFreeAsync(p, s->copy_stream);
            lk.lock();
            s->used -= b;
        }
        bool any_busy = false;
        for (auto& sl : s->slots) any_busy = any_busy || sl->busy;
        const bool any_pending = !s->pending[0].empty() || !s->pending[1].empty();
        if (s->stop && !any_pending && !any_busy) break;
        bool launched = false, freed = false;
        for (int pass = 0; pass < 2 * kLanes && !launched && !freed; pass++) {
            // passes 0, 1: each lane's queue on a free slot of that lane; passes 2, 3:
            // a lane's queue on a free slot of the other lane (whose own queue is empty)
            const int lane = pass % kLanes;
            const int slot_lane = pass < kLanes ? lane : 1 - lane;
            std::deque<Request*>& q = s->pending[lane];
            if (q.empty()) continue;
            if (pass >= kLanes && !s->pending[slot_lane].empty()) continue;
            Slot* free_slot = nullptr;
            for (auto& sl : s->slots)
                if (!sl->busy && sl->lane == slot_lane) {
                    free_slot = sl.get();
                    break;
                }
            if (!free_slot) continue;
            // admit in arrival order while the batch size and the memory budget allow; the
            // budget covers the requests' buffers and the scratch growth of the batch
            std::vector<Request*> batch;
            uint64_t reserved = 0;  // growth of the slot's scratch this batch will cause
            uint64_t V = 0, T = 0, P = 0;
            uint32_t L = 1;
            const uint64_t cur = free_slot->js.scratch_bytes;
            const uint32_t cap = lane == 1 ? std::min(s->max_batch, kLargeBatch) : s->max_batch;
            while (!q.empty() && batch.size() < cap) {
                Request* r = q.front();
                const Object& o = s->ctx->objects[r->scene.objects[0]];
                const uint64_t V2 = V + o.nv, T2 = T + o.ntri_opaque, P2 = P + r->scene.width * r->scene.height;
                const uint32_t L2 = std::max<uint32_t>(L, (uint32_t)r->scene.lights.size());
                const uint64_t after = slot_scratch_after(free_slot->js, V2, T2, L2, P2);
                const uint64_t grow_by = after > cur ? after - cur : 0;
                auto pit = s->pool.find(r->size_key);
                const bool pooled = !r->fail_alloc && pit != s->pool.end() && !pit->second.empty();
                const uint64_t need = (grow_by - reserved) + (pooled ? 0 : r->bytes);
                if (s->used + need > s->budget) {
                    // release pooled buffers of other sizes, then try again
                    for (auto& kv : s->pool) {
                        if (kv.first == r->size_key) continue;
                        const uint64_t w = kv.first >> 32, h = kv.first & 0xFFFFFFFFull;
                        for (void* m : kv.second) {
                            s->to_free.push_back(m);
                            s->to_free_bytes.push_back(request_bytes(w, h));
                            s->pooled_bytes -= request_bytes(w, h);
                            freed = true;
                        }
                        kv.second.clear();
                    }
                    break;
                }
                if (pooled) {
                    r->mem = pit->second.back();
                    pit->second.pop_back();
                    s->pooled_bytes -= r->bytes;
                }
                s->used += need;
                reserved = grow_by;
                V = V2;
                T = T2;
                P = P2;
                L = L2;
                s->peak_used = std::max(s->peak_used, s->used);
                q.pop_front();
                r->state = kRunning;
                r->t_start = now_s();
                batch.push_back(r);
            }
            if (batch.empty()) {
                if (!freed && !any_busy && s->held_done == 0 && s->to_free.empty()) {
                    // nothing runs, nothing waits to be collected and no pooled buffer
                    // can be released, yet the head request (with the scratch its job
                    // needs) does not fit the budget: refuse it
                    Request* r = q.front();
                    q.pop_front();
                    r->state = kDone;
                    r->status = DG_E_OOM;
                    r->t_done = now_s();
                    s->cv_done.notify_all();
                    freed = true;  // look at the queues again
                }
                continue;
            }
            free_slot->busy = true;
            s->batches++;
            lk.unlock();
            dg_status e = launch_batch(s, free_slot, batch, reserved);
            lk.lock();
            launched = true;
            if (e) {
                // the batch did not launch: its requests complete with the error
                if (!s->sticky) s->sticky = e;
                const double t = now_s();
                for (Request* r : batch) {
                    if (r->state == kDone) continue;
                    r->state = kDone;
                    r->status = e;
                    r->t_done = t;
                    if (r->mem) {
                        s->to_free.push_back(r->mem);
                        s->to_free_bytes.push_back(r->bytes);
                        r->mem = nullptr;
                    } else {
                        s->used -= r->bytes;
                    }
                }
                free_slot->batch.clear();
                free_slot->busy = false;
                s->cv_done.notify_all();
            }
        }
        if (!launched && !freed) s->cv_sched.wait(lk);
    }
}

}  // namespace

extern "C" {

dg_status dg_server_create(dg_ctx* ctx, uint64_t budget_bytes, uint32_t max_batch, uint32_t streams,
                           dg_server** out) {
    if (!ctx || !out || max_batch == 0 || streams == 0 || streams > 16) return DG_E_INVALID;
    *out = nullptr;
    dg_status e = set_device(ctx);
    if (e) return e;
    std::unique_ptr<dg_server> s(new (std::nothrow) dg_server());
    if (!s) return DG_E_OOM;
    s->ctx = ctx;
    s->budget = budget_bytes;
    s->max_batch = max_batch;
    // keep freed request buffers in the stream-ordered pool for reuse
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, ctx->device) == cudaSuccess) {
        uint64_t thr = budget_bytes;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    cudaGetLastError();
    if (cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking) != cudaSuccess) return DG_E_CUDA;
    e = sync_tex_table(ctx, ctx->main.stream);
    if (e) return e;
    for (uint32_t i = 0; i < streams; i++) {
        auto sl = std::make_unique<Slot>();
        sl->srv = s.get();
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess) return DG_E_CUDA;
        e = slot_init(ctx, sl->js, st);
        if (e) return e;
        if (cudaMallocHost((void**)&sl->h_err, 4) != cudaSuccess) return DG_E_OOM;
        *sl->h_err = 0;
        // one slot in three (at least one) serves the large lane when there are two or more
        sl->lane = (streams > 1 && i < std::max<uint32_t>(1u, streams / 3u)) ? 1 : 0;
        s->slots.push_back(std::move(sl));
    }
    s->thr = std::thread(scheduler, s.get());
    *out = s.release();
    return DG_OK;
}

dg_status dg_server_submit(dg_server* s, const dg_request* q, uint64_t* ticket) {
    if (!s || !q || !ticket) return DG_E_INVALID;
    dg_ctx* c = s->ctx;
    if (q->object < 0 || (size_t)q->object >= c->objects.size() || !c->objects[q->object].alive) return DG_E_INVALID;
    if (c->objects[q->object].nt > 0) return DG_E_LIMIT;  // requests render opaque meshes only
    if (q->width == 0 || q->height == 0 || q->width > 65535 || q->height > 65535) return DG_E_INVALID;
    if (q->nlights == 0 || q->nlights > DG_MAX_LIGHTS) return DG_E_INVALID;
    auto r = std::make_unique<Request>();
    r->scene.width = q->width;
    r->scene.height = q->height;
    r->scene.objects.push_back(q->object);
    for (uint32_t l = 0; l < q->nlights; l++) r->scene.lights.push_back(h3(q->lights[l][0], q->lights[l][1], q->lights[l][2]));
    r->scene.exponent = q->exponent;
    const float ratio = (float)q->width / (float)q->height;
    dg_status e = camera_init(r->scene.cam, h3(q->cam_pos[0], q->cam_pos[1], q->cam_pos[2]),
                              h3(q->cam_dir[0], q->cam_dir[1], q->cam_dir[2]), ratio, q->near_, q->far_, q->fov_x_deg);
    if (e) return e;
    r->tgt.clear_depth = q->clear_depth;
    r->bytes = request_bytes(q->width, q->height);
    r->size_key = ((uint64_t)q->width << 32) | q->height;
    r->discard = q->discard != 0;
    std::lock_guard<std::mutex> lk(s->mu);
    if (s->stop) return DG_E_INVALID;
    if (r->bytes > s->budget) return DG_E_OOM;  // could never be admitted
    r->lane = lane_of(s, (uint64_t)q->width * q->height, c->objects[q->object].ntri_opaque);
    r->ticket = s->next_ticket++;
    r->t_submit = now_s();
    *ticket = r->ticket;
    s->pending[r->lane].push_back(r.get());
    s->reqs.emplace(r->ticket, std::move(r));
    s->cv_sched.notify_all();
    return DG_OK;
}

dg_status dg_server_wait(dg_server* s, uint64_t ticket, uint8_t* bgra, float* depth, double* latency_ms) {
    if (!s) return DG_E_INVALID;
    Request* r = nullptr;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return DG_E_INVALID;
    r = it->second.get();
    s->cv_done.wait(lk, [&] { return r->state == kDone; });
    dg_status st = r->status;
    if (latency_ms) *latency_ms = (r->t_done - r->t_submit) * 1e3;
    void* mem = r->mem;
    const uint64_t bytes = r->bytes;
    const uint64_t size_key = r->size_key;
    const uint64_t n = r->scene.width * r->scene.height;
    r->mem = nullptr;
    s->reqs.erase(it);
    lk.unlock();
    if (mem) {
        cudaSetDevice(s->ctx->device);
        uint8_t* base = static_cast<uint8_t*>(mem);
        const dg_status frame_st = st;
        if (st == DG_OK && bgra && cudaMemcpy(bgra, base + n * 8, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = DG_E_CUDA;
        if (st == DG_OK && depth && cudaMemcpy(depth, base + n * 12, n * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            st = DG_E_CUDA;
        lk.lock();
        if (frame_st == DG_OK) {  // the frame reset its keys: the buffers go back to the pool
            s->pool[size_key].push_back(mem);
            s->pooled_bytes += bytes;
        } else {
            s->to_free.push_back(mem);
            s->to_free_bytes.push_back(bytes);
        }
        s->held_done -= bytes;
        s->cv_sched.notify_all();
    }
    return st;
}

dg_status dg_server_stats(dg_server* s, double* out, int32_t n) {
    if (!s || !out || n < 0) return DG_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    std::vector<double> l = s->latencies_ms;
    std::sort(l.begin(), l.end());
    auto pct = [&](double p) {
        if (l.empty()) return 0.0;
        size_t i = (size_t)std::min<double>(l.size() - 1, std::max(0.0, p * (l.size() - 1) + 0.5));
        return l[i];
    };
    double v[9] = {(double)l.size(), pct(0.5), pct(0.99), l.empty() ? 0.0 : l.back(), (double)s->batches,
                   s->batches ? (double)s->frames / (double)s->batches : 0.0, (double)s->peak_used,
                   (double)s->sticky, (double)s->allocations};
    for (int i = 0; i < n && i < 9; i++) out[i] = v[i];
    return DG_OK;
}

dg_status dg_server_reset_stats(dg_server* s) {
    if (!s) return DG_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    s->latencies_ms.clear();
    s->batches = 0;
    s->frames = 0;
    s->allocations = 0;
    s->peak_used = s->used;
    return DG_OK;
}

dg_status dg_server_cancel(dg_server* s, uint64_t ticket) {
    if (!s) return DG_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end() || it->second->state != kPending) return DG_E_INVALID;
    Request* r = it->second.get();
    std::deque<Request*>& q = s->pending[r->lane];
    q.erase(std::find(q.begin(), q.end(), r));
    r->state = kDone;
    r->status = DG_E_CANCELLED;
    r->t_done = now_s();
    s->cv_done.notify_all();
    return DG_OK;
}

dg_status dg_server_inject_alloc_failure(dg_server* s, uint64_t ticket) {
    if (!s) return DG_E_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end() || it->second->state != kPending) return DG_E_INVALID;
    it->second->fail_alloc = true;
    return DG_OK;
}

dg_status dg_server_destroy(dg_server* s) {
    if (!s) return DG_E_INVALID;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        s->cv_sched.notify_all();
    }
    if (s->thr.joinable()) s->thr.join();
    cudaSetDevice(s->ctx->device);
    for (auto& kv : s->reqs)
        if (kv.second->mem) cudaFreeAsync(kv.second->mem, s->copy_stream);
    for (void* p : s->to_free) cudaFreeAsync(p, s->copy_stream);
    for (auto& kv : s->pool)
        for (void* p : kv.second) cudaFreeAsync(p, s->copy_stream);
    cudaStreamSynchronize(s->copy_stream);
    for (auto& sl : s->slots) {
        cudaStream_t st = sl->js.stream;
        slot_free(sl->js);
        if (st) cudaStreamDestroy(st);
        if (sl->h_err) cudaFreeHost(sl->h_err);
    }
    cudaStreamDestroy(s->copy_stream);
    delete s;
    return DG_OK;
}

}  // extern "C"
