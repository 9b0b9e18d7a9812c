// Serving engine: continuous batching over one device-resident arena.
//
// One cudaMalloc of the HBM budget at start-up holds everything the engine
// puts on the device: request payloads, per-launch scratch (mesh table,
// meshlet queue, descriptors, scan sums, walk entries, status) and result
// buffers.  A first-fit allocator with coalescing hands out 256-byte aligned
// ranges of it, so admission is "does this request's payload (and its share
// of a launch's outputs and scratch) fit right now".
//
// A scheduler thread forms a launch from the queued requests in arrival
// order (up to max_batch of them, as many as the arena admits), uploads
// their payloads -- each copied into pinned memory by the thread that
// submitted it (up to a pinned budget; past it through a pinned staging
// buffer) -- and runs the same scan / connectivity / vertex kernels as a
// batch over their concatenated meshlet queue on one of n_streams
// non-blocking streams.  Up to n_streams launches
// are in flight, so requests that arrive while others decode are admitted as
// soon as a stream and arena space are free, and their copies and kernels
// overlap the running launch on the device.  A host function placed on the
// stream after the kernels (and after the optional copies to host) marks the
// launch finished; it only touches a completion list, never the engine lock,
// so the scheduler may hold that lock across CUDA calls.
//
// A launch whose status reports an error fails the request that owns the
// failing meshlet and re-queues the others (the kernels stop early once an
// error is recorded, so their outputs are incomplete); each request's result
// is therefore exactly what decoding it alone gives.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "stride_common.cuh"
#include "stride_gb300.h"
#include "stride_internal.h"

using namespace stride;

namespace {

constexpr uint64_t kAlign = 256;
// Pinned host slab for the payloads of queued and running requests
// (stride_server_opts::pinned_budget_bytes, 0: this), pinned once when the
// server is created: pinning on the submit path took milliseconds per new
// buffer and held the engine lock meanwhile.  A payload that finds no room
// waits in pageable memory and goes through a launch's staging buffer.
constexpr uint64_t kPayloadSlab = uint64_t(1) << 30;

uint64_t up(uint64_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

double now_us(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
}

// First-fit allocator over [0, size) with coalescing of neighbours.
class Arena {
  public:
    void reset(uint64_t size) {
        size_ = size;
        free_.clear();
        if (size) free_[0] = size;
        used_ = peak_ = 0;
    }
    bool alloc(uint64_t bytes, uint64_t* off) {
        bytes = up(std::max<uint64_t>(bytes, 1));
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            *off = it->first;
            const uint64_t rest = it->second - bytes;
            const uint64_t next = it->first + bytes;
            free_.erase(it);
            if (rest) free_[next] = rest;
            used_ += bytes;
            peak_ = std::max(peak_, used_);
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t bytes) {
        bytes = up(std::max<uint64_t>(bytes, 1));
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    uint64_t size() const { return size_; }
    uint64_t peak() const { return peak_; }

  private:
    uint64_t size_ = 0, used_ = 0, peak_ = 0;
    std::map<uint64_t, uint64_t> free_;
};

// Device scratch of one launch over these totals (arena bytes).
struct ScratchPlan {
    uint64_t params, map, lut_list, descs, sums, prefix, walk, lut, status, total;
};

// lut_floats: dequantisation table floats of the launch's meshes
ScratchPlan plan_scratch(uint32_t n_meshes, uint32_t meshlets, uint64_t n_v, uint64_t lut_floats) {
    ScratchPlan s;
    const uint32_t nb = std::max<uint32_t>(1u, scan_blocks(meshlets));
    uint64_t o = 0;
    s.params = o;
    o += up(sizeof(MeshParams) * n_meshes);
    s.map = o;
    o += up(4ull * std::max<uint32_t>(1u, meshlets));
    s.lut_list = o;
    o += up(4ull * n_meshes);
    s.descs = o;
    o += up(sizeof(MeshletDesc) * std::max<uint32_t>(1u, meshlets));
    s.sums = o;
    o += up(sizeof(uint4) * nb);
    s.prefix = o;
    o += up(sizeof(BlockPrefix) * nb);
    s.walk = o;
    o += up(4ull * walk_scratch_words(n_v, meshlets));
    s.lut = o;
    o += up(4ull * lut_floats);
    s.status = o;
    o += up(sizeof(Status));
    s.total = o;
    return s;
}

uint64_t out_bytes(uint64_t n_v, uint64_t n_t) { return up(12ull * n_t) + up(12ull * n_v); }

struct Launch;

// Pinned host buffer, recycled through the engine's pool.
struct Pinned {
    uint8_t* ptr = nullptr;
    size_t bytes = 0;
};

struct Request {
    uint64_t id = 0;
    std::vector<uint8_t> data;  // the payload, unless it is in `pay`
    size_t len = 0;             // payload bytes
    MeshParams p{};
    enum State { kQueued, kRunning, kDone } state = kQueued;
    int status = STRIDE_OK;
    uint64_t blob_off = 0;  // arena, while running
    bool has_blob = false;
    std::shared_ptr<Launch> launch;  // owner of the result buffers once done
    uint8_t* pay = nullptr;          // the payload and kBlobPad zero bytes in the pinned slab (when set)
    uint64_t pay_off = 0;            // its offset in the slab
    uint64_t t_rel = 0, v_rel = 0;   // offsets inside the launch's outputs
    double t_submit = 0, t_admit = 0, t_done = 0;
};

struct Launch {
    uint64_t seq = 0;
    int slot = 0;
    std::vector<Request*> reqs;
    uint64_t total_v = 0, total_t = 0;
    uint32_t total_meshlets = 0;
    uint64_t out_off = 0, out_size = 0;
    uint64_t scratch_off = 0, scratch_size = 0;
    bool has_out = false, has_scratch = false;
    Pinned host;  // copies of the outputs (copy_to_host)
    int live = 0;  // requests whose results are not yet released
    std::atomic<int> finished{0};
    double t_done = 0;
    stride_server* srv = nullptr;
};

struct Slot {
    cudaStream_t stream = nullptr;
    Pinned stage;                   // payloads + mesh table + meshlet map
    Status* h_status = nullptr;     // pinned
    std::shared_ptr<Launch> busy;   // launch in flight on this stream
};

}  // namespace

struct stride_server {
    stride_server_opts opts{};
    int device = 0;
    std::chrono::steady_clock::time_point t0;
    uint8_t* d_arena = nullptr;
    Arena arena;

    std::mutex mu;                        // engine state
    std::condition_variable done_cv;      // request finished (waiters)
    std::deque<Request*> queue;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<Slot> slots;
    std::vector<Pinned> pinned_pool;      // staging and host-output buffers
    uint8_t* h_pay = nullptr;             // pinned payload slab
    Arena pay_arena;                      // its free space
    uint64_t next_id = 1, launches = 0, completed = 0, seq = 0;
    std::atomic<bool> stop{false};
    bool hold = false;                    // queue without dispatching (stride_server_hold)

    std::mutex cb_mu;                     // completion list + wake-ups only
    std::condition_variable cb_cv;
    std::vector<Launch*> finished;
    bool wake = false;

    std::thread scheduler;
};

namespace {

void notify_scheduler(stride_server* s) {
    {
        std::lock_guard<std::mutex> g(s->cb_mu);
        s->wake = true;
    }
    s->cb_cv.notify_one();
}

void CUDART_CB on_launch_done(void* arg) {
    Launch* l = static_cast<Launch*>(arg);
    stride_server* s = l->srv;
    l->t_done = now_us(s->t0);
    l->finished.store(1);
    {
        std::lock_guard<std::mutex> g(s->cb_mu);
        s->finished.push_back(l);
        s->wake = true;
    }
    s->cb_cv.notify_one();
}

bool pinned_get(stride_server* s, size_t bytes, Pinned* out) {
    // smallest pooled buffer that fits, else a new one
    size_t best = SIZE_MAX;
    for (size_t i = 0; i < s->pinned_pool.size(); i++)
        if (s->pinned_pool[i].bytes >= bytes && (best == SIZE_MAX || s->pinned_pool[i].bytes < s->pinned_pool[best].bytes))
            best = i;
    if (best != SIZE_MAX) {
        *out = s->pinned_pool[best];
        s->pinned_pool.erase(s->pinned_pool.begin() + best);
        return true;
    }
    // sizes in powers of two from 1 MiB: pinning host memory takes
    // milliseconds per tens of MiB and stalls every queued request, so the
    // pool settles on a few size classes after a handful of allocations
    // instead of growing by one odd size per launch
    Pinned p;
    p.bytes = size_t(1) << 20;
    while (p.bytes < bytes) p.bytes <<= 1;
    if (cudaHostAlloc(reinterpret_cast<void**>(&p.ptr), p.bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    *out = p;
    return true;
}

void pinned_put(stride_server* s, Pinned& p) {
    if (p.ptr) s->pinned_pool.push_back(p);
    p = Pinned{};
}

// Arena bytes one request needs when it runs alone.
uint64_t footprint(const MeshParams& p, size_t len) {
    return up(blob_alloc_bytes(len)) + out_bytes(p.n_v, p.n_t) + plan_scratch(1, p.n_meshlets, p.n_v, lut_entries(p)).total;
}

void finish_request(stride_server* s, Request* r, int status) {
    r->status = status;
    r->state = Request::kDone;
    if (r->has_blob) {
        s->arena.release(r->blob_off, blob_alloc_bytes(r->len));
        r->has_blob = false;
    }
    if (r->pay) {  // its upload, if any, has completed: the launch retired
        s->pay_arena.release(r->pay_off, r->len + kBlobPad);
        r->pay = nullptr;
    }
    s->completed++;
}

void free_launch_buffers(stride_server* s, Launch* l) {
    if (l->has_scratch) s->arena.release(l->scratch_off, l->scratch_size);
    l->has_scratch = false;
}

void free_launch_outputs(stride_server* s, Launch* l) {
    if (l->has_out) s->arena.release(l->out_off, l->out_size);
    l->has_out = false;
    pinned_put(s, l->host);
}

// Completed launch: read its status, finish or re-queue its requests.
void retire(stride_server* s, Launch* l) {
    Slot& slot = s->slots[l->slot];
    std::shared_ptr<Launch> keep = slot.busy;  // == l
    slot.busy.reset();
    // surfaces launch faults; "not ready" is the completion host function
    // itself, which may not yet count as finished when this runs
    const cudaError_t ce = cudaStreamQuery(slot.stream);
    uint32_t bad = 0;
    int code = (ce == cudaSuccess || ce == cudaErrorNotReady) ? status_to_code(*slot.h_status, &bad)
                                                              : STRIDE_ERR_CUDA;
    free_launch_buffers(s, l);
    if (code == STRIDE_OK) {
        for (Request* r : l->reqs) {
            r->t_done = l->t_done;
            r->launch = keep;
            finish_request(s, r, STRIDE_OK);
        }
        l->live = static_cast<int>(l->reqs.size());
        if (l->live == 0) free_launch_outputs(s, l);
    } else {
        // the request owning the failing meshlet fails; the rest run again
        std::vector<Request*> again;
        for (Request* r : l->reqs) {
            const uint32_t b = r->p.meshlet_begin;
            const bool culprit = code == STRIDE_ERR_CUDA || l->reqs.size() == 1 ||
                                 (bad >= b && bad < b + r->p.n_meshlets);
            if (culprit) {
                r->t_done = l->t_done;
                finish_request(s, r, code);
            } else {
                if (r->has_blob) {
                    s->arena.release(r->blob_off, blob_alloc_bytes(r->len));
                    r->has_blob = false;
                }
                r->state = Request::kQueued;
                again.push_back(r);
            }
        }
        for (auto it = again.rbegin(); it != again.rend(); ++it) s->queue.push_front(*it);
        l->reqs.clear();
        free_launch_outputs(s, l);
    }
    s->done_cv.notify_all();
}

// Forms and enqueues one launch on `slot_i` from the queue head; false if
// nothing could be admitted.
bool dispatch(stride_server* s, int slot_i) {
    Slot& slot = s->slots[slot_i];
    auto l = std::make_shared<Launch>();
    l->srv = s;
    l->slot = slot_i;
    const uint32_t max_batch = s->opts.max_batch ? s->opts.max_batch : 256u;
    // take requests in arrival order while payload, outputs and scratch fit
    std::vector<Request*> take;
    uint64_t tv = 0, tt = 0, tl = 0;
    uint32_t tm = 0;
    for (Request* r : s->queue) {
        if (take.size() >= max_batch) break;
        if (static_cast<uint64_t>(tm) + r->p.n_meshlets > 0xFFFFFFF0ull) break;
        uint64_t off = 0;
        if (!s->arena.alloc(blob_alloc_bytes(r->len), &off)) break;
        // outputs + scratch for the launch with this request in it
        const uint64_t need = out_bytes(tv + r->p.n_v, tt + r->p.n_t) +
                              plan_scratch(static_cast<uint32_t>(take.size() + 1), tm + r->p.n_meshlets,
                                           tv + r->p.n_v, tl + lut_entries(r->p)).total;
        uint64_t probe = 0;
        if (!s->arena.alloc(need, &probe)) {
            s->arena.release(off, blob_alloc_bytes(r->len));
            break;
        }
        s->arena.release(probe, need);
        r->blob_off = off;
        r->has_blob = true;
        take.push_back(r);
        tv += r->p.n_v;
        tt += r->p.n_t;
        tm += r->p.n_meshlets;
        tl += lut_entries(r->p);
    }
    if (take.empty()) return false;
    const ScratchPlan sp = plan_scratch(static_cast<uint32_t>(take.size()), tm, tv, tl);
    l->out_size = out_bytes(tv, tt);
    l->scratch_size = sp.total;
    // the probe above reserved nothing, so allocate for real (cannot fail:
    // the same bytes were free a moment ago and nothing ran in between)
    l->has_out = s->arena.alloc(l->out_size, &l->out_off);
    l->has_scratch = l->has_out && s->arena.alloc(l->scratch_size, &l->scratch_off);
    if (!l->has_scratch) {
        if (l->has_out) s->arena.release(l->out_off, l->out_size);
        l->has_out = false;
        for (Request* r : take) {
            s->arena.release(r->blob_off, blob_alloc_bytes(r->len));
            r->has_blob = false;
        }
        return false;
    }
    for (size_t i = 0; i < take.size(); i++) s->queue.pop_front();
    l->reqs = take;
    l->total_v = tv;
    l->total_t = tt;
    l->total_meshlets = tm;
    l->seq = ++s->seq;

    // mesh table: offsets relative to this launch's outputs
    std::vector<MeshParams> params(take.size());
    uint64_t v = 0, t = 0;
    uint32_t m = 0;
    const double t_admit = now_us(s->t0);
    for (size_t i = 0; i < take.size(); i++) {
        Request* r = take[i];
        MeshParams p = r->p;
        p.blob_off = r->blob_off;
        p.meshlet_begin = m;
        p.v_offset = v;
        p.t_offset = t;
        r->p.meshlet_begin = m;  // for error attribution
        r->v_rel = v;
        r->t_rel = t;
        r->t_admit = t_admit;
        r->state = Request::kRunning;
        params[i] = p;
        v += p.n_v;
        t += p.n_t;
        m += p.n_meshlets;
    }
    uint32_t n_lut = 0, lut_max = 0;
    std::vector<uint32_t> lut_list(take.size());
    plan_luts(params.data(), static_cast<uint32_t>(take.size()), lut_list.data(),
              static_cast<uint32_t>(take.size()), &n_lut, &lut_max);
    // stage: mesh table | meshlet->mesh map | table mesh list | payloads
    const size_t list_off = up(sizeof(MeshParams) * take.size()) + up(4ull * std::max<uint32_t>(1u, tm));
    size_t stage_bytes = list_off + up(4ull * take.size());
    for (Request* r : take) stage_bytes += r->pay ? 0u : up(r->len);
    if (slot.stage.bytes < stage_bytes) {
        pinned_put(s, slot.stage);  // idle: the slot's previous launch has retired
        if (!pinned_get(s, stage_bytes, &slot.stage)) {
            for (Request* r : take) finish_request(s, r, STRIDE_ERR_NOMEM);
            free_launch_buffers(s, l.get());
            free_launch_outputs(s, l.get());
            s->done_cv.notify_all();
            return true;
        }
    }
    uint8_t* hs = slot.stage.ptr;
    std::memcpy(hs, params.data(), sizeof(MeshParams) * take.size());
    uint32_t* hmap = reinterpret_cast<uint32_t*>(hs + up(sizeof(MeshParams) * take.size()));
    for (size_t i = 0; i < take.size(); i++)
        std::fill(hmap + params[i].meshlet_begin, hmap + params[i].meshlet_begin + params[i].n_meshlets,
                  static_cast<uint32_t>(i));
    std::memcpy(hs + list_off, lut_list.data(), 4ull * n_lut);
    uint8_t* hp = hs + list_off + up(4ull * take.size());
    cudaStream_t st = slot.stream;
    uint8_t* base = s->d_arena;
    uint8_t* sc = base + l->scratch_off;
    cudaError_t e = cudaSuccess;
    e = cudaMemcpyAsync(sc + sp.params, hs, sizeof(MeshParams) * take.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && tm)
        e = cudaMemcpyAsync(sc + sp.map, hmap, 4ull * tm, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && n_lut)
        e = cudaMemcpyAsync(sc + sp.lut_list, hs + list_off, 4ull * n_lut, cudaMemcpyHostToDevice, st);
    for (Request* r : take) {
        if (e != cudaSuccess) break;
        if (r->pay) {  // payload and padding already pinned: one copy
            e = cudaMemcpyAsync(base + r->blob_off, r->pay, r->len + kBlobPad, cudaMemcpyHostToDevice, st);
            continue;
        }
        std::memcpy(hp, r->data.data(), r->len);
        e = cudaMemcpyAsync(base + r->blob_off, hp, r->len, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(base + r->blob_off + r->len, 0, kBlobPad, st);
        hp += up(r->len);
    }
    int rc = e == cudaSuccess ? STRIDE_OK : STRIDE_ERR_CUDA;
    if (rc == STRIDE_OK) {
        DecodeArgs a;
        a.arena = base;
        a.meshes = reinterpret_cast<const MeshParams*>(sc + sp.params);
        a.meshlet_mesh = reinterpret_cast<const uint32_t*>(sc + sp.map);
        a.total_meshlets = tm;
        a.n_meshes = static_cast<uint32_t>(take.size());
        a.descs = reinterpret_cast<MeshletDesc*>(sc + sp.descs);
        a.blk_sums = reinterpret_cast<uint4*>(sc + sp.sums);
        a.blk_prefix = reinterpret_cast<BlockPrefix*>(sc + sp.prefix);
        a.walk_scratch = reinterpret_cast<uint32_t*>(sc + sp.walk);
        a.walk_cap = walk_scratch_words(tv, tm);
        a.status = reinterpret_cast<Status*>(sc + sp.status);
        a.idx = reinterpret_cast<uint32_t*>(base + l->out_off);
        a.pos = reinterpret_cast<float*>(base + l->out_off + up(12ull * tt));
        a.codes = nullptr;
        a.lut = reinterpret_cast<float*>(sc + sp.lut);
        a.lut_meshes = reinterpret_cast<const uint32_t*>(sc + sp.lut_list);
        a.n_lut_meshes = n_lut;
        a.lut_max = lut_max;
        a.wide_codes = false;
        for (const MeshParams& p : params)
            a.wide_codes = a.wide_codes || p.g_bits[0] > 16 || p.g_bits[1] > 16 || p.g_bits[2] > 16;
        LaunchCfg cfg = default_config(tm);  // the launch's shape by its size
        if (a.wide_codes) cfg.code_bytes = std::max<uint32_t>(cfg.code_bytes, kMaxLocal * 4u);
        rc = enqueue_decode(a, cfg, st);
        if (rc == STRIDE_OK &&
            cudaMemcpyAsync(slot.h_status, a.status, sizeof(Status), cudaMemcpyDeviceToHost, st) != cudaSuccess)
            rc = STRIDE_ERR_CUDA;
        if (rc == STRIDE_OK && s->opts.copy_to_host) {
            if (!pinned_get(s, l->out_size, &l->host)) {
                rc = STRIDE_ERR_NOMEM;
            } else if (cudaMemcpyAsync(l->host.ptr, base + l->out_off, l->out_size, cudaMemcpyDeviceToHost, st) !=
                       cudaSuccess) {
                rc = STRIDE_ERR_CUDA;
            }
        }
        if (rc == STRIDE_OK && cudaLaunchHostFunc(st, on_launch_done, l.get()) != cudaSuccess) rc = STRIDE_ERR_CUDA;
    }
    if (rc != STRIDE_OK) {
        cudaStreamSynchronize(st);
        cudaGetLastError();
        for (Request* r : take) finish_request(s, r, rc);
        free_launch_buffers(s, l.get());
        free_launch_outputs(s, l.get());
        s->done_cv.notify_all();
        return true;
    }
    slot.busy = l;
    s->launches++;
    return true;
}

void scheduler_main(stride_server* s) {
    cudaSetDevice(s->device);
    for (;;) {
        std::vector<Launch*> done;
        {
            std::unique_lock<std::mutex> g(s->cb_mu);
            s->cb_cv.wait_for(g, std::chrono::milliseconds(50), [s] { return s->wake; });
            s->wake = false;
            done.swap(s->finished);
        }
        std::lock_guard<std::mutex> g(s->mu);
        for (Launch* l : done) retire(s, l);
        // a launch whose stream reports an error never reaches its host
        // function: retire it here with the error
        for (Slot& sl : s->slots) {
            if (!sl.busy || sl.busy->finished.load()) continue;
            const cudaError_t q = cudaStreamQuery(sl.stream);
            if (q != cudaSuccess && q != cudaErrorNotReady) {
                sl.busy->t_done = now_us(s->t0);
                retire(s, sl.busy.get());
            }
        }
        const bool stopping = s->stop.load();
        bool any_busy = false;
        for (Slot& sl : s->slots) any_busy = any_busy || sl.busy != nullptr;
        if (stopping) {
            while (!s->queue.empty()) {  // never admitted: fail them
                Request* r = s->queue.front();
                s->queue.pop_front();
                r->t_done = now_us(s->t0);
                finish_request(s, r, STRIDE_ERR_ARG);
            }
            s->done_cv.notify_all();
            if (!any_busy) break;
            continue;
        }
        // fill every idle stream while the queue admits something
        for (size_t i = 0; i < s->slots.size() && !s->queue.empty() && !s->hold; i++) {
            if (s->slots[i].busy) continue;
            if (!dispatch(s, static_cast<int>(i))) break;
        }
    }
}

}  // namespace

extern "C" {

int stride_server_create(const stride_server_opts* opts, stride_server** out) {
    if (!out || !opts) return fail(STRIDE_ERR_ARG, "null argument");
    *out = nullptr;
    if (opts->hbm_budget_bytes < (1ull << 20)) return fail(STRIDE_ERR_ARG, "HBM budget below 1 MiB");
    auto s = std::make_unique<stride_server>();
    s->opts = *opts;
    if (!s->opts.n_streams) s->opts.n_streams = 2;
    if (s->opts.n_streams > 16) s->opts.n_streams = 16;
    if (!s->opts.max_queue) s->opts.max_queue = 1u << 16;
    s->t0 = std::chrono::steady_clock::now();
    cudaError_t e = cudaGetDevice(&s->device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    const uint64_t budget = s->opts.hbm_budget_bytes & ~(kAlign - 1);
    if ((e = cudaMalloc(&s->d_arena, budget)) != cudaSuccess) return cuda_fail(e, "cudaMalloc(arena)");
    s->arena.reset(budget);
    const uint64_t slab = up(s->opts.pinned_budget_bytes ? s->opts.pinned_budget_bytes : kPayloadSlab);
    if ((e = cudaHostAlloc(reinterpret_cast<void**>(&s->h_pay), slab, cudaHostAllocDefault)) != cudaSuccess) {
        cudaFree(s->d_arena);
        return cuda_fail(e, "cudaHostAlloc(payload slab)");
    }
    s->pay_arena.reset(slab);
    s->slots.resize(s->opts.n_streams);
    for (Slot& sl : s->slots) {
        if ((e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking)) != cudaSuccess ||
            (e = cudaHostAlloc(reinterpret_cast<void**>(&sl.h_status), sizeof(Status), cudaHostAllocDefault)) !=
                cudaSuccess) {
            for (Slot& x : s->slots) {
                if (x.stream) cudaStreamDestroy(x.stream);
                if (x.h_status) cudaFreeHost(x.h_status);
            }
            cudaFreeHost(s->h_pay);
            cudaFree(s->d_arena);
            return cuda_fail(e, "stride_server_create");
        }
    }
    stride_server* raw = s.release();
    raw->scheduler = std::thread(scheduler_main, raw);
    *out = raw;
    return STRIDE_OK;
}

int stride_server_submit(stride_server* s, const uint8_t* data, size_t len, uint64_t* req_id) {
    if (!s || !data || !req_id) return fail(STRIDE_ERR_ARG, "null argument");
    auto r = std::make_unique<Request>();
    char why[256] = {0};
    const int rc = parse_header(data, len, &r->p, why, sizeof(why));
    if (rc) return fail(rc, "%s", why);
    if (footprint(r->p, len) > s->arena.size())
        return fail(STRIDE_ERR_NOMEM, "request needs %llu arena bytes alone; the HBM budget is %llu",
                    static_cast<unsigned long long>(footprint(r->p, len)),
                    static_cast<unsigned long long>(s->arena.size()));
    r->len = len;
    {  // room in the pinned slab, if any; the copy runs on this thread, unlocked
        std::lock_guard<std::mutex> g(s->mu);
        uint64_t off = 0;
        if (s->h_pay && s->pay_arena.alloc(len + kBlobPad, &off)) {
            r->pay = s->h_pay + off;
            r->pay_off = off;
        }
    }
    if (r->pay) {
        std::memcpy(r->pay, data, len);
        std::memset(r->pay + len, 0, kBlobPad);
    } else {
        r->data.assign(data, data + len);
    }
    {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->stop.load() || s->queue.size() >= s->opts.max_queue) {
            if (r->pay) s->pay_arena.release(r->pay_off, len + kBlobPad);
            if (s->stop.load()) return fail(STRIDE_ERR_ARG, "server is shutting down");
            return fail(STRIDE_ERR_BUSY, "request queue full");
        }
        r->id = s->next_id++;
        r->t_submit = now_us(s->t0);
        *req_id = r->id;
        s->queue.push_back(r.get());
        s->reqs.emplace(r->id, std::move(r));
    }
    notify_scheduler(s);
    return STRIDE_OK;
}

int stride_server_wait(stride_server* s, uint64_t req_id, int timeout_ms, stride_result* out) {
    if (!s || !out) return fail(STRIDE_ERR_ARG, "null argument");
    std::unique_lock<std::mutex> g(s->mu);
    auto it = s->reqs.find(req_id);
    if (it == s->reqs.end()) return fail(STRIDE_ERR_ARG, "unknown request %llu", static_cast<unsigned long long>(req_id));
    Request* r = it->second.get();
    auto ready = [r] { return r->state == Request::kDone; };
    if (timeout_ms < 0) {
        s->done_cv.wait(g, ready);
    } else if (!s->done_cv.wait_for(g, std::chrono::milliseconds(timeout_ms), ready)) {
        return fail(STRIDE_ERR_TIMEOUT, "request %llu still running", static_cast<unsigned long long>(req_id));
    }
    std::memset(out, 0, sizeof(*out));
    out->status = r->status;
    out->n_v = r->p.n_v;
    out->n_t = r->p.n_t;
    out->t_submit_us = r->t_submit;
    out->t_admit_us = r->t_admit;
    out->t_done_us = r->t_done;
    if (r->status == STRIDE_OK && r->launch) {
        Launch* l = r->launch.get();
        const uint64_t pos_off = up(12ull * l->total_t);
        out->d_idx = reinterpret_cast<const uint32_t*>(s->d_arena + l->out_off) + 3ull * r->t_rel;
        out->d_pos = reinterpret_cast<const float*>(s->d_arena + l->out_off + pos_off) + 3ull * r->v_rel;
        if (l->host.ptr) {
            out->h_idx = reinterpret_cast<const uint32_t*>(l->host.ptr) + 3ull * r->t_rel;
            out->h_pos = reinterpret_cast<const float*>(l->host.ptr + pos_off) + 3ull * r->v_rel;
        }
    }
    return STRIDE_OK;
}

int stride_server_release(stride_server* s, uint64_t req_id) {
    if (!s) return fail(STRIDE_ERR_ARG, "null server");
    {
        std::lock_guard<std::mutex> g(s->mu);
        auto it = s->reqs.find(req_id);
        if (it == s->reqs.end())
            return fail(STRIDE_ERR_ARG, "unknown request %llu", static_cast<unsigned long long>(req_id));
        Request* r = it->second.get();
        if (r->state != Request::kDone) return fail(STRIDE_ERR_BUSY, "request still queued or running");
        if (r->launch) {
            Launch* l = r->launch.get();
            if (--l->live == 0) free_launch_outputs(s, l);
            r->launch.reset();
        }
        s->reqs.erase(it);
    }
    notify_scheduler(s);
    return STRIDE_OK;
}

int stride_server_hold(stride_server* s, int hold) {
    if (!s) return fail(STRIDE_ERR_ARG, "null server");
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->hold = hold != 0;
    }
    notify_scheduler(s);
    return STRIDE_OK;
}

int stride_server_stats(stride_server* s, uint64_t* launches, uint64_t* completed, uint64_t* arena_peak_bytes) {
    if (!s) return fail(STRIDE_ERR_ARG, "null server");
    std::lock_guard<std::mutex> g(s->mu);
    if (launches) *launches = s->launches;
    if (completed) *completed = s->completed;
    if (arena_peak_bytes) *arena_peak_bytes = s->arena.peak();
    return STRIDE_OK;
}

void stride_server_destroy(stride_server* s) {
    if (!s) return;
    s->stop.store(true);
    notify_scheduler(s);
    if (s->scheduler.joinable()) s->scheduler.join();
    for (Slot& sl : s->slots) {
        cudaStreamSynchronize(sl.stream);
        cudaStreamDestroy(sl.stream);
        cudaFreeHost(sl.h_status);
        if (sl.stage.ptr) cudaFreeHost(sl.stage.ptr);
    }
    for (auto& kv : s->reqs) {
        if (kv.second->launch && kv.second->launch->host.ptr) {
            cudaFreeHost(kv.second->launch->host.ptr);
            kv.second->launch->host = Pinned{};
        }
    }
    for (Pinned& p : s->pinned_pool) cudaFreeHost(p.ptr);
    cudaFreeHost(s->h_pay);
    cudaFree(s->d_arena);
    delete s;
}

}  // extern "C"
