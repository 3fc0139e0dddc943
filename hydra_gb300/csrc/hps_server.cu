// hps_server.cu -- request server with continuous batching over the batched persistent kernels.
//
// Host threads submit requests; one scheduler thread per server
//   1. retires finished launches (a host callback on the stream counts completions),
//   2. admits queued requests in arrival order while their output memory fits the budget,
//   3. builds the next launch from every admitted request that still has work -- store requests
//      in slices of at most slice_events events, AverageOn requests whole -- and enqueues it
//      (at most two launches in flight, on two plans used in turn),
//   4. sleeps until a submission, a release or a completed launch wakes it.
// A request's outputs are written by the same work units as hps_generate / hps_average_on at
// FP32_FIX, so they do not depend on the other requests in its launches.
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "common.h"

using namespace hps;

namespace {

double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

enum ReqState { kQueued = 0, kRunning = 1, kDone = 2, kCancelled = 3, kFailed = 4 };

struct Req {
    hps_request req{};
    ReqState state = kQueued;
    hps_status status = HPS_OK;
    uint64_t issued = 0;         // events handed to launches
    void* buf = nullptr;         // store outputs
    uint64_t bytes = 0;
    int slot = -1;               // AverageOn result slot
    double t_submit = 0, t_admit = 0, t_done = 0;
    hps_stats stats{0.0, 0.0, 0.0};
};

struct Launch {
    uint64_t seq = 0;                      // launch number; complete when completed_ >= seq
    std::vector<hps_ticket> finishing;     // requests whose last work is in this launch
};

uint64_t store_bytes(const hps_request& r)
{
    const uint64_t n = r.n_events;
    const uint64_t b = n * 32ull * (uint64_t)r.channel.n_daughters + n * 8ull + (r.want_flags ? n : 0ull);
    return (b + 255) / 256 * 256;
}

}  // namespace

struct hps_server {
    hps_server_config cfg{};
    int device = 0;
    std::mutex mu;
    std::condition_variable cv_sched;
    std::condition_variable cv_done;
    std::deque<hps_ticket> pending;
    std::unordered_map<hps_ticket, Req> reqs;
    std::vector<hps_ticket> active;        // admitted, with events not yet handed to a launch
    hps_ticket next_ticket = 1;
    hps_server_stats st{};
    cudaStream_t stream = nullptr;
    hps_batch_plan* plans[2] = {nullptr, nullptr};
    int next_plan = 0;
    std::deque<Launch> inflight;
    std::deque<hps_ticket> finished;       // completion queue for hps_server_next_done
    uint64_t launched = 0;
    std::atomic<uint64_t> completed{0};
    hps_stats* slots_host = nullptr;       // pinned, mapped: AverageOn results land here
    hps_stats* slots_dev = nullptr;
    std::vector<int> free_slots;
    int allocs = 0;
    bool stop = false;
    uint64_t wake_gen = 0;                 // bumped by submit / cancel / release / destroy
    hps_status fatal = HPS_OK;
    char fatal_msg[256] = "";
    std::thread thread;
};

namespace {

// Runs on the CUDA callback thread after a launch; takes no lock (the scheduler may hold the
// server lock while it enqueues work), so a wake-up that races the scheduler's predicate check
// is caught by its short timed wait instead.
void CUDART_CB on_launch_done(void* p)
{
    hps_server* s = static_cast<hps_server*>(p);
    s->completed.fetch_add(1, std::memory_order_release);
    s->cv_sched.notify_all();
}

void fail_request(hps_server* s, hps_ticket t, Req& r, hps_status status)
{
    r.state = kFailed;
    r.status = status;
    r.t_done = now_s();
    s->st.failed++;
    s->finished.push_back(t);
}

// Called with the lock held.
void retire(hps_server* s)
{
    const uint64_t done = s->completed.load(std::memory_order_acquire);
    bool any = false;
    while (!s->inflight.empty() && s->inflight.front().seq <= done) {
        for (hps_ticket t : s->inflight.front().finishing) {
            auto it = s->reqs.find(t);
            if (it == s->reqs.end()) continue;
            Req& r = it->second;
            if (r.state != kRunning) continue;
            if (r.req.mode == HPS_MODE_AVERAGE) {
                r.stats = s->slots_host[r.slot];
                s->free_slots.push_back(r.slot);
                r.slot = -1;
            }
            r.state = kDone;
            r.t_done = now_s();
            s->st.completed++;
            s->st.events_done += r.req.n_events;
            s->finished.push_back(t);
        }
        s->inflight.pop_front();
        any = true;
    }
    if (any) s->cv_done.notify_all();
}

// Called with the lock held.
void admit(hps_server* s)
{
    while (!s->pending.empty()) {
        const hps_ticket t = s->pending.front();
        auto it = s->reqs.find(t);
        if (it == s->reqs.end() || it->second.state != kQueued) {
            s->pending.pop_front();
            continue;
        }
        Req& r = it->second;
        if (r.req.mode == HPS_MODE_AVERAGE) {
            if (s->free_slots.empty()) break;
            r.slot = s->free_slots.back();
            s->free_slots.pop_back();
        } else {
            const uint64_t need = store_bytes(r.req);
            if (s->st.bytes_in_use + need > s->cfg.budget_bytes) break;   // first in, first admitted
            ++s->allocs;
            cudaError_t e = cudaSuccess;
            if (s->cfg.fail_alloc_after > 0 && s->allocs == s->cfg.fail_alloc_after) {
                e = cudaErrorMemoryAllocation;          // injected failure (test hook)
            } else {
                e = cudaMallocAsync(&r.buf, need, s->stream);
            }
            if (e != cudaSuccess) {
                cudaGetLastError();
                r.buf = nullptr;
                s->pending.pop_front();
                fail_request(s, t, r, HPS_ERR_OOM);
                s->cv_done.notify_all();
                continue;
            }
            r.bytes = need;
            s->st.bytes_in_use += need;
            if (s->st.bytes_in_use > s->st.bytes_peak) s->st.bytes_peak = s->st.bytes_in_use;
        }
        r.state = kRunning;
        r.t_admit = now_s();
        s->st.admitted++;
        s->active.push_back(t);
        s->pending.pop_front();
    }
}

void fill_result(const Req& r, hps_result* out)
{
    std::memset(out, 0, sizeof(*out));
    out->status = (r.state == kCancelled) ? HPS_ERR_BAD_ARG : r.status;
    out->mode = r.req.mode;
    out->n_events = r.req.n_events;
    out->t_submit = r.t_submit;
    out->t_admit = r.t_admit;
    out->t_done = r.t_done;
    if (r.req.mode == HPS_MODE_STORE && r.buf) {
        const uint64_t n = r.req.n_events;
        char* base = static_cast<char*>(r.buf);
        for (int k = 0; k < r.req.channel.n_daughters; ++k)
            out->cols[k] = reinterpret_cast<double*>(base + (uint64_t)k * n * 32);
        out->weights = reinterpret_cast<double*>(base + (uint64_t)r.req.channel.n_daughters * n * 32);
        if (r.req.want_flags)
            out->flags = reinterpret_cast<uint8_t*>(base + (uint64_t)r.req.channel.n_daughters * n * 32 + n * 8);
    }
    out->stats = r.stats;
}

// Builds and enqueues one launch from the admitted requests; false if there was nothing to
// launch.  Called with the lock held.
bool launch(hps_server* s)
{
    std::vector<hps_batch_item> items;
    Launch L;
    uint64_t avg_events = 0;
    std::vector<hps_ticket> still;
    for (hps_ticket t : s->active) {
        Req& r = s->reqs[t];
        const bool room = (int)items.size() < s->cfg.max_batch_items;
        const uint64_t remaining = r.req.n_events - r.issued;
        if (!room || remaining == 0) {
            if (remaining > 0) still.push_back(t);
            continue;
        }
        hps_batch_item it;
        std::memset(&it, 0, sizeof(it));
        it.channel = r.req.channel;
        it.mode = r.req.mode;
        if (r.req.mode == HPS_MODE_AVERAGE) {
            if (avg_events + r.req.n_events > s->cfg.max_average_events) {
                still.push_back(t);                  // next launch
                continue;
            }
            avg_events += r.req.n_events;
            it.first_evt = r.req.first_evt;
            it.n_events = r.req.n_events;
            it.functor = r.req.functor;
            it.stats = s->slots_dev + r.slot;
            r.issued = r.req.n_events;
        } else {
            const uint64_t n = r.req.n_events;
            const uint64_t m = remaining < s->cfg.slice_events ? remaining : s->cfg.slice_events;
            char* base = static_cast<char*>(r.buf);
            it.first_evt = r.req.first_evt + r.issued;
            it.n_events = m;
            for (int k = 0; k < r.req.channel.n_daughters; ++k)
                it.cols[k] = reinterpret_cast<double*>(base + (uint64_t)k * n * 32 + r.issued * 32);
            it.weights = reinterpret_cast<double*>(base + (uint64_t)r.req.channel.n_daughters * n * 32 + r.issued * 8);
            if (r.req.want_flags)
                it.flags = reinterpret_cast<uint8_t*>(base + (uint64_t)r.req.channel.n_daughters * n * 32 + n * 8 +
                                                      r.issued);
            it.unweight_seed = r.req.unweight_seed;
            r.issued += m;
        }
        items.push_back(it);
        if (r.issued == r.req.n_events) L.finishing.push_back(t);
        else still.push_back(t);
    }
    if (items.empty()) return false;
    s->active.swap(still);
    hps_batch_plan* plan = s->plans[s->next_plan];
    s->next_plan ^= 1;
    hps_status stt = hps_batch_set_items(plan, items.data(), (int32_t)items.size(), s->stream);
    if (stt == HPS_OK) stt = hps_batch_launch(plan, s->stream);
    if (stt == HPS_OK) {
        cudaError_t e = cudaLaunchHostFunc(s->stream, on_launch_done, s);
        if (e != cudaSuccess) stt = cuda_status(e, "cudaLaunchHostFunc");
    }
    if (stt != HPS_OK) {
        // the server cannot make progress: fail everything that is not finished
        s->fatal = stt;
        std::snprintf(s->fatal_msg, sizeof(s->fatal_msg), "%s", hps_last_error());
        for (auto& kv : s->reqs)
            if (kv.second.state == kRunning || kv.second.state == kQueued) fail_request(s, kv.first, kv.second, stt);
        s->active.clear();
        s->pending.clear();
        s->cv_done.notify_all();
        return false;
    }
    L.seq = ++s->launched;
    s->st.launches++;
    s->inflight.push_back(std::move(L));
    return true;
}

void scheduler(hps_server* s)
{
    cudaSetDevice(s->device);
    std::unique_lock<std::mutex> lock(s->mu);
    for (;;) {
        retire(s);
        bool launched = false;
        if (s->stop) {
            if (s->inflight.empty()) break;
        } else if (s->fatal == HPS_OK) {
            admit(s);
            if (s->inflight.size() < 2 && !s->active.empty()) launched = launch(s);
        }
        if (launched) continue;
        // Sleep until something can change: a launch completes, or a request is submitted,
        // cancelled or released (a queued request blocked by the budget waits for a release).
        // The timed wait also covers a completion whose notify raced this check.
        const uint64_t seen = s->completed.load(std::memory_order_acquire);
        const uint64_t gen = s->wake_gen;
        s->cv_sched.wait_for(lock, std::chrono::microseconds(200), [&] {
            return s->stop || s->completed.load(std::memory_order_acquire) != seen || s->wake_gen != gen;
        });
    }
}

}  // namespace

extern "C" {

hps_status hps_server_create(hps_server** out, const hps_server_config* cfg)
{
    HPS_ENTRY();
    if (!out || !cfg) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    *out = nullptr;
    if (cfg->budget_bytes == 0) return set_error(HPS_ERR_BAD_ARG, "budget_bytes is 0");
    hps_server* s = new hps_server();
    s->cfg = *cfg;
    if (!s->cfg.slice_events) s->cfg.slice_events = 1ull << 22;
    if (s->cfg.max_batch_items <= 0) s->cfg.max_batch_items = 1024;
    if (s->cfg.max_inflight <= 0) s->cfg.max_inflight = 4096;
    if (!s->cfg.max_average_events) s->cfg.max_average_events = 1ull << 30;
    s->cfg.slice_events = (s->cfg.slice_events + 255) / 256 * 256;
    cudaError_t e = cudaGetDevice(&s->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess)
        e = cudaHostAlloc(&s->slots_host, sizeof(hps_stats) * s->cfg.max_inflight, cudaHostAllocMapped);
    if (e == cudaSuccess) e = cudaHostGetDevicePointer(reinterpret_cast<void**>(&s->slots_dev), s->slots_host, 0);
    hps_status st = cuda_status(e, "server set-up");
    const uint64_t avg_tiles = (s->cfg.max_average_events + HPS_AVG_TILE - 1) / HPS_AVG_TILE + 1;
    for (int i = 0; i < 2 && st == HPS_OK; ++i)
        st = hps_batch_create(&s->plans[i], s->cfg.max_batch_items, avg_tiles, HPS_PREC_FP32_FIX, nullptr);
    if (st != HPS_OK) {
        for (int i = 0; i < 2; ++i) hps_batch_destroy(s->plans[i]);
        if (s->slots_host) cudaFreeHost(s->slots_host);
        if (s->stream) cudaStreamDestroy(s->stream);
        delete s;
        return st;
    }
    for (int i = s->cfg.max_inflight - 1; i >= 0; --i) s->free_slots.push_back(i);
    s->thread = std::thread(scheduler, s);
    *out = s;
    return HPS_OK;
}

hps_status hps_server_submit(hps_server* s, const hps_request* req, hps_ticket* ticket)
{
    HPS_ENTRY();
    if (!s || !req || !ticket) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    DevChannel dc;
    hps_status st = to_device_channel(&req->channel, &dc);
    if (st != HPS_OK) return st;
    if (req->mode != HPS_MODE_STORE && req->mode != HPS_MODE_AVERAGE)
        return set_error(HPS_ERR_BAD_ARG, "unknown mode %d", req->mode);
    if (!range_ok(req->first_evt, req->n_events)) return set_error(HPS_ERR_BAD_ARG, "event range wraps 2^64");
    if (req->mode == HPS_MODE_AVERAGE) {
        DevFunctor f;
        if ((st = to_device_functor(&req->functor, req->channel.n_daughters, &f)) != HPS_OK) return st;
        if (req->n_events > s->cfg.max_average_events)
            return set_error(HPS_ERR_BUDGET, "AverageOn of %llu events exceeds the per-launch limit %llu",
                             (unsigned long long)req->n_events, (unsigned long long)s->cfg.max_average_events);
    } else if (store_bytes(*req) > s->cfg.budget_bytes) {
        return set_error(HPS_ERR_BUDGET, "request needs %llu bytes, budget is %llu",
                         (unsigned long long)store_bytes(*req), (unsigned long long)s->cfg.budget_bytes);
    }
    std::lock_guard<std::mutex> lock(s->mu);
    if (s->fatal != HPS_OK) return set_error(s->fatal, "server stopped: %s", s->fatal_msg);
    if (s->stop) return set_error(HPS_ERR_BAD_ARG, "server is shutting down");
    const hps_ticket t = s->next_ticket++;
    Req& r = s->reqs[t];
    r.req = *req;
    r.t_submit = now_s();
    s->pending.push_back(t);
    s->st.submitted++;
    *ticket = t;
    s->wake_gen++;
    s->cv_sched.notify_all();
    return HPS_OK;
}

hps_status hps_server_poll(hps_server* s, hps_ticket t, hps_result* result, int32_t* done)
{
    HPS_ENTRY();
    if (!s || !done) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(t);
    if (it == s->reqs.end()) return set_error(HPS_ERR_BAD_ARG, "unknown ticket %llu", (unsigned long long)t);
    const Req& r = it->second;
    *done = (r.state == kDone || r.state == kFailed || r.state == kCancelled) ? 1 : 0;
    if (*done && result) fill_result(r, result);
    return HPS_OK;
}

hps_status hps_server_wait(hps_server* s, hps_ticket t, hps_result* result, double timeout_s)
{
    HPS_ENTRY();
    if (!s) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    std::unique_lock<std::mutex> lock(s->mu);
    auto finished = [&] {
        auto it = s->reqs.find(t);
        if (it == s->reqs.end()) return true;
        const ReqState stt = it->second.state;
        return stt == kDone || stt == kFailed || stt == kCancelled;
    };
    const auto deadline = std::chrono::steady_clock::now() +
                          std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                              std::chrono::duration<double>(timeout_s < 0 ? 0 : timeout_s));
    if (!s->cv_done.wait_until(lock, deadline, finished))
        return set_error(HPS_ERR_TIMEOUT, "request %llu still running after %.3f s", (unsigned long long)t, timeout_s);
    auto it = s->reqs.find(t);
    if (it == s->reqs.end()) return set_error(HPS_ERR_BAD_ARG, "unknown ticket %llu", (unsigned long long)t);
    if (result) fill_result(it->second, result);
    return HPS_OK;
}

hps_status hps_server_cancel(hps_server* s, hps_ticket t)
{
    HPS_ENTRY();
    if (!s) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(t);
    if (it == s->reqs.end()) return set_error(HPS_ERR_BAD_ARG, "unknown ticket %llu", (unsigned long long)t);
    Req& r = it->second;
    if (r.state != kQueued) return set_error(HPS_ERR_BAD_ARG, "request %llu is not queued", (unsigned long long)t);
    r.state = kCancelled;
    r.t_done = now_s();
    s->st.cancelled++;
    s->finished.push_back(t);
    s->wake_gen++;
    s->cv_done.notify_all();
    s->cv_sched.notify_all();
    return HPS_OK;
}

hps_status hps_server_next_done(hps_server* s, hps_ticket* ticket, hps_result* result, double timeout_s)
{
    HPS_ENTRY();
    if (!s || !ticket) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    std::unique_lock<std::mutex> lock(s->mu);
    const auto deadline = std::chrono::steady_clock::now() +
                          std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                              std::chrono::duration<double>(timeout_s < 0 ? 0 : timeout_s));
    for (;;) {
        while (!s->finished.empty()) {
            const hps_ticket t = s->finished.front();
            s->finished.pop_front();
            auto it = s->reqs.find(t);
            if (it == s->reqs.end()) continue;          // released already
            *ticket = t;
            if (result) fill_result(it->second, result);
            return HPS_OK;
        }
        if (s->cv_done.wait_until(lock, deadline) == std::cv_status::timeout && s->finished.empty())
            return set_error(HPS_ERR_TIMEOUT, "no request finished within %.3f s", timeout_s);
    }
}

hps_status hps_server_release(hps_server* s, hps_ticket t)
{
    HPS_ENTRY();
    if (!s) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    std::lock_guard<std::mutex> lock(s->mu);
    auto it = s->reqs.find(t);
    if (it == s->reqs.end()) return set_error(HPS_ERR_BAD_ARG, "unknown ticket %llu", (unsigned long long)t);
    Req& r = it->second;
    if (r.state == kQueued || r.state == kRunning)
        return set_error(HPS_ERR_BAD_ARG, "request %llu has not finished", (unsigned long long)t);
    if (r.buf) {
        cudaError_t e = cudaFreeAsync(r.buf, s->stream);
        r.buf = nullptr;
        if (e != cudaSuccess) return cuda_status(e, "cudaFreeAsync");
    }
    s->st.bytes_in_use -= r.bytes;
    if (r.slot >= 0) s->free_slots.push_back(r.slot);
    s->reqs.erase(it);
    s->st.released++;
    s->wake_gen++;
    s->cv_sched.notify_all();
    return HPS_OK;
}

hps_status hps_server_get_stats(hps_server* s, hps_server_stats* out)
{
    HPS_ENTRY();
    if (!s || !out) return set_error(HPS_ERR_BAD_ARG, "NULL argument");
    std::lock_guard<std::mutex> lock(s->mu);
    *out = s->st;
    return HPS_OK;
}

hps_status hps_server_destroy(hps_server* s)
{
    if (!s) return HPS_OK;
    {
        std::lock_guard<std::mutex> lock(s->mu);
        s->stop = true;
        for (hps_ticket t : s->pending) {
            auto it = s->reqs.find(t);
            if (it != s->reqs.end() && it->second.state == kQueued) {
                it->second.state = kCancelled;
                s->st.cancelled++;
            }
        }
        s->pending.clear();
        s->wake_gen++;
        s->cv_sched.notify_all();
        s->cv_done.notify_all();
    }
    if (s->thread.joinable()) s->thread.join();
    cudaStreamSynchronize(s->stream);
    for (auto& kv : s->reqs)
        if (kv.second.buf) cudaFreeAsync(kv.second.buf, s->stream);
    cudaStreamSynchronize(s->stream);
    for (int i = 0; i < 2; ++i) hps_batch_destroy(s->plans[i]);
    if (s->slots_host) cudaFreeHost(s->slots_host);
    cudaStreamDestroy(s->stream);
    delete s;
    return HPS_OK;
}

}  // extern "C"
