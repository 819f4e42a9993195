// ifx_serve.cu -- the serving loop: continuous batching of filter requests.
//
// Requests arrive through ifx_server_submit at any time.  One engine thread
//   1. admits queued requests in arrival order while the device bytes they
//      need (staged input, outputs) fit under the HBM cap and in the device's
//      available memory (free memory plus the pool's unused part, less a
//      reserve: a shared device may have less than the cap); device memory
//      comes from the stream-ordered allocator and host images are uploaded
//      on a copy stream as soon as a request is admitted;
//   2. while fewer than `max_inflight` batches run, packs admitted requests
//      into one batched launch (the persistent tile work-queue kernel of
//      ifx_batch.cu) on the compute stream, which waits for the uploads of
//      that batch's requests only; after an idle period the first batches
//      are smaller (1/8, 1/4, 1/2 of max_batch), so that results start
//      flowing back over the link early;
//   3. queues, with each batch, the copies of its host outputs on a download
//      stream behind the batch's kernel (the link's two directions overlap)
//      and the release of its requests' device memory after those copies;
//   4. records submit -> done latency of every request.
// Requests admitted while other batches run overlap with them on the device:
// uploads of batch k+1 run on the copy stream during batch k.
#include "ifx_internal.h"
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

namespace ifx {

using Clock = std::chrono::steady_clock;

struct SReq {
    uint64_t ticket = 0;
    ifx_request_t q{};
    std::vector<double> w0, w1;             // owned copies of the weights
    bool host_in = false, host_out[2] = {false, false};
    void *d_in = nullptr, *d_out[2] = {nullptr, nullptr};
    size_t in_bytes = 0, out_bytes[2] = {0, 0};
    int64_t need = 0;                      // device bytes held while in flight
    long long pixels = 0;
    Clock::time_point t_submit;
    int status = IFX_OK;
    bool done = false;
    BatchItem item{};                      // validated form (fill values)
    cudaEvent_t staged_ev = nullptr;       // after this request's allocations and upload (copy stream)
};

struct SBatch {
    std::vector<std::shared_ptr<SReq>> reqs;
    cudaEvent_t compute_done = nullptr, copy_done = nullptr;
};

} // namespace ifx

struct ifx_server {
    ifx_context_t *ctx = nullptr;
    int device = 0;
    ifx_server_config_t cfg{};
    cudaStream_t copy = nullptr, compute = nullptr;   // copy: uploads; compute: batches
    cudaStream_t down = nullptr;                        // downloads and releases
    uint64_t deferred_free = 0;                         // admissions held back by free device memory
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<std::shared_ptr<ifx::SReq>> incoming;           // submitted, not seen by the engine
    std::deque<std::shared_ptr<ifx::SReq>> queue;              // waiting for admission
    std::vector<std::shared_ptr<ifx::SReq>> staged;            // admitted, not yet in a batch
    std::deque<ifx::SBatch> inflight;
    std::unordered_map<uint64_t, std::shared_ptr<ifx::SReq>> by_ticket;
    std::vector<double> latencies;
    uint64_t next_ticket = 1, submitted = 0, completed = 0, failed = 0, batches = 0;
    int ramp = 0;                          // batches launched since the engine was last idle
    int inject_fail = 0;                   // launches still to report as failed (host-side injection)
    bool paused = false;                   // admission goes on, no new batches launch
    long long pixels = 0;
    int64_t hbm_in_use = 0, hbm_peak = 0;
    bool have_first = false;
    ifx::Clock::time_point first_submit, last_done;
    std::atomic<bool> stop{false};
    std::thread engine;
    std::string engine_error;
};

namespace ifx {

static size_t bytes_of(const ifx_array_t &a)
{
    size_t e = a.eltype == IFX_F64 ? 8 : a.eltype == IFX_F32 ? 4 : a.eltype == IFX_I16 ? 2 : 1;
    size_t n = 1;
    for (int d = 0; d < a.ndim; ++d) n *= (size_t)a.size[d];
    return n * e;
}

static bool dev_ptr(const void *p)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        (void)cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

static int nouts(const ifx_request_t &q) { return q.op == IFX_OP_GRADIENTS2D ? 2 : 1; }

// Queues a launched batch's downloads and releases on the download stream,
// behind the batch's kernel (srv->mu held).  They are queued when the batch is
// launched, so the copies start as soon as the kernel ends, whatever the
// engine thread is doing then.
static void enqueue_downloads(ifx_server *S, SBatch &b)
{
    cudaStreamWaitEvent(S->down, b.compute_done, 0);
    for (auto &r : b.reqs)
        for (int o = 0; o < nouts(r->q) && r->status == IFX_OK; ++o)
            if (r->host_out[o])
                cudaMemcpyAsync(r->q.out[o].data, r->d_out[o], r->out_bytes[o], cudaMemcpyDeviceToHost, S->down);
    for (auto &r : b.reqs) {
        if (r->host_in && r->d_in) cudaFreeAsync(r->d_in, S->down);
        for (int o = 0; o < 2; ++o)
            if (r->host_out[o] && r->d_out[o]) cudaFreeAsync(r->d_out[o], S->down);
    }
    cudaEventRecord(b.copy_done, S->down);
}

// Called with srv->mu held: move batches whose downloads have finished to done.
static void finish_batches(ifx_server *S)
{
    while (!S->inflight.empty()) {
        SBatch &b = S->inflight.front();
        if (cudaEventQuery(b.copy_done) == cudaErrorNotReady) return;
        const auto now = Clock::now();
        for (auto &r : b.reqs) {
            r->done = true;
            S->hbm_in_use -= r->need;
            if (r->status != IFX_OK) {            // a failed launch: no outputs, no latency sample
                ++S->failed;
                continue;
            }
            S->latencies.push_back(std::chrono::duration<double>(now - r->t_submit).count());
            S->pixels += r->pixels;
            ++S->completed;
        }
        S->last_done = now;
        cudaEventDestroy(b.compute_done);
        cudaEventDestroy(b.copy_done);
        S->inflight.pop_front();
        S->cv_done.notify_all();
    }
}

// Device memory the server can still take: the device's free memory plus what
// its stream-ordered pool holds but does not use, less a reserve kept for
// other users of the device and for the library's own buffers.
constexpr size_t kFreeReserve = 256ull << 20;

static size_t device_available(const ifx_server *S)
{
    size_t free_b = 0, total_b = 0;
    if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) {
        (void)cudaGetLastError();
        return SIZE_MAX;                     // no answer: the cap alone decides
    }
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, S->device) == cudaSuccess) {
        uint64_t reserved = 0, used = 0;
        if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved) == cudaSuccess &&
            cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &used) == cudaSuccess && reserved > used)
            free_b += (size_t)(reserved - used);
    }
    (void)cudaGetLastError();
    return free_b > kFreeReserve ? free_b - kFreeReserve : 0;
}

// Admission in arrival order while a request fits both the HBM cap and the
// device's available memory (srv->mu held).  With nothing admitted a request
// is admitted anyway: waiting could not free any memory of this server, and
// an allocation failure then fails that request alone.
static void admit(ifx_server *S)
{
    size_t avail = 0;
    bool have_avail = false;
    while (!S->queue.empty()) {
        auto r = S->queue.front();
        if (S->hbm_in_use > 0) {
            if (S->hbm_in_use + r->need > S->cfg.hbm_cap_bytes) return;
            if (!have_avail) {
                avail = device_available(S);
                have_avail = true;
            }
            if (r->need > avail) {
                ++S->deferred_free;
                return;
            }
            avail -= r->need;
        }
        bool ok = true;
        if (r->host_in) {
            ok &= cudaMallocAsync(&r->d_in, r->in_bytes, S->copy) == cudaSuccess;
            if (ok) ok &= cudaMemcpyAsync(r->d_in, r->q.img.data, r->in_bytes, cudaMemcpyHostToDevice,
                                          S->copy) == cudaSuccess;
        } else {
            r->d_in = r->q.img.data;
        }
        for (int o = 0; o < nouts(r->q) && ok; ++o) {
            if (r->host_out[o]) ok &= cudaMallocAsync(&r->d_out[o], r->out_bytes[o], S->copy) == cudaSuccess;
            else r->d_out[o] = r->q.out[o].data;
        }
        S->queue.pop_front();
        if (ok && (r->host_in || r->host_out[0] || r->host_out[1])) {
            // the batch that takes this request waits for this point of the copy stream only
            ok &= cudaEventCreateWithFlags(&r->staged_ev, cudaEventDisableTiming) == cudaSuccess;
            if (ok) ok &= cudaEventRecord(r->staged_ev, S->copy) == cudaSuccess;
        }
        if (!ok) {
            (void)cudaGetLastError();
            if (r->staged_ev) {
                cudaEventDestroy(r->staged_ev);
                r->staged_ev = nullptr;
            }
            r->status = IFX_ERR_NOMEM;
            r->done = true;
            ++S->failed;
            S->cv_done.notify_all();
            continue;
        }
        S->hbm_in_use += r->need;
        S->hbm_peak = std::max(S->hbm_peak, S->hbm_in_use);
        S->staged.push_back(r);
    }
}

// Launch one batch of staged requests (srv->mu held).
static void launch(ifx_server *S)
{
    if (S->paused || S->staged.empty() || (int)S->inflight.size() >= S->cfg.max_inflight) return;
    IFX_RANGE("ifx_server_launch_batch");
    // Ramp: after an idle engine the first batches are 1/8, 1/4, 1/2 of max_batch, so
    // that the first results reach the download stream early (a served stream is
    // bound by the host link, and the link's download direction idles until then).
    const size_t cap = std::max<size_t>(std::min<size_t>(16, (size_t)S->cfg.max_batch),
                                        (size_t)S->cfg.max_batch >> std::max(0, 3 - S->ramp));
    const size_t n = std::min(S->staged.size(), cap);
    ++S->ramp;
    SBatch b;
    b.reqs.assign(S->staged.begin(), S->staged.begin() + n);
    S->staged.erase(S->staged.begin(), S->staged.begin() + n);
    // wait for the copy-stream work of this batch's requests only: uploads are in
    // admission order, so the last request's event covers the earlier ones
    cudaEvent_t last = nullptr;
    for (auto &r : b.reqs)
        if (r->staged_ev) last = r->staged_ev;
    if (last) cudaStreamWaitEvent(S->compute, last, 0);
    for (auto &r : b.reqs)
        if (r->staged_ev) {
            cudaEventDestroy(r->staged_ev);                 // released once it has completed
            r->staged_ev = nullptr;
        }
    std::vector<BatchItem> items(n);
    for (size_t i = 0; i < n; ++i) {
        const SReq &r = *b.reqs[i];
        const ifx_request_t &q = r.q;
        BatchItem &it = items[i];
        memset(&it, 0, sizeof it);
        it.op = q.op;
        it.in_type = q.img.eltype;
        it.out_type = q.out[0].eltype;
        it.style = q.border.style;
        it.nx = (int)q.img.size[0];
        it.ny = (int)q.img.size[1];
        it.window = q.window;
        it.in = r.d_in;
        it.out0 = r.d_out[0];
        it.out1 = r.d_out[1];
        it.fill_code = r.item.fill_code;
        it.fill = r.item.fill;
        it.kx = q.taps[0];
        it.ky = q.taps[1];
        it.fx = (int)q.first[0];
        it.fy = (int)q.first[1];
        it.wx = r.w0.empty() ? nullptr : r.w0.data();
        it.wy = r.w1.empty() ? nullptr : r.w1.data();
    }
    cudaEventCreateWithFlags(&b.compute_done, cudaEventDisableTiming);
    cudaEventCreateWithFlags(&b.copy_done, cudaEventDisableTiming);
    long long tiles = 0;
    cudaError_t e;
    if (S->inject_fail > 0) {                     // injected on the host: the kernel never runs
        --S->inject_fail;
        e = cudaErrorLaunchFailure;
    } else {
        e = launch_batch(S->device, items.data(), (int)n, S->compute, &tiles);
    }
    if (e != cudaSuccess) {
        S->engine_error = cudaGetErrorString(e);
        for (auto &r : b.reqs) r->status = IFX_ERR_CUDA;
    }
    cudaEventRecord(b.compute_done, S->compute);
    enqueue_downloads(S, b);
    ++S->batches;
    S->inflight.push_back(std::move(b));
}

static void engine_loop(ifx_server *S)
{
    cudaSetDevice(S->device);
    std::unique_lock<std::mutex> lk(S->mu);
    while (!S->stop.load()) {
        while (!S->incoming.empty()) {
            S->queue.push_back(S->incoming.front());
            S->incoming.pop_front();
        }
        finish_batches(S);
        admit(S);
        launch(S);
        const bool idle = S->incoming.empty() && S->queue.empty() && S->staged.empty() &&
                          S->inflight.empty();
        if (idle) S->ramp = 0;
        if (idle) S->cv_work.wait_for(lk, std::chrono::milliseconds(5));
        else {
            lk.unlock();
            std::this_thread::sleep_for(std::chrono::microseconds(20));
            lk.lock();
        }
    }
}

} // namespace ifx

using namespace ifx;

extern "C" {

int ifx_server_create(ifx_context_t *ctx, const ifx_server_config_t *cfg, ifx_server_t **out)
{
    IFX_RANGE("ifx_server_create");
    if (!ctx || !cfg || !out) return set_error(IFX_ERR_ARGUMENT, "NULL argument");
    if (cfg->hbm_cap_bytes <= 0 || cfg->max_batch < 1 || cfg->max_inflight < 1)
        return set_error(IFX_ERR_ARGUMENT, "server config: cap, max_batch and max_inflight must be positive");
    auto *S = new ifx_server();
    S->ctx = ctx;
    S->cfg = *cfg;
    cudaGetDevice(&S->device);
    if (cudaStreamCreateWithFlags(&S->copy, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&S->down, cudaStreamNonBlocking) != cudaSuccess ||
        cudaStreamCreateWithFlags(&S->compute, cudaStreamNonBlocking) != cudaSuccess) {
        delete S;
        return IFX_ERR_CUDA;
    }
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, S->device) == cudaSuccess) {
        uint64_t keep = (uint64_t)cfg->hbm_cap_bytes;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    S->engine = std::thread(engine_loop, S);
    *out = S;
    return IFX_OK;
}

int ifx_server_submit(ifx_server_t *S, const ifx_request_t *q, uint64_t *ticket)
{
    IFX_RANGE("ifx_server_submit");
    if (!S || !q || !ticket) return IFX_ERR_ARGUMENT;
    // validate exactly as a batch would, then keep an owned copy
    BatchItem it;
    int rc = request_item(*q, 0, false, it);
    if (rc) return rc;
    auto r = std::make_shared<SReq>();
    r->q = *q;
    const int no = nouts(*q);
    if (q->op == IFX_OP_FACTORED2D || q->op == IFX_OP_GRADIENTS2D) {
        r->w0.assign(q->weights[0], q->weights[0] + q->taps[0]);
        r->w1.assign(q->weights[1], q->weights[1] + q->taps[1]);
        r->q.weights[0] = r->w0.data();
        r->q.weights[1] = r->w1.data();
    }
    r->host_in = !dev_ptr(q->img.data);
    r->in_bytes = bytes_of(q->img);
    r->need = r->host_in ? (int64_t)r->in_bytes : 0;
    for (int o = 0; o < no; ++o) {
        r->host_out[o] = !dev_ptr(q->out[o].data);
        r->out_bytes[o] = bytes_of(q->out[o]);
        if (r->host_out[o]) r->need += (int64_t)r->out_bytes[o];
    }
    r->pixels = (long long)q->img.size[0] * q->img.size[1];
    if (r->need > S->cfg.hbm_cap_bytes)
        return set_error(IFX_ERR_NOMEM, "request needs more device memory than the server's cap");
    r->item = it;
    r->t_submit = Clock::now();
    {
        std::lock_guard<std::mutex> lk(S->mu);
        r->ticket = S->next_ticket++;
        if (!S->have_first) {
            S->first_submit = r->t_submit;
            S->have_first = true;
        }
        S->by_ticket[r->ticket] = r;
        S->incoming.push_back(r);
        ++S->submitted;
    }
    S->cv_work.notify_one();
    *ticket = r->ticket;
    return IFX_OK;
}

int ifx_server_wait(ifx_server_t *S, uint64_t ticket, double timeout_s, int32_t *status)
{
    IFX_RANGE("ifx_server_wait");
    if (!S) return IFX_ERR_ARGUMENT;
    std::unique_lock<std::mutex> lk(S->mu);
    auto it = S->by_ticket.find(ticket);
    if (it == S->by_ticket.end()) return IFX_ERR_ARGUMENT;
    auto r = it->second;
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                          std::chrono::duration<double>(timeout_s));
    while (!r->done) {
        if (S->cv_done.wait_until(lk, until) == std::cv_status::timeout && !r->done)
            return IFX_ERR_TIMEOUT;
    }
    if (status) *status = r->status;
    S->by_ticket.erase(ticket);
    return IFX_OK;
}

int ifx_server_cancel(ifx_server_t *S, uint64_t ticket)
{
    IFX_RANGE("ifx_server_cancel");
    if (!S) return IFX_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    auto it = S->by_ticket.find(ticket);
    if (it == S->by_ticket.end()) return set_error(IFX_ERR_ARGUMENT, "unknown ticket");
    auto r = it->second;
    if (r->done) return set_error(IFX_ERR_ARGUMENT, "the request is done");
    auto drop = [&](auto &seq) {
        for (auto q = seq.begin(); q != seq.end(); ++q)
            if (q->get() == r.get()) {
                seq.erase(q);
                return true;
            }
        return false;
    };
    if (!drop(S->incoming) && !drop(S->queue)) {
        if (!drop(S->staged)) return set_error(IFX_ERR_ARGUMENT, "the request is already in a launched batch");
        // admitted: its device memory goes back once the copy stream has passed its uploads
        if (r->host_in && r->d_in) cudaFreeAsync(r->d_in, S->copy);
        for (int o = 0; o < 2; ++o)
            if (r->host_out[o] && r->d_out[o]) cudaFreeAsync(r->d_out[o], S->copy);
        if (r->staged_ev) {
            cudaEventDestroy(r->staged_ev);
            r->staged_ev = nullptr;
        }
        S->hbm_in_use -= r->need;
    }
    r->status = IFX_ERR_CANCELLED;
    r->done = true;
    ++S->failed;
    S->cv_done.notify_all();
    return IFX_OK;
}

int ifx_server_pause(ifx_server_t *S, int32_t paused)
{
    IFX_RANGE("ifx_server_pause");
    if (!S) return IFX_ERR_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(S->mu);
        S->paused = paused != 0;
    }
    S->cv_work.notify_one();
    return IFX_OK;
}

int ifx_server_inject_launch_error(ifx_server_t *S, int32_t count)
{
    IFX_RANGE("ifx_server_inject_launch_error");
    if (!S || count < 0) return IFX_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    S->inject_fail = count;
    return IFX_OK;
}

int ifx_server_drain(ifx_server_t *S, double timeout_s)
{
    IFX_RANGE("ifx_server_drain");
    if (!S) return IFX_ERR_ARGUMENT;
    std::unique_lock<std::mutex> lk(S->mu);
    const auto until = Clock::now() + std::chrono::duration_cast<Clock::duration>(
                                          std::chrono::duration<double>(timeout_s));
    while (S->completed + S->failed < S->submitted) {
        if (S->cv_done.wait_until(lk, until) == std::cv_status::timeout &&
            S->completed + S->failed < S->submitted)
            return IFX_ERR_TIMEOUT;
    }
    return IFX_OK;
}

int ifx_server_metrics(ifx_server_t *S, ifx_server_metrics_t *m)
{
    IFX_RANGE("ifx_server_metrics");
    if (!S || !m) return IFX_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    memset(m, 0, sizeof *m);
    m->submitted = S->submitted;
    m->completed = S->completed;
    m->failed = S->failed;
    m->pixels = (uint64_t)S->pixels;
    m->batches = S->batches;
    m->hbm_in_use = S->hbm_in_use;
    m->hbm_peak = S->hbm_peak;
    m->queue_depth = (int32_t)(S->incoming.size() + S->queue.size());
    m->deferred_free = S->deferred_free;
    if (!S->latencies.empty()) {
        std::vector<double> v = S->latencies;
        std::sort(v.begin(), v.end());
        auto pct = [&](double p) { return v[std::min(v.size() - 1, (size_t)(p * (v.size() - 1) + 0.5))]; };
        m->p50_latency_s = pct(0.50);
        m->p99_latency_s = pct(0.99);
        m->max_latency_s = v.back();
    }
    if (S->have_first && S->completed)
        m->busy_s = std::chrono::duration<double>(S->last_done - S->first_submit).count();
    return IFX_OK;
}

int ifx_server_reset_metrics(ifx_server_t *S)
{
    IFX_RANGE("ifx_server_reset_metrics");
    if (!S) return IFX_ERR_ARGUMENT;
    std::lock_guard<std::mutex> lk(S->mu);
    if (S->completed + S->failed != S->submitted) return IFX_ERR_ARGUMENT;
    S->latencies.clear();
    S->submitted = S->completed = S->failed = S->batches = 0;
    S->pixels = 0;
    S->hbm_peak = S->hbm_in_use;
    S->have_first = false;
    return IFX_OK;
}

int ifx_server_destroy(ifx_server_t *S)
{
    IFX_RANGE("ifx_server_destroy");
    if (!S) return IFX_OK;
    ifx_server_drain(S, 60.0);
    S->stop.store(true);
    S->cv_work.notify_all();
    if (S->engine.joinable()) S->engine.join();
    cudaStreamSynchronize(S->copy);
    cudaStreamSynchronize(S->down);
    cudaStreamSynchronize(S->compute);
    cudaStreamDestroy(S->copy);
    cudaStreamDestroy(S->down);
    cudaStreamDestroy(S->compute);
    // the pool kept freed request memory (up to the cap) for the next
    // admissions; with the server gone it goes back to the device
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, S->device) == cudaSuccess) {
        const uint64_t zero = 0;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, (void *)&zero);
        cudaMemPoolTrimTo(pool, 0);
    }
    (void)cudaGetLastError();
    delete S;
    return IFX_OK;
}

} // extern "C"
