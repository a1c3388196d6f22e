// Request loop (gbo_server_*): continuous admission of validity / motion / nearestK requests from many
// clients onto a fixed set of streams, bounded by a device arena (HBM footprint admission).
//
// One dispatcher thread owns all device work: it retires requests whose completion event has fired
// (freeing their stream slot and arena range), then admits pending requests in arrival order,
// skipping any that does not fit yet (or whose nearest-neighbour index is busy) so that small
// requests are not held behind a large one, copies inputs host->device, launches the library's
// kernels on the slot's stream, copies results device->host, and records an event.
//
// Host staging: submit() copies a request's inputs into a page-locked staging arena (on the caller's
// thread) when it has room, so that the dispatcher's copies are asynchronous DMA in both directions
// and never wait for a stream; results land in staging and are copied to the caller's arrays when the
// request retires. A request that finds no staging room uses the caller's arrays directly (a copy
// from or to pageable memory then blocks the dispatcher until it is done).
#include <algorithm>
#include <chrono>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include "../../include/gbompl.h"
#include <cuda_runtime.h>

namespace
{
using Clock = std::chrono::steady_clock;

// First-fit allocator over one device range, or one page-locked host range (256-byte granules).
class Arena
{
public:
    bool init(size_t bytes, bool host = false)
    {
        host_ = host;
        if ((host ? cudaHostAlloc((void **)&base_, bytes, cudaHostAllocDefault) : cudaMalloc(&base_, bytes)) !=
            cudaSuccess)
        {
            base_ = nullptr;
            return false;
        }
        size_ = bytes;
        free_[0] = bytes;
        return true;
    }
    ~Arena()
    {
        if (base_)
            host_ ? cudaFreeHost(base_) : cudaFree(base_);
    }
    long alloc(size_t bytes)
    {
        bytes = (bytes + 255) & ~size_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it)
            if (it->second >= bytes)
            {
                const size_t off = it->first, sz = it->second;
                free_.erase(it);
                if (sz > bytes)
                    free_[off + bytes] = sz - bytes;
                used_ += bytes;
                return (long)off;
            }
        return -1;
    }
    void release(size_t off, size_t bytes)
    {
        bytes = (bytes + 255) & ~size_t(255);
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first)
        {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin())
        {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first)
            {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    char *ptr(size_t off) const { return base_ + off; }
    size_t used() const { return used_; }
    size_t size() const { return size_; }

private:
    char *base_ = nullptr;
    bool host_ = false;
    size_t size_ = 0, used_ = 0;
    std::map<size_t, size_t> free_;
};

struct Job
{
    uint64_t ticket;
    gbo_request req;
    Clock::time_point submitted;
    size_t bytes = 0;
    long off = -1;
    long hoff = -1;  // host staging range (same layout as the device range), -1: none
    int slot = -1;
    cudaEvent_t done = nullptr;
    gbo_status status = GBO_OK;
    bool finished = false;
    double latency = 0.0;
    std::string error;
};

}  // namespace

namespace gbo
{
gbo_status internal_fail(gbo_status s, const char *msg);
gbo_status internal_request_dim(const gbo_request *r, int *dim);
}  // namespace gbo
using gbo::internal_request_dim;

struct gbo_server
{
    Arena arena;
    Arena staging;  // page-locked host copy of admitted requests' inputs and outputs (may be empty)
    std::vector<cudaEvent_t> slot_event;
    std::vector<cudaStream_t> streams;
    std::vector<Job *> slot_job;
    std::mutex mu;
    std::condition_variable cv_done, cv_work;
    std::deque<Job *> pending;
    std::unordered_map<uint64_t, Job *> jobs;
    std::unordered_set<const void *> busy_nn;
    uint64_t next_ticket = 1, submitted = 0, completed = 0;
    int inflight = 0, max_inflight = 0;
    bool stop = false;
    std::thread worker;
    int device = 0;

    void run();
    bool launch(Job *j);
};

static size_t pad256(size_t b)
{
    return (b + 255) & ~size_t(255);
}

// Byte offsets of a request's arrays inside its arena range (the host staging range uses the same
// layout): inputs first ([0, in_end)), then outputs ([out_begin, out_end)).
struct ReqLayout
{
    size_t in2 = 0, in_end = 0, ok = 0, fj = 0, nd = 0, idx = 0, dist = 0, out_begin = 0, out_end = 0;
};

static ReqLayout req_layout(const gbo_request &r, int dim)
{
    ReqLayout L;
    const size_t n = (size_t)r.n, rows = n * dim * sizeof(double);
    if (r.kind == GBO_REQ_VALIDITY)
    {
        L.in_end = rows;
        L.ok = L.out_begin = pad256(rows);
        L.out_end = L.ok + n;
    }
    else if (r.kind == GBO_REQ_MOTION)
    {
        L.in2 = pad256(rows);
        L.in_end = L.in2 + rows;
        L.fj = L.out_begin = L.in2 + pad256(rows);
        L.nd = L.fj + pad256(4 * n);
        L.ok = L.nd + pad256(4 * n);
        L.out_end = L.ok + n;
    }
    else
    {
        L.in_end = rows;
        L.idx = L.out_begin = pad256(rows);
        L.dist = L.idx + pad256(n * r.k * 8);
        L.out_end = L.dist + n * r.k * 8;
    }
    return L;
}

// Inputs into the job's staging range (caller's thread, before the job is queued).
static void stage_inputs(const gbo_request &r, int dim, char *h)
{
    const ReqLayout L = req_layout(r, dim);
    const size_t rows = (size_t)r.n * dim * sizeof(double);
    if (rows)
    {
        std::memcpy(h, r.states, rows);
        if (r.kind == GBO_REQ_MOTION)
            std::memcpy(h + L.in2, r.states2, rows);
    }
}

// Results from the job's staging range into the caller's arrays (dispatcher, at retirement).
static void unstage_outputs(const gbo_request &r, int dim, const char *h)
{
    const ReqLayout L = req_layout(r, dim);
    const size_t n = (size_t)r.n;
    if (r.kind == GBO_REQ_KNN)
    {
        std::memcpy(r.idx, h + L.idx, n * r.k * 8);
        if (r.dist)
            std::memcpy(r.dist, h + L.dist, n * r.k * 8);
        return;
    }
    std::memcpy(r.ok, h + L.ok, n);
    if (r.kind == GBO_REQ_MOTION)
    {
        if (r.first_j)
            std::memcpy(r.first_j, h + L.fj, 4 * n);
        if (r.nd)
            std::memcpy(r.nd, h + L.nd, 4 * n);
    }
}

bool gbo_server::launch(Job *j)
{
    const gbo_request &r = j->req;
    cudaStream_t st = streams[j->slot];
    int dim = 0;
    internal_request_dim(&r, &dim);
    const ReqLayout L = req_layout(r, dim);
    char *d = arena.ptr((size_t)j->off);
    char *h = j->hoff >= 0 ? staging.ptr((size_t)j->hoff) : nullptr;  // staged: pinned copies
    const size_t n = (size_t)r.n, rows = n * dim * sizeof(double);
    gbo_status s = GBO_OK;
    cudaMemcpyAsync(d, h ? h : (const char *)r.states, rows, cudaMemcpyHostToDevice, st);
    if (r.kind == GBO_REQ_VALIDITY)
    {
        s = gbo_is_valid(r.checker, (const double *)d, r.n, dim, GBO_LAYOUT_AOS, (uint8_t *)(d + L.ok), st);
        if (s == GBO_OK)
            cudaMemcpyAsync(h ? (void *)(h + L.ok) : (void *)r.ok, d + L.ok, n, cudaMemcpyDeviceToHost, st);
    }
    else if (r.kind == GBO_REQ_MOTION)
    {
        cudaMemcpyAsync(d + L.in2, h ? h + L.in2 : (const char *)r.states2, rows, cudaMemcpyHostToDevice, st);
        s = gbo_check_motion(r.checker, (const double *)d, (const double *)(d + L.in2), r.n, dim, GBO_LAYOUT_AOS,
                             r.schedule, (uint8_t *)(d + L.ok), (int32_t *)(d + L.fj), (int32_t *)(d + L.nd), st);
        if (s == GBO_OK)
        {
            if (h)  // one copy of the whole output block
                cudaMemcpyAsync(h + L.out_begin, d + L.out_begin, L.out_end - L.out_begin, cudaMemcpyDeviceToHost,
                                st);
            else
            {
                cudaMemcpyAsync(r.ok, d + L.ok, n, cudaMemcpyDeviceToHost, st);
                if (r.first_j)
                    cudaMemcpyAsync(r.first_j, d + L.fj, 4 * n, cudaMemcpyDeviceToHost, st);
                if (r.nd)
                    cudaMemcpyAsync(r.nd, d + L.nd, 4 * n, cudaMemcpyDeviceToHost, st);
            }
        }
    }
    else
    {
        s = gbo_nn_nearest_k(r.nn, (const double *)d, r.n, dim, GBO_LAYOUT_AOS, r.k, nullptr, (int64_t *)(d + L.idx),
                             r.dist ? (double *)(d + L.dist) : nullptr, st);
        if (s == GBO_OK)
        {
            cudaMemcpyAsync(h ? (void *)(h + L.idx) : (void *)r.idx, d + L.idx, n * r.k * 8, cudaMemcpyDeviceToHost,
                            st);
            if (r.dist)
                cudaMemcpyAsync(h ? (void *)(h + L.dist) : (void *)r.dist, d + L.dist, n * r.k * 8,
                                cudaMemcpyDeviceToHost, st);
        }
    }
    if (s != GBO_OK)
    {
        j->status = s;
        j->error = gbo_last_error();
    }
    j->done = slot_event[j->slot];
    cudaEventRecord(j->done, st);
    return true;
}

void gbo_server::run()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    while (true)
    {
        // retire finished requests
        for (size_t si = 0; si < slot_job.size(); ++si)
        {
            Job *j = slot_job[si];
            if (!j)
                continue;
            const cudaError_t q = cudaEventQuery(j->done);
            if (q == cudaErrorNotReady)
                continue;
            if (q != cudaSuccess && j->status == GBO_OK)
            {
                j->status = GBO_ERR_CUDA;
                j->error = cudaGetErrorString(q);
            }
            if (j->hoff >= 0)
            {
                if (j->status == GBO_OK)
                {
                    int dim = 0;
                    internal_request_dim(&j->req, &dim);
                    unstage_outputs(j->req, dim, staging.ptr((size_t)j->hoff));
                }
                staging.release((size_t)j->hoff, j->bytes);
            }
            arena.release((size_t)j->off, j->bytes);
            if (j->req.kind == GBO_REQ_KNN)
                busy_nn.erase(j->req.nn);
            j->latency = std::chrono::duration<double>(Clock::now() - j->submitted).count();
            j->finished = true;
            slot_job[si] = nullptr;
            --inflight;
            ++completed;
            cv_done.notify_all();
        }
        // admit pending requests into free slots, in arrival order, skipping those that do not fit yet;
        // the admitted ones are launched after the lock is released (submit() may append meanwhile)
        std::vector<Job *> admit;
        for (auto it = pending.begin(); it != pending.end() && inflight < (int)slot_job.size();)
        {
            Job *j = *it;
            if (j->req.kind == GBO_REQ_KNN && busy_nn.count(j->req.nn))
            {
                ++it;
                continue;
            }
            const long off = arena.alloc(j->bytes);
            if (off < 0)
            {
                ++it;
                continue;
            }
            j->off = off;
            for (size_t si = 0; si < slot_job.size(); ++si)
                if (!slot_job[si])
                {
                    j->slot = (int)si;
                    slot_job[si] = j;
                    break;
                }
            if (j->req.kind == GBO_REQ_KNN)
                busy_nn.insert(j->req.nn);
            ++inflight;
            max_inflight = std::max(max_inflight, inflight);
            it = pending.erase(it);
            admit.push_back(j);
        }
        if (!admit.empty())
        {
            lk.unlock();
            for (Job *j : admit)
                launch(j);
            lk.lock();
            continue;  // re-check completions and the queue before sleeping
        }
        if (stop && pending.empty() && inflight == 0)
            break;
        if (inflight > 0)
            cv_work.wait_for(lk, std::chrono::microseconds(20));
        else
            cv_work.wait_for(lk, std::chrono::milliseconds(5));
    }
}

extern "C" {

gbo_status gbo_server_create(int n_streams, int64_t arena_bytes, gbo_server **out)
{
    if (!out || n_streams < 1 || n_streams > 256 || arena_bytes < 4096)
        return GBO_ERR_INVALID_ARGUMENT;
    int sm = 0;
    if (gbo_device_check(&sm, nullptr, nullptr) != GBO_OK)
        return GBO_ERR_NO_DEVICE;
    auto *s = new gbo_server();
    cudaGetDevice(&s->device);
    if (!s->arena.init((size_t)arena_bytes))
    {
        delete s;
        return GBO_ERR_OUT_OF_MEMORY;
    }
    for (int i = 0; i < n_streams; ++i)
    {
        cudaStream_t st;
        if (cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) != cudaSuccess)
        {
            for (auto x : s->streams)
                cudaStreamDestroy(x);
            delete s;
            return GBO_ERR_CUDA;
        }
        s->streams.push_back(st);
    }
    s->slot_job.assign(n_streams, nullptr);
    for (int i = 0; i < n_streams; ++i)
    {
        cudaEvent_t ev;
        cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        s->slot_event.push_back(ev);
    }
    // host staging: as large as the device arena up to 2 GiB; without it requests use the caller's arrays
    s->staging.init(std::min<size_t>((size_t)arena_bytes, (size_t)2 << 30), true);
    s->worker = std::thread([s] { s->run(); });
    *out = s;
    return GBO_OK;
}

gbo_status gbo_server_destroy(gbo_server *s)
{
    if (!s)
        return GBO_ERR_INVALID_ARGUMENT;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    s->worker.join();
    for (auto &kv : s->jobs)
        delete kv.second;
    for (auto st : s->streams)
        cudaStreamDestroy(st);
    for (auto ev : s->slot_event)
        cudaEventDestroy(ev);
    delete s;
    return GBO_OK;
}

gbo_status gbo_server_submit(gbo_server *s, const gbo_request *req, uint64_t *ticket)
{
    if (!s || !req || !ticket || req->n < 0)
        return GBO_ERR_INVALID_ARGUMENT;
    int dim = 0;
    if (internal_request_dim(req, &dim) != GBO_OK)
        return GBO_ERR_INVALID_ARGUMENT;
    const gbo_request &r = *req;
    if ((r.kind == GBO_REQ_KNN && (!r.nn || !r.idx || r.k < 1)) ||
        (r.kind != GBO_REQ_KNN && (!r.checker || !r.ok)) || (r.n > 0 && !r.states) ||
        (r.kind == GBO_REQ_MOTION && r.n > 0 && !r.states2))
        return GBO_ERR_INVALID_ARGUMENT;
    auto *j = new Job();
    j->req = r;
    j->bytes = req_layout(r, dim).out_end + 256;
    j->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (j->bytes > s->arena.size())
        {
            delete j;
            return GBO_ERR_OUT_OF_MEMORY;  // can never be admitted
        }
        if (s->staging.size())
            j->hoff = s->staging.alloc(j->bytes);
    }
    if (j->hoff >= 0)
        stage_inputs(r, dim, s->staging.ptr((size_t)j->hoff));  // on the caller's thread, outside the lock
    {
        std::lock_guard<std::mutex> lk(s->mu);
        j->ticket = s->next_ticket++;
        *ticket = j->ticket;
        s->jobs[j->ticket] = j;
        s->pending.push_back(j);
        ++s->submitted;
    }
    s->cv_work.notify_all();
    return GBO_OK;
}

gbo_status gbo_server_wait(gbo_server *s, uint64_t ticket, double timeout_s, double *latency_s)
{
    if (!s)
        return GBO_ERR_INVALID_ARGUMENT;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->jobs.find(ticket);
    if (it == s->jobs.end())
        return GBO_ERR_INVALID_ARGUMENT;
    Job *j = it->second;
    auto pred = [&] { return j->finished; };
    if (timeout_s < 0)
        s->cv_done.wait(lk, pred);
    else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), pred))
        return GBO_ERR_TIMEOUT;
    if (latency_s)
        *latency_s = j->latency;
    const gbo_status st = j->status;
    if (st != GBO_OK)
        gbo::internal_fail(st, j->error.c_str());
    s->jobs.erase(it);
    delete j;
    return st;
}

gbo_status gbo_server_stats(gbo_server *s, uint64_t *submitted, uint64_t *completed, int64_t *arena_in_use,
                            int *max_concurrent)
{
    if (!s)
        return GBO_ERR_INVALID_ARGUMENT;
    std::lock_guard<std::mutex> lk(s->mu);
    if (submitted)
        *submitted = s->submitted;
    if (completed)
        *completed = s->completed;
    if (arena_in_use)
        *arena_in_use = (int64_t)s->arena.used();
    if (max_concurrent)
        *max_concurrent = s->max_inflight;
    return GBO_OK;
}

}  // extern "C"
