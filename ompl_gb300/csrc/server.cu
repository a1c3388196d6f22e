// Request loop (gbo_server_*): continuous admission of validity / motion / nearestK requests from many
// clients onto a fixed set of streams, bounded by a device arena (HBM footprint admission).
//
// One dispatcher thread owns all device work: it retires requests whose completion event has fired
// (freeing their stream slot and arena range), then admits pending requests in arrival order,
// skipping any that does not fit yet (or whose nearest-neighbour index is busy) so that small
// requests are not held behind a large one, copies inputs host->device, launches the library's
// kernels on the slot's stream, copies results device->host, and records an event.
#include <chrono>
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

// First-fit allocator over one device range (256-byte granules).
class Arena
{
public:
    bool init(size_t bytes)
    {
        if (cudaMalloc(&base_, bytes) != cudaSuccess)
            return false;
        size_ = bytes;
        free_[0] = bytes;
        return true;
    }
    ~Arena()
    {
        if (base_)
            cudaFree(base_);
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
    int slot = -1;
    cudaEvent_t done = nullptr;
    gbo_status status = GBO_OK;
    bool finished = false;
    double latency = 0.0;
    std::string error;
};

size_t footprint(const gbo_request &r, int dim)
{
    const size_t rows = (size_t)r.n * dim * sizeof(double);
    switch (r.kind)
    {
        case GBO_REQ_VALIDITY:
            return rows + (size_t)r.n + 512;
        case GBO_REQ_MOTION:
            return 2 * rows + 9 * (size_t)r.n + 1024;
        default:
            return rows + (size_t)r.n * r.k * 16 + 512;
    }
}
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

bool gbo_server::launch(Job *j)
{
    const gbo_request &r = j->req;
    cudaStream_t st = streams[j->slot];
    int dim = 0;
    internal_request_dim(&r, &dim);
    char *d = arena.ptr((size_t)j->off);
    const size_t rows = (size_t)r.n * dim * sizeof(double);
    gbo_status s = GBO_OK;
    if (r.kind == GBO_REQ_VALIDITY)
    {
        uint8_t *dok = (uint8_t *)(d + pad256(rows));
        cudaMemcpyAsync(d, r.states, rows, cudaMemcpyHostToDevice, st);
        s = gbo_is_valid(r.checker, (const double *)d, r.n, dim, GBO_LAYOUT_AOS, dok, st);
        if (s == GBO_OK)
            cudaMemcpyAsync(r.ok, dok, (size_t)r.n, cudaMemcpyDeviceToHost, st);
    }
    else if (r.kind == GBO_REQ_MOTION)
    {
        char *d2 = d + pad256(rows);
        int32_t *dfj = (int32_t *)(d2 + pad256(rows));
        int32_t *dnd = (int32_t *)((char *)dfj + pad256(4 * (size_t)r.n));
        uint8_t *dok = (uint8_t *)((char *)dnd + pad256(4 * (size_t)r.n));
        cudaMemcpyAsync(d, r.states, rows, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(d2, r.states2, rows, cudaMemcpyHostToDevice, st);
        s = gbo_check_motion(r.checker, (const double *)d, (const double *)d2, r.n, dim, GBO_LAYOUT_AOS, r.schedule,
                             dok, dfj, dnd, st);
        if (s == GBO_OK)
        {
            cudaMemcpyAsync(r.ok, dok, (size_t)r.n, cudaMemcpyDeviceToHost, st);
            if (r.first_j)
                cudaMemcpyAsync(r.first_j, dfj, 4 * (size_t)r.n, cudaMemcpyDeviceToHost, st);
            if (r.nd)
                cudaMemcpyAsync(r.nd, dnd, 4 * (size_t)r.n, cudaMemcpyDeviceToHost, st);
        }
    }
    else
    {
        int64_t *didx = (int64_t *)(d + pad256(rows));
        double *ddist = (double *)((char *)didx + pad256((size_t)r.n * r.k * 8));
        cudaMemcpyAsync(d, r.states, rows, cudaMemcpyHostToDevice, st);
        s = gbo_nn_nearest_k(r.nn, (const double *)d, r.n, dim, GBO_LAYOUT_AOS, r.k, nullptr, didx,
                             r.dist ? ddist : nullptr, st);
        if (s == GBO_OK)
        {
            cudaMemcpyAsync(r.idx, didx, (size_t)r.n * r.k * 8, cudaMemcpyDeviceToHost, st);
            if (r.dist)
                cudaMemcpyAsync(r.dist, ddist, (size_t)r.n * r.k * 8, cudaMemcpyDeviceToHost, st);
        }
    }
    if (s != GBO_OK)
    {
        j->status = s;
        j->error = gbo_last_error();
    }
    cudaEventCreateWithFlags(&j->done, cudaEventDisableTiming);
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
            cudaEventDestroy(j->done);
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
    j->bytes = footprint(r, dim);
    j->submitted = Clock::now();
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (j->bytes > s->arena.size())
        {
            delete j;
            return GBO_ERR_OUT_OF_MEMORY;  // can never be admitted
        }
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
