// gbo_nn_nearest_k_noalloc: nearestK without any device allocation during the call.
//
// Who needs it: callers that must not allocate device memory after set-up — code recorded into a
// CUDA graph (an allocation cannot be captured), planning inside a real-time control cycle (an
// allocation can block, fail under memory pressure, or take milliseconds), and processes whose GPU
// memory is owned by another allocator's pool (a raw cudaMalloc may fail there). The regular
// gbo_nn_nearest_k grows per-index scratch buffers with cudaMalloc when a batch is larger than any
// before; this variant takes its scratch from the fixed array below instead.
//
// The scratch is a file-scope device array of GBO_NOALLOC_SCRATCH_BYTES (16 MiB) that every GPU
// which loads the library holds until the process exits. Its device address is looked up once per
// device with cudaGetSymbolAddress, on the first call made with that device current (so make that
// first call before any stream capture). All calls share the one array and it keeps the contents of
// the last call: each call clears the counters it needs, and calls that overlap on the GPU (on
// different streams) race on the array and must not be made.
#include <cstdio>
#include <mutex>

#include "kernels_nn.cuh"

#define GBO_NOALLOC_SCRATCH_BYTES (16u << 20)

static __device__ __align__(256) unsigned char g_noalloc_scratch[GBO_NOALLOC_SCRATCH_BYTES];

namespace gbo
{
gbo_status internal_fail(gbo_status s, const char *msg);
gbo_status internal_ensure_device(int *sm_count);
bool internal_nn_view(const gbo_nn *nn, NNArgs *a, SpaceParams *sp, int *precision, int *features);
}  // namespace gbo

namespace
{
std::mutex g_mu;
void *g_addr[64] = {};

gbo_status scratch_address(unsigned char **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
        return gbo::internal_fail(GBO_ERR_NO_DEVICE, "no current CUDA device");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_addr[dev])
    {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            return gbo::internal_fail(GBO_ERR_CUDA, "cudaGetSymbolAddress of the no-alloc scratch failed");
        g_addr[dev] = p;
    }
    *out = (unsigned char *)g_addr[dev];
    return GBO_OK;
}

size_t align256(size_t b)
{
    return (b + 255) & ~size_t(255);
}
}  // namespace

extern "C" gbo_status gbo_nn_nearest_k_noalloc(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout,
                                               int k, const int64_t *prefix, int64_t *idx, double *dist,
                                               gbo_stream stream)
{
    using namespace gbo;
    NNArgs a;
    SpaceParams sp;
    int precision = 0, F = 0;
    if (!internal_nn_view(nn, &a, &sp, &precision, &F) || nq < 0 || k < 1 || (nq > 0 && (!q || !idx)) ||
        !(layout == GBO_LAYOUT_SOA ? ld >= nq : (layout == GBO_LAYOUT_AOS && ld >= sp.dim)))
        return internal_fail(GBO_ERR_INVALID_ARGUMENT, "bad nearestK arguments");
    if (k > 64)
        return internal_fail(GBO_ERR_UNSUPPORTED, "nearestK supports k <= 64");
    int sm_count = 0;
    if (auto st = internal_ensure_device(&sm_count))
        return st;
    unsigned char *scratch = nullptr;
    if (auto st = scratch_address(&scratch))
        return st;
    if (nq == 0)
        return GBO_OK;
    LaunchCfg lc;
    lc.stream = (cudaStream_t)stream;
    lc.sm_count = sm_count;
    const StatesView qv = make_view(q, ld, layout);
    RunCounters *ctr = (RunCounters *)scratch;
    const bool fp32 = precision == GBO_PRECISION_FP32_GUARDED && k <= knn_fp32_max_k(sp) &&
                      ((sp.kind == GBO_SPACE_KINEMATIC_CHAIN && sp.dim <= 10) ||
                       ((sp.kind == GBO_SPACE_WRAP_L2 || sp.kind == GBO_SPACE_REAL_VECTOR) && sp.dim <= 8));
    if (!fp32)
    {
        // the exact FP64 scan needs no scratch
        launch_knn_exact(lc, a, sp, qv, nq, k, prefix, idx, dist, nullptr, nullptr, nq);
        return cudaGetLastError() == cudaSuccess ? GBO_OK : internal_fail(GBO_ERR_CUDA, "kernel launch failed");
    }
    // scratch layout: counters | query features [F][nq] | fallback list [nq] | partial lists
    const int keep = knn_keep(k);
    const size_t head = align256(sizeof(RunCounters));
    const size_t feat = align256((size_t)F * nq * sizeof(float));
    const size_t fbl = align256((size_t)nq * sizeof(unsigned long long));
    const size_t per_chunk = (size_t)nq * keep * (sizeof(int64_t) + sizeof(float));
    int P = knn_chunks(lc, nq, a.size);
    while (P > 1 && head + feat + fbl + (size_t)P * per_chunk + 256 > GBO_NOALLOC_SCRATCH_BYTES)
        --P;
    if (head + feat + fbl + (size_t)P * per_chunk + 256 > GBO_NOALLOC_SCRATCH_BYTES)
    {
        const size_t per_query = (size_t)F * sizeof(float) + sizeof(unsigned long long) + keep * 12;
        char msg[160];
        snprintf(msg, sizeof(msg), "gbo_nn_nearest_k_noalloc: %lld queries exceed the 16 MiB scratch (at most %lld)",
                 (long long)nq, (long long)((GBO_NOALLOC_SCRATCH_BYTES - 4096) / per_query));
        return internal_fail(GBO_ERR_OUT_OF_MEMORY, msg);
    }
    float *qf = (float *)(scratch + head);
    unsigned long long *fb_list = (unsigned long long *)(scratch + head + feat);
    int64_t *part_k = (int64_t *)(scratch + head + feat + fbl);
    float *part_d = (float *)(part_k + (size_t)P * nq * keep);
    // the counters (fallback count, re-check statistics) must start at zero
    if (cudaMemsetAsync(ctr, 0, sizeof(RunCounters), lc.stream) != cudaSuccess)
        return internal_fail(GBO_ERR_CUDA, "clearing the no-alloc counters failed");
    unsigned long long *fb_n = &ctr->queue;
    launch_features(lc, sp, qv, nq, qf, nq);
    launch_knn_fp32(lc, a, sp, qv, qf, nq, k, prefix, idx, dist, fb_list, fb_n, ctr, part_d, part_k, P, nullptr,
                    nullptr);
    launch_knn_exact(lc, a, sp, qv, nq, k, prefix, idx, dist, fb_list, fb_n, nq < 4096 ? nq : 4096);
    return cudaGetLastError() == cudaSuccess ? GBO_OK : internal_fail(GBO_ERR_CUDA, "kernel launch failed");
}
