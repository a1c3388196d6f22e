// Nearest-neighbour kernels behind NearestNeighbors<T>::nearestK / nearestR.
//
// Result order is (FP64 distance, key), key = insertion index: the order NearestNeighborsLinear
// produces (NearestNeighborsLinear.h:119-142) whenever distances are distinct, with ties resolved by
// insertion order. distance is evaluated as distance(element, query) (ElemSort, :159-172).
//
//   knn_exact_kernel  FP64, one warp per query: lanes scan keys lane, lane+32, ... keeping a sorted
//                     register top-k; the warp then merges the 32 lists with shuffle argmin rounds.
//   knn_scan_kernel   FP32 bulk, one thread per query over one chunk of the elements (CTA grid =
//                     query blocks x chunks, so that few queries still fill the GPU), element features
//                     staged in shared-memory tiles and read as float4; keeps the best K_KEEP by FP32
//                     distance (kinematic chain: an L1 lower bound skips the square roots of far elements).
//   knn_bcell_warp_kernel, knn_ccell_warp_kernel
//                     FP32 bulk over a cell index of the elements (box / wrapped spaces; the chain
//                     metric), one warp per query: the lanes test 32 cell boxes at a time and scan a
//                     needed cell's elements 32 at a time; the kept list lives in the lanes.
//   knn_finish_kernel merges the chunk lists; every kept element within 2*eps of the k-th FP32
//                     distance is re-evaluated in FP64 and the final order is decided in FP64. If the
//                     band may hold more than K_KEEP elements the query is queued for knn_exact_kernel.
//   radius kernels    FP64 count / fill (CSR), sorted by (distance, key).
#include <climits>

#include <cuda_fp16.h>

#include "kernels_nn.cuh"

namespace gbo
{

template <int MAXD>
__device__ __forceinline__ void load_point(const double *pts, int64_t cap, int dim, int64_t key, double *x)
{
#pragma unroll
    for (int d = 0; d < MAXD; ++d)
        x[d] = d < dim ? pts[(int64_t)d * cap + key] : 0.0;
}

template <int MAXD>
__device__ __forceinline__ void load_query(const StatesView &v, int64_t i, int dim, double *x)
{
#pragma unroll
    for (int d = 0; d < MAXD; ++d)
        x[d] = d < dim ? v(i, d) : 0.0;
}

// Insert (d, key) into an ascending register list; equal distances keep the earlier entry first.
template <int K, class T, class I>
__device__ __forceinline__ void topk_insert(T *dk, I *ik, T d, I key)
{
#pragma unroll
    for (int j = K - 1; j >= 0; --j)
    {
        const bool shift = (j > 0) && (d < dk[j > 0 ? j - 1 : 0]);
        const bool here = !shift && (d < dk[j]);
        if (shift)
        {
            dk[j] = dk[j - 1];
            ik[j] = ik[j - 1];
        }
        else if (here)
        {
            dk[j] = d;
            ik[j] = key;
        }
    }
}

__device__ __forceinline__ bool less_dk(double a, int64_t ka, double b, int64_t kb)
{
    return a < b || (a == b && ka < kb);
}

template <int K, int MAXD>
__device__ void knn_exact_query(const NNArgs &nn, const SpaceParams &sp, const double *q, int k, int64_t limit,
                                int64_t *idx_out, double *dist_out)
{
    const int lane = threadIdx.x & 31;
    double dk[K];
    int64_t ik[K];
#pragma unroll
    for (int j = 0; j < K; ++j)
    {
        dk[j] = __longlong_as_double(0x7ff0000000000000ll);
        ik[j] = -1;
    }
    for (int64_t key = lane; key < limit; key += 32)
    {
        if (!nn.alive[key])
            continue;
        double x[MAXD];
        load_point<MAXD>(nn.pts64, nn.cap, sp.dim, key, x);
        const double d = distance64<MAXD, false>(sp, x, q);
        if (d < dk[K - 1])
            topk_insert<K>(dk, ik, d, key);
    }
    // merge: k rounds of warp-wide (distance, key) argmin over list heads
    for (int r = 0; r < k; ++r)
    {
        double bd = dk[0];
        int64_t bk = ik[0] < 0 ? INT64_MAX : ik[0];
        int bl = lane;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            const double od = __shfl_xor_sync(0xffffffffu, bd, o);
            const int64_t ok = __shfl_xor_sync(0xffffffffu, bk, o);
            const int ol = __shfl_xor_sync(0xffffffffu, bl, o);
            if (less_dk(od, ok, bd, bk))
            {
                bd = od;
                bk = ok;
                bl = ol;
            }
        }
        if (lane == 0)
        {
            idx_out[r] = bk == INT64_MAX ? -1 : bk;
            if (dist_out)
                dist_out[r] = bd;
        }
        if (lane == bl)
        {
#pragma unroll
            for (int j = 0; j < K - 1; ++j)
            {
                dk[j] = dk[j + 1];
                ik[j] = ik[j + 1];
            }
            dk[K - 1] = __longlong_as_double(0x7ff0000000000000ll);
            ik[K - 1] = -1;
        }
    }
}

template <int K, int MAXD>
__global__ void __launch_bounds__(256) knn_exact_kernel(NNArgs nn, SpaceParams sp, StatesView qv, int64_t nq, int k,
                                                        const int64_t *prefix, int64_t *idx, double *dist,
                                                        const unsigned long long *list, const unsigned long long *list_n)
{
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t count = list ? (int64_t)*list_n : nq;
    for (int64_t w = warp; w < count; w += nwarps)
    {
        const int64_t qi = list ? (int64_t)list[w] : w;
        double q[MAXD];
        load_query<MAXD>(qv, qi, sp.dim, q);
        int64_t limit = nn.size;
        if (prefix)
            limit = min(limit, prefix[qi]);
        knn_exact_query<K, MAXD>(nn, sp, q, k, limit, idx + qi * k, dist ? dist + qi * k : nullptr);
    }
}

// ---------------------------------------------------------------- FP32 scan

// Element features: REAL_VECTOR / WRAP_L2 / SO2: the coordinates (F = dim); KINEMATIC_CHAIN: the
// cumulative link-direction sums interleaved (X_1, Y_1, ..., X_n, Y_n), F = 2 dim, so that
// distance = L * sum_i |(X_i(a) - X_i(b), Y_i(a) - Y_i(b))|. All indices below are compile-time.
template <int KIND, int MAXF>
__device__ __forceinline__ float box_dist2(const float *a, const float *b, int dim)
{
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < MAXF; ++i)
        if (i < dim)
        {
            float d = a[i] - b[i];
            if constexpr (KIND == GBO_SPACE_WRAP_L2 || KIND == GBO_SPACE_SO2)
            {
                d = fabsf(d);
                d = fminf(d, 6.28318530717958647692f - d);
            }
            s = fmaf(d, d, s);
        }
    return s;
}

// Partial L1 lower bound over links [i0, i1): sum (|dx_i| + |dy_i|) <= sqrt(2) * sum |(dx_i, dy_i)|.
template <int MAXF>
__device__ __forceinline__ float chain_l1(const float *a, const float *b, int dim, int i0, int i1)
{
    float l1 = 0.f;
#pragma unroll
    for (int i = 0; i < MAXF / 2; ++i)
        if (i >= i0 && i < i1 && i < dim)
            l1 += fabsf(a[2 * i] - b[2 * i]) + fabsf(a[2 * i + 1] - b[2 * i + 1]);
    return l1;
}

__device__ __forceinline__ float sqrt_approx(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <int MAXF>
__device__ __forceinline__ float chain_dist32(const float *a, const float *b, int dim)
{
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < MAXF / 2; ++i)
        if (i < dim)
        {
            const float dx = a[2 * i] - b[2 * i], dy = a[2 * i + 1] - b[2 * i + 1];
            s += sqrt_approx(fmaf(dx, dx, dy * dy));
        }
    return s;
}

// Partial scan: CTA (x = block of 128 queries, y = chunk of elements). Each thread keeps the K_KEEP
// smallest FP32 distances (squared for box/wrapped kinds) of its query within the chunk. qorder
// (nullable): thread qs takes query qorder[qs] (queries in spatial order, so that the lanes of a warp
// prune the same elements); its list is kept at position qs.
// qkey (nullable): only the queries with qkey < key_limit are this launch's (the others' lists are
// written by the cell kernel).
// thr (nullable): per query position, the smallest K_KEEP-th distance any chunk has reached so far
// (float bits; non-negative floats order like their bits). Every chunk's list is an upper bound on the
// query's K_KEEP-th smallest distance, so each CTA prunes against the smallest one published, reading
// and publishing it once per tile. An element dropped that way is beyond the merged list's last entry,
// which the finish kernel's overflow test already treats as possibly dropped.
template <int KIND, int MAXF, int K_KEEP>
__global__ void __launch_bounds__(128) knn_scan_kernel(NNArgs nn, SpaceParams sp, const float *qf, int64_t nq,
                                                       const int64_t *prefix, int64_t chunk, float *part_d,
                                                       int64_t *part_k, const int64_t *qorder, const int *qkey,
                                                       int key_limit, unsigned *thr)
{
    constexpr int TILE = 128;
    constexpr int FP = (MAXF + 3) / 4 * 4;
    __shared__ __align__(16) float tile[TILE][FP];
    __shared__ unsigned char tile_alive[TILE];
    __shared__ unsigned long long s_limit;
    const int F = KIND == GBO_SPACE_KINEMATIC_CHAIN ? 2 * sp.dim : sp.dim;
    const int64_t qs = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const int64_t qi = qs < nq && qorder ? qorder[qs] : qs;
    const bool active = qs < nq && (!qkey || qkey[qi] < key_limit);
    const int64_t c0 = (int64_t)blockIdx.y * chunk;
    const int64_t c1 = min(c0 + chunk, nn.size);
    float qfe[FP];
#pragma unroll
    for (int f = 0; f < FP; ++f)
        qfe[f] = (active && f < F) ? qf[(int64_t)f * nq + qi] : 0.f;
    int64_t limit = c1;
    if (active && prefix)
        limit = min(limit, prefix[qi]);
    if (threadIdx.x == 0)
        s_limit = 0;
    __syncthreads();
    if (active && limit > c0)
        atomicMax(&s_limit, (unsigned long long)limit);
    __syncthreads();
    const int64_t block_end = (int64_t)s_limit;

    float dk[K_KEEP];
    int ik[K_KEEP];
#pragma unroll
    for (int j = 0; j < K_KEEP; ++j)
    {
        dk[j] = __int_as_float(0x7f800000);
        ik[j] = -1;
    }
    const float lscale = KIND == GBO_SPACE_KINEMATIC_CHAIN ? 0.70710678f * (1.0f - 1e-5f) * (float)sp.link : 1.0f;
    float g = __int_as_float(0x7f800000);  // the shared bound last read
    for (int64_t base = c0; base < block_end; base += TILE)
    {
        __syncthreads();
        for (int i = threadIdx.x; i < TILE * F; i += blockDim.x)
        {
            const int f = i / TILE, t = i - f * TILE;
            const int64_t key = base + t;
            tile[t][f] = key < block_end ? nn.feat32[(int64_t)f * nn.cap + key] : 0.f;
        }
        for (int t = threadIdx.x; t < TILE; t += blockDim.x)
            tile_alive[t] = (base + t < block_end) ? nn.alive[base + t] : 0;
        __syncthreads();
        if (!active)
            continue;
        if (thr)
            g = __uint_as_float(__ldcg(thr + qs));
        float cut = fminf(dk[K_KEEP - 1], g);
        const int tn = (int)max((int64_t)0, min((int64_t)TILE, limit - base));
        for (int t = 0; t < tn; ++t)
        {
            if (!tile_alive[t])
                continue;
            float pf[FP];
#pragma unroll
            for (int f = 0; f < FP; f += 4)
            {
                const float4 v = *reinterpret_cast<const float4 *>(&tile[t][f]);
                pf[f] = v.x;
                pf[f + 1] = v.y;
                pf[f + 2] = v.z;
                pf[f + 3] = v.w;
            }
            float d;
            if constexpr (KIND == GBO_SPACE_KINEMATIC_CHAIN)
            {
                // outer links first: their terms are the largest, so most elements stop here
                const int half = sp.dim >> 1;
                float lb = chain_l1<MAXF>(pf, qfe, sp.dim, half, sp.dim);
                if (lb * lscale >= cut)
                    continue;
                lb += chain_l1<MAXF>(pf, qfe, sp.dim, 0, half);
                if (lb * lscale >= cut)
                    continue;
                d = chain_dist32<MAXF>(pf, qfe, sp.dim) * (float)sp.link;
            }
            else
                d = box_dist2<KIND, MAXF>(pf, qfe, sp.dim);
            if (d < cut)
            {
                topk_insert<K_KEEP>(dk, ik, d, (int)(base + t));
                cut = fminf(cut, dk[K_KEEP - 1]);
            }
        }
        if (thr && dk[K_KEEP - 1] < g)
            atomicMin(thr + qs, __float_as_uint(dk[K_KEEP - 1]));
    }
    if (!active)
        return;
    const int64_t o = ((int64_t)blockIdx.y * nq + qs) * K_KEEP;
#pragma unroll
    for (int j = 0; j < K_KEEP; ++j)
    {
        part_d[o + j] = dk[j];
        part_k[o + j] = ik[j];
    }
}

// Merge the per-chunk lists, then decide in FP64: every element within 2*eps of the k-th FP32
// distance is re-evaluated with the reference-order FP64 distance and the final order is
// (FP64 distance, key). If the band may hold more than K_KEEP elements the query goes to the FP64 scan.
// qorder (nullable): the lists are kept per position qs of the query order, query qorder[qs].
template <int KIND, int MAXD, int K_KEEP>
__global__ void __launch_bounds__(128) knn_finish_kernel(NNArgs nn, SpaceParams sp, StatesView qv, int64_t nq, int k,
                                                         int P, const float *part_d, const int64_t *part_k,
                                                         int64_t *idx, double *dist, unsigned long long *fb_list,
                                                         unsigned long long *fb_n, RunCounters *ctr,
                                                         const int64_t *qorder)
{
    const int64_t qs = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (qs >= nq)
        return;
    const int64_t qi = qorder ? qorder[qs] : qs;
    float dk[K_KEEP];
    int64_t ik[K_KEEP];
#pragma unroll
    for (int j = 0; j < K_KEEP; ++j)
    {
        dk[j] = __int_as_float(0x7f800000);
        ik[j] = -1;
    }
    // dropped: smallest distance of an element that fell out of some chunk's list (bounds the rest)
    for (int c = 0; c < P; ++c)
    {
        const int64_t o = ((int64_t)c * nq + qs) * K_KEEP;
        for (int j = 0; j < K_KEEP; ++j)
        {
            const int64_t key = part_k[o + j];
            if (key < 0)
                break;
            const float d = part_d[o + j];
            if (d < dk[K_KEEP - 1] || (d == dk[K_KEEP - 1] && ik[K_KEEP - 1] < 0))
                topk_insert<K_KEEP>(dk, ik, d, key);
        }
    }
    const float eps = nn.eps32;
    const float kth = dk[k - 1];
    float band;
    if constexpr (KIND == GBO_SPACE_KINEMATIC_CHAIN)
        band = kth + 2.f * eps;
    else
    {
        const float r = sqrtf(kth) + 2.f * eps;
        band = r * r * (1.0f + 1e-6f);
    }
    // A full kept list whose last entry is inside the band, or any chunk list that was full and whose
    // last entry is inside the band, means elements of the band may have been dropped.
    bool overflow = ik[K_KEEP - 1] >= 0 && !(dk[K_KEEP - 1] > band);
    for (int c = 0; c < P && !overflow; ++c)
    {
        const int64_t o = ((int64_t)c * nq + qs) * K_KEEP;
        overflow = part_k[o + K_KEEP - 1] >= 0 && !(part_d[o + K_KEEP - 1] > band);
    }
    if (overflow)
    {
        const unsigned long long pos = atomicAdd(fb_n, 1ull);
        fb_list[pos] = (unsigned long long)qi;
        atomicAdd(&ctr->fallbacks, 1ull);
        return;
    }
    double q64[MAXD];
    load_query<MAXD>(qv, qi, sp.dim, q64);
    double d64[K_KEEP];
    int64_t k64[K_KEEP];
#pragma unroll
    for (int j = 0; j < K_KEEP; ++j)
    {
        d64[j] = __longlong_as_double(0x7ff0000000000000ll);
        k64[j] = INT64_MAX;
    }
    int nc = 0;
    float max_err = 0.f;
    for (int j = 0; j < K_KEEP; ++j)
    {
        if (ik[j] < 0 || !(j < k || dk[j] <= band))
            break;
        double x[MAXD];
        load_point<MAXD>(nn.pts64, nn.cap, sp.dim, ik[j], x);
        double cd = distance64<MAXD, false>(sp, x, q64);
        // measured FP32 metric error (the lists hold distances for the chain, squares otherwise)
        const float d32 = KIND == GBO_SPACE_KINEMATIC_CHAIN ? dk[j] : sqrtf(dk[j]);
        max_err = fmaxf(max_err, fabsf((float)(cd - (double)d32)));
        int64_t ck = ik[j];
#pragma unroll
        for (int m = 0; m < K_KEEP; ++m)
            if (less_dk(cd, ck, d64[m], k64[m]))
            {
                const double td = d64[m];
                const int64_t tk = k64[m];
                d64[m] = cd;
                k64[m] = ck;
                cd = td;
                ck = tk;
            }
        ++nc;
    }
    atomicAdd(&ctr->rechecked, (unsigned long long)nc);
    if (max_err > 0.f)
        atomicMax(&ctr->max_err_bits, __float_as_uint(max_err));  // non-negative floats order as integers
    for (int j = 0; j < k; ++j)
    {
        const bool have = k64[j] != INT64_MAX;
        idx[qi * k + j] = have ? k64[j] : -1;
        if (dist)
            dist[qi * k + j] = have ? d64[j] : __longlong_as_double(0x7ff0000000000000ll);
    }
}

// ---------------------------------------------------------------- features
template <int MAXD>
__global__ void features_kernel(SpaceParams sp, StatesView v, int64_t n, float *out, int64_t ld_out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    if (sp.kind == GBO_SPACE_KINEMATIC_CHAIN)
    {
        double theta = 0.;
        float X = 0.f, Y = 0.f;
        for (int d = 0; d < sp.dim; ++d)
        {
            theta = dadd(theta, v(i, d));
            float c, s;
            dir32(theta, c, s);
            X += c;
            Y += s;
            out[(int64_t)(2 * d) * ld_out + i] = X;
            out[(int64_t)(2 * d + 1) * ld_out + i] = Y;
        }
    }
    else
    {
        for (int d = 0; d < sp.dim; ++d)
            out[(int64_t)d * ld_out + i] = (float)v(i, d);
    }
}

template <int MAXD>
__global__ void store_points_kernel(StatesView v, int64_t n, int dim, double *pts, int64_t cap, int64_t first,
                                    unsigned char *alive)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    for (int d = 0; d < dim; ++d)
        pts[(int64_t)d * cap + first + i] = v(i, d);
    alive[first + i] = 1;
}

__global__ void remove_kernel(const int64_t *keys, int64_t n, int64_t size, unsigned char *alive)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && keys[i] >= 0 && keys[i] < size)
        alive[keys[i]] = 0;
}

// ---------------------------------------------------------------- radius (FP64)
template <int MAXD>
__global__ void __launch_bounds__(256) radius_kernel(NNArgs nn, SpaceParams sp, StatesView qv, int64_t nq, double r,
                                                     int64_t *counts, const int64_t *offsets, int64_t *idx,
                                                     double *dist)
{
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t qi = warp; qi < nq; qi += nwarps)
    {
        double q[MAXD];
        load_query<MAXD>(qv, qi, sp.dim, q);
        int64_t c = 0;
        int64_t out = offsets ? offsets[qi] : 0;
        for (int64_t base = 0; base < nn.size; base += 32)
        {
            const int64_t key = base + lane;
            bool hit = false;
            double d = 0.0;
            if (key < nn.size && nn.alive[key])
            {
                double x[MAXD];
                load_point<MAXD>(nn.pts64, nn.cap, sp.dim, key, x);
                d = distance64<MAXD, false>(sp, x, q);
                hit = d <= r;
            }
            const unsigned m = __ballot_sync(0xffffffffu, hit);
            if (offsets && hit)
            {
                const int64_t pos = out + __popc(m & ((1u << lane) - 1u));
                idx[pos] = key;
                dist[pos] = d;
            }
            out += __popc(m);
            c += __popc(m);
        }
        if (lane == 0 && counts)
            counts[qi] = c;
        __syncwarp();
        if (offsets && lane == 0)
        {
            // stable insertion sort of the segment by distance (keys already ascending)
            const int64_t b = offsets[qi], e = b + c;
            for (int64_t i = b + 1; i < e; ++i)
            {
                const double dv = dist[i];
                const int64_t kv = idx[i];
                int64_t j = i - 1;
                while (j >= b && dist[j] > dv)
                {
                    dist[j + 1] = dist[j];
                    idx[j + 1] = idx[j];
                    --j;
                }
                dist[j + 1] = dv;
                idx[j + 1] = kv;
            }
        }
        __syncwarp();
    }
}

// ---------------------------------------------------------------- launchers
static int grid_for(int64_t items, int per_block, int cap_blocks)
{
    int64_t g = (items + per_block - 1) / per_block;
    if (g < 1)
        g = 1;
    return (int)(g < cap_blocks ? g : cap_blocks);
}

template <int MAXD>
static void launch_exact_t(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, int64_t nq,
                           int k, const int64_t *prefix, int64_t *idx, double *dist, const unsigned long long *list,
                           const unsigned long long *list_n, int64_t max_items)
{
    const int grid = grid_for(max_items * 32, 256, lc.sm_count * 16);
    if (k <= 16)
        knn_exact_kernel<16, MAXD><<<grid, 256, 0, lc.stream>>>(nn, sp, qv, nq, k, prefix, idx, dist, list, list_n);
    else if (k <= 32)
        knn_exact_kernel<32, MAXD><<<grid, 256, 0, lc.stream>>>(nn, sp, qv, nq, k, prefix, idx, dist, list, list_n);
    else
        knn_exact_kernel<64, MAXD><<<grid, 256, 0, lc.stream>>>(nn, sp, qv, nq, k, prefix, idx, dist, list, list_n);
    note_launch();
}

void launch_knn_exact(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, int64_t nq, int k,
                      const int64_t *prefix, int64_t *idx, double *dist, const unsigned long long *list,
                      const unsigned long long *list_n, int64_t max_items)
{
    if (sp.dim <= 2)
        launch_exact_t<2>(lc, nn, sp, qv, nq, k, prefix, idx, dist, list, list_n, max_items);
    else if (sp.dim <= 8)
        launch_exact_t<8>(lc, nn, sp, qv, nq, k, prefix, idx, dist, list, list_n, max_items);
    else
        launch_exact_t<16>(lc, nn, sp, qv, nq, k, prefix, idx, dist, list, list_n, max_items);
}

// NearestNeighborsSqrtApprox::nearest (NearestNeighborsSqrtApprox.h:91-115) for queries made one after
// another: query q examines positions (j checks + off_q) % n, j < checks, of the n present elements in
// insertion order (key rank[pos], or pos when none was removed) and returns the first strict minimum of
// the FP64 distance (element, query) in j order. One warp per query, lanes over j, then the warp's
// minimum of (distance, j). off_q is off0 for the first query and (off0 + q) % checks after it, as the
// structure's offset advances by one (mod checks) per call.
template <int MAXD>
__global__ void __launch_bounds__(256) sqrt_approx_kernel(NNArgs nn, SpaceParams sp, StatesView qv, int64_t nq,
                                                          int64_t n, int64_t checks, unsigned long long off0,
                                                          const int64_t *rank, int64_t *idx, double *dist)
{
    const int lane = threadIdx.x & 31;
    const int64_t q = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (q >= nq)
        return;
    const unsigned long long un = (unsigned long long)n, uc = (unsigned long long)checks;
    const unsigned long long off = q == 0 ? off0 : (off0 + (unsigned long long)q) % uc;
    double qs[MAXD];
    load_query<MAXD>(qv, q, sp.dim, qs);
    double best = 0.0;
    int64_t bj = -1;
    for (int64_t j = lane; j < checks; j += 32)
    {
        const int64_t pos = (int64_t)(((unsigned long long)j * uc + off) % un);
        const int64_t key = rank ? rank[pos] : pos;
        double x[MAXD];
        load_point<MAXD>(nn.pts64, nn.cap, sp.dim, key, x);
        const double dd = distance64<MAXD>(sp, x, qs);
        if (bj < 0 || dd < best)
        {
            best = dd;
            bj = j;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        const double ob = __shfl_xor_sync(0xffffffffu, best, o);
        const int64_t oj = __shfl_xor_sync(0xffffffffu, bj, o);
        if (oj >= 0 && (bj < 0 || ob < best || (ob == best && oj < bj)))
        {
            best = ob;
            bj = oj;
        }
    }
    if (lane == 0)
    {
        const int64_t pos = (int64_t)(((unsigned long long)bj * uc + off) % un);
        idx[q] = rank ? rank[pos] : pos;
        dist[q] = best;
    }
}

void launch_sqrt_approx(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, int64_t nq,
                        int64_t n, int64_t checks, unsigned long long off0, const int64_t *rank, int64_t *idx,
                        double *dist)
{
    if (nq == 0)
        return;
    const int grid = (int)((nq * 32 + 255) / 256);
    if (sp.dim <= 2)
        sqrt_approx_kernel<2><<<grid, 256, 0, lc.stream>>>(nn, sp, qv, nq, n, checks, off0, rank, idx, dist);
    else if (sp.dim <= 8)
        sqrt_approx_kernel<8><<<grid, 256, 0, lc.stream>>>(nn, sp, qv, nq, n, checks, off0, rank, idx, dist);
    else
        sqrt_approx_kernel<16><<<grid, 256, 0, lc.stream>>>(nn, sp, qv, nq, n, checks, off0, rank, idx, dist);
    note_launch();
}

template <int KIND, int MAXD, int MAXF, int K_KEEP>
static void launch_fp32_t(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, const float *qf,
                          int64_t nq, int k, const int64_t *prefix, int64_t *idx, double *dist,
                          unsigned long long *fb_list, unsigned long long *fb_n, RunCounters *ctr, float *part_d,
                          int64_t *part_k, int P, int64_t chunk, const int64_t *qorder, unsigned *thr)
{
    const int qb = (int)((nq + 127) / 128);
    if (thr && P > 1)
        cudaMemsetAsync(thr, 0x7f, (size_t)nq * sizeof(unsigned), lc.stream);  // 3.4e38: no bound yet
    knn_scan_kernel<KIND, MAXF, K_KEEP><<<dim3(qb, P), 128, 0, lc.stream>>>(nn, sp, qf, nq, prefix, chunk, part_d,
                                                                           part_k, qorder, nullptr, 0,
                                                                           P > 1 ? thr : nullptr);
    knn_finish_kernel<KIND, MAXD, K_KEEP><<<qb, 128, 0, lc.stream>>>(nn, sp, qv, nq, k, P, part_d, part_k, idx, dist,
                                                                    fb_list, fb_n, ctr, qorder);
    note_launch();
    note_launch();
}

int knn_fp32_max_k(const SpaceParams &sp)
{
    return (sp.kind == GBO_SPACE_WRAP_L2 || sp.kind == GBO_SPACE_REAL_VECTOR) && sp.dim <= 8 ? 64 : 20;
}

int knn_keep(int k)
{
    return k <= 12 ? 16 : k <= 20 ? 24 : k <= 40 ? 48 : 72;
}

int knn_chunks(const LaunchCfg &lc, int64_t nq, int64_t size)
{
    const int64_t qb = (nq + 127) / 128;
    int64_t P = (lc.sm_count * 8 + qb - 1) / qb;
    P = std::min<int64_t>(P, std::max<int64_t>(1, size / 4096));
    return (int)std::max<int64_t>(1, std::min<int64_t>(P, 64));
}

bool launch_knn_fp32(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, const float *qf,
                     int64_t nq, int k, const int64_t *prefix, int64_t *idx, double *dist, unsigned long long *fb_list,
                     unsigned long long *fb_n, RunCounters *ctr, float *part_d, int64_t *part_k, int P,
                     const int64_t *qorder, unsigned *thr)
{
    if (nq == 0 || k > knn_fp32_max_k(sp))
        return false;
    const int64_t chunk = (nn.size + P - 1) / P;
#define GBO_FP32(KIND, MAXD, MAXF, KK)                                                                                 \
    launch_fp32_t<KIND, MAXD, MAXF, KK>(lc, nn, sp, qv, qf, nq, k, prefix, idx, dist, fb_list, fb_n, ctr, part_d,     \
                                        part_k, P, chunk, qorder, thr)
#define GBO_FP32_K(KIND, MAXD, MAXF)                                                                                   \
    do                                                                                                                \
    {                                                                                                                 \
        if (k <= 12)                                                                                                  \
            GBO_FP32(KIND, MAXD, MAXF, 16);                                                                           \
        else if (k <= 20)                                                                                             \
            GBO_FP32(KIND, MAXD, MAXF, 24);                                                                           \
        else if (k <= 40)                                                                                             \
            GBO_FP32(KIND, MAXD, MAXF, 48);                                                                           \
        else                                                                                                          \
            GBO_FP32(KIND, MAXD, MAXF, 72);                                                                           \
    } while (0)
    if (sp.kind == GBO_SPACE_KINEMATIC_CHAIN && sp.dim <= 10)
    {
        if (k <= 12)
            GBO_FP32(GBO_SPACE_KINEMATIC_CHAIN, 10, 20, 16);
        else
            GBO_FP32(GBO_SPACE_KINEMATIC_CHAIN, 10, 20, 24);
    }
    else if (sp.kind == GBO_SPACE_WRAP_L2 && sp.dim <= 8)
        GBO_FP32_K(GBO_SPACE_WRAP_L2, 8, 8);
    else if (sp.kind == GBO_SPACE_REAL_VECTOR && sp.dim <= 8)
        GBO_FP32_K(GBO_SPACE_REAL_VECTOR, 8, 8);
    else
        return false;
#undef GBO_FP32_K
#undef GBO_FP32
    return true;
}

void launch_features(const LaunchCfg &lc, const SpaceParams &sp, StatesView v, int64_t n, float *out, int64_t ld_out)
{
    if (n == 0)
        return;
    features_kernel<GBO_MAXD><<<(int)((n + 255) / 256), 256, 0, lc.stream>>>(sp, v, n, out, ld_out);
    note_launch();
}

void launch_store_points(const LaunchCfg &lc, StatesView v, int64_t n, int dim, double *pts, int64_t cap,
                         int64_t first, unsigned char *alive)
{
    if (n == 0)
        return;
    store_points_kernel<GBO_MAXD><<<(int)((n + 255) / 256), 256, 0, lc.stream>>>(v, n, dim, pts, cap, first, alive);
    note_launch();
}

void launch_remove(const LaunchCfg &lc, const int64_t *keys, int64_t n, int64_t size, unsigned char *alive)
{
    if (n == 0)
        return;
    remove_kernel<<<(int)((n + 255) / 256), 256, 0, lc.stream>>>(keys, n, size, alive);
    note_launch();
}

void launch_radius(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, int64_t nq, double r,
                   int64_t *counts, const int64_t *offsets, int64_t *idx, double *dist)
{
    if (nq == 0)
        return;
    const int grid = grid_for(nq * 32, 256, lc.sm_count * 16);
    if (sp.dim <= 2)
        radius_kernel<2><<<grid, 256, 0, lc.stream>>>(nn, sp, qv, nq, r, counts, offsets, idx, dist);
    else if (sp.dim <= 8)
        radius_kernel<8><<<grid, 256, 0, lc.stream>>>(nn, sp, qv, nq, r, counts, offsets, idx, dist);
    else
        radius_kernel<16><<<grid, 256, 0, lc.stream>>>(nn, sp, qv, nq, r, counts, offsets, idx, dist);
    note_launch();
}

// ---------------------------------------------------------------- query order (large batches)
// A cell key per query from a few quantised features: chain metric, the tip and middle-joint points
// (X_i, Y_i in units of the link length: roughly mean 0 and variance (i + 1) / 2 for uniform joints,
// 8 levels over +-2.5 standard deviations each); box and wrapped kinds, the first four coordinates over
// their bounds (8 levels each). A counting sort by key gives the processing order.
__device__ __forceinline__ int query_level(float v, float lo, float hi)
{
    int l = (int)floorf((v - lo) * (8.0f / (hi - lo)));
    return l < 0 ? 0 : (l > 7 ? 7 : l);
}

// Key of row i of SoA features f (row stride ld).
__device__ __forceinline__ int order_key(const SpaceParams &sp, const float *f, int64_t ld, int64_t i)
{
    int c = 0;
    if (sp.kind == GBO_SPACE_KINEMATIC_CHAIN)
    {
        const int links[2] = {sp.dim - 1, sp.dim / 2 - 1 > 0 ? sp.dim / 2 - 1 : 0};
        for (int t = 0; t < 2; ++t)
        {
            const float r = 2.5f * sqrtf(0.5f * (float)(links[t] + 1));
            c = c * 64 + query_level(f[(int64_t)(2 * links[t]) * ld + i], -r, r) * 8 +
                query_level(f[(int64_t)(2 * links[t] + 1) * ld + i], -r, r);
        }
    }
    else
    {
        for (int d = 0; d < 4; ++d)
        {
            int l = 0;
            if (d < sp.dim)
            {
                const float lo = sp.kind == GBO_SPACE_REAL_VECTOR ? (float)sp.low[d] : -3.14159265f;
                const float hi = sp.kind == GBO_SPACE_REAL_VECTOR ? (float)sp.high[d] : 3.14159265f;
                l = hi > lo ? query_level(f[(int64_t)d * ld + i], lo, hi) : 0;
            }
            c = c * 8 + l;
        }
    }
    return c;
}

// keys of rows [0, n) of features with row stride ld; alive (nullable): rows whose flag is 0 get -1
__global__ void query_key_kernel(SpaceParams sp, const float *qf, int64_t ld, int64_t n, const unsigned char *alive,
                                 int *key, int *count)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        if (alive && !alive[i])
        {
            key[i] = -1;
            continue;
        }
        const int c = order_key(sp, qf, ld, i);
        key[i] = c;
        atomicAdd(&count[c], 1);
    }
}

// exclusive scan of the 4096 key counts (one CTA of 1024 threads, 4 keys each); fill[] cleared
__global__ void __launch_bounds__(1024) query_scan_kernel(const int *count, int *start, int *fill)
{
    __shared__ int part[1024];
    const int i0 = threadIdx.x * 4;
    const int s0 = count[i0], s1 = count[i0 + 1], s2 = count[i0 + 2], s3 = count[i0 + 3];
    part[threadIdx.x] = s0 + s1 + s2 + s3;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1)
    {
        const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    const int run = part[threadIdx.x] - (s0 + s1 + s2 + s3);
    start[i0] = run;
    start[i0 + 1] = run + s0;
    start[i0 + 2] = run + s0 + s1;
    start[i0 + 3] = run + s0 + s1 + s2;
    fill[i0] = fill[i0 + 1] = fill[i0 + 2] = fill[i0 + 3] = 0;
}

__global__ void query_scatter_kernel(const int *key, int64_t nq, const int *start, int *fill, int64_t *order)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x)
    {
        const int c = key[i];
        if (c >= 0)
            order[start[c] + atomicAdd(&fill[c], 1)] = i;
    }
}

void launch_query_order(const LaunchCfg &lc, const SpaceParams &sp, const float *qf, int64_t nq, int *work,
                        int64_t *order)
{
    int *count = work, *start = work + kQueryKeys, *fill = work + 2 * kQueryKeys, *key = work + 3 * kQueryKeys;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((nq + 255) / 256, (int64_t)lc.sm_count * 8));
    cudaMemsetAsync(count, 0, kQueryKeys * sizeof(int), lc.stream);
    query_key_kernel<<<grid, 256, 0, lc.stream>>>(sp, qf, nq, nq, nullptr, key, count);
    query_scan_kernel<<<1, 1024, 0, lc.stream>>>(count, start, fill);
    query_scatter_kernel<<<grid, 256, 0, lc.stream>>>(key, nq, start, fill, order);
    for (int i = 0; i < 3; ++i)
        note_launch();
}

// ---------------------------------------------------------------- cell index for box and wrapped spaces
// Large batches over a large RealVector / wrapped index (PRM's prefix kNN): the alive elements are
// bucketed by a uniform grid of L levels per coordinate (counting sort); each cell keeps its elements'
// FP32 coordinates (two float4 per element, sorted by cell) and their bounding box. Queries are
// processed in (band of their prefix limit, cell) order: each query seeds its threshold T with the k-th
// FP32 distance among the eligible elements of its own cell (an upper bound on its k-th overall), and
// skips a cell when the distance from the query to the cell's box is at least min(T, its current
// K_KEEP-th). Elements beyond T are left out of the lists; the FP64 band of the finish kernel lies
// below T, so its decisions are unchanged.

__device__ __forceinline__ void bcell_range(const SpaceParams &sp, int d, float &lo, float &hi)
{
    if (sp.kind == GBO_SPACE_REAL_VECTOR)
    {
        lo = (float)sp.low[d];
        hi = (float)sp.high[d];
    }
    else
    {
        lo = -3.14159265358979f;
        hi = 3.14159265358979f;
    }
}

__device__ __forceinline__ int bcell_of(const SpaceParams &sp, int L, const float *f, int64_t ld, int64_t i)
{
    int c = 0;
    for (int d = sp.dim - 1; d >= 0; --d)
    {
        float lo, hi;
        bcell_range(sp, d, lo, hi);
        int l = hi > lo ? (int)floorf((f[(int64_t)d * ld + i] - lo) * ((float)L / (hi - lo))) : 0;
        l = l < 0 ? 0 : (l >= L ? L - 1 : l);
        c = c * L + l;
    }
    return c;
}

__global__ void bcell_assign_kernel(SpaceParams sp, int L, const float *feat, int64_t cap,
                                    const unsigned char *alive, int64_t n, int *cell, int *count)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        if (!alive[i])
        {
            cell[i] = -1;
            continue;
        }
        const int c = bcell_of(sp, L, feat, cap, i);
        cell[i] = c;
        atomicAdd(&count[c], 1);
    }
}

// Exclusive scan of C counts (one CTA of 1024 threads): start[0..C], fill[] cleared.
__global__ void __launch_bounds__(1024) bcell_scan_kernel(const int *count, int C, int *start, int *fill)
{
    __shared__ int part[1024];
    const int per = (C + 1023) / 1024, i0 = threadIdx.x * per, i1 = min(i0 + per, C);
    int s = 0;
    for (int i = i0; i < i1; ++i)
        s += count[i];
    part[threadIdx.x] = s;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1)
    {
        const int v = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += v;
        __syncthreads();
    }
    int run = part[threadIdx.x] - s;
    for (int i = i0; i < i1; ++i)
    {
        start[i] = run;
        fill[i] = 0;
        run += count[i];
    }
    if (threadIdx.x == 1023)
        start[C] = part[1023];
}

// out[start[c] + arrival order] = i for every row i with c = cell[i] >= 0
__global__ void bcell_scatter_kernel(const int *cell, int64_t n, const int *start, int *fill, int64_t *out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        const int c = cell[i];
        if (c >= 0)
            out[start[c] + atomicAdd(&fill[c], 1)] = i;
    }
}

// sorted coordinates: pts8[2p], pts8[2p + 1] = element skey[p] (unused coordinates 0), p < start[C]
__global__ void bcell_gather_kernel(const int64_t *skey, const int *start, int C, const float *feat, int64_t cap,
                                    int dim, float4 *pts8)
{
    const int64_t total = start[C];
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < total; p += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t key = skey[p];
        float v[8];
#pragma unroll
        for (int d = 0; d < 8; ++d)
            v[d] = d < dim ? feat[(int64_t)d * cap + key] : 0.f;
        pts8[2 * p] = make_float4(v[0], v[1], v[2], v[3]);
        pts8[2 * p + 1] = make_float4(v[4], v[5], v[6], v[7]);
    }
}

// box[c] = 4 float4: min of coordinates 0-3, 4-7, then max (warp per cell)
__global__ void bcell_box_kernel(const float4 *pts8, const int *start, int C, float4 *box)
{
    const int lane = threadIdx.x & 31;
    for (int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); c < C; c += (int)((gridDim.x * blockDim.x) >> 5))
    {
        float mn[8], mx[8];
#pragma unroll
        for (int d = 0; d < 8; ++d)
        {
            mn[d] = __int_as_float(0x7f800000);
            mx[d] = -__int_as_float(0x7f800000);
        }
        for (int p = start[c] + lane; p < start[c + 1]; p += 32)
        {
            const float4 a = pts8[2 * p], b = pts8[2 * p + 1];
            const float v[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
#pragma unroll
            for (int d = 0; d < 8; ++d)
            {
                mn[d] = fminf(mn[d], v[d]);
                mx[d] = fmaxf(mx[d], v[d]);
            }
        }
#pragma unroll
        for (int d = 0; d < 8; ++d)
            for (int o = 16; o > 0; o >>= 1)
            {
                mn[d] = fminf(mn[d], __shfl_xor_sync(0xffffffffu, mn[d], o));
                mx[d] = fmaxf(mx[d], __shfl_xor_sync(0xffffffffu, mx[d], o));
            }
        if (lane == 0)
        {
            box[4 * c] = make_float4(mn[0], mn[1], mn[2], mn[3]);
            box[4 * c + 1] = make_float4(mn[4], mn[5], mn[6], mn[7]);
            box[4 * c + 2] = make_float4(mx[0], mx[1], mx[2], mx[3]);
            box[4 * c + 3] = make_float4(mx[4], mx[5], mx[6], mx[7]);
        }
    }
}

// query key: band then cell. Without prefix limits one band. With them, band 0 holds the queries whose
// limit is below a quarter of the index (left to the prefix scan: few eligible elements, no useful
// threshold; keyed by decreasing limit), bands 1 .. bands - 1 split the rest evenly.
__global__ void bcell_query_key_kernel(SpaceParams sp, int L, int C, const float *qf, int64_t nq,
                                       const int64_t *prefix, int64_t index_n, int bands, int *key, int *count)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += (int64_t)gridDim.x * blockDim.x)
    {
        int band = 0, c;
        if (prefix && bands > 1)
        {
            const int64_t lim = prefix[i] < 0 ? 0 : (prefix[i] > index_n ? index_n : prefix[i]);
            const int64_t q4 = index_n / 4, rest = index_n - q4;
            band = lim < q4 ? 0 : 1 + (int)min((int64_t)bands - 2, (lim - q4) * (bands - 1) / (rest > 0 ? rest : 1));
            // band 0 goes to the prefix scan, whose CTAs scan up to their largest limit: its queries are
            // ordered by decreasing limit (C buckets), so that a CTA's limits are close and the longest
            // CTAs start first
            c = band == 0 ? (C - 1) - (int)min((int64_t)C - 1, lim * C / (q4 > 0 ? q4 : 1))
                          : band * C + bcell_of(sp, L, qf, nq, i);
        }
        else
            c = bcell_of(sp, L, qf, nq, i);
        key[i] = c;
        atomicAdd(&count[c], 1);
    }
}

// distance from query q to the box (lo, hi per coordinate), squared, scaled down by (1 - 1e-5) against
// the rounding of both sides
template <int KIND, int MAXF>
__device__ __forceinline__ float bcell_lb(const float4 *b, const float *q, int dim)
{
    const float4 l0 = b[0], l1 = b[1], h0 = b[2], h1 = b[3];
    const float lo[8] = {l0.x, l0.y, l0.z, l0.w, l1.x, l1.y, l1.z, l1.w};
    const float hi[8] = {h0.x, h0.y, h0.z, h0.w, h1.x, h1.y, h1.z, h1.w};
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < MAXF; ++i)
        if (i < dim)
        {
            const float x = q[i];
            float d;
            if constexpr (KIND == GBO_SPACE_WRAP_L2 || KIND == GBO_SPACE_SO2)
            {
                // nearest point of [lo, hi] on the circle: 0 inside, else the nearer end
                const float a = fabsf(x - lo[i]), c = fabsf(x - hi[i]);
                const float wa = fminf(a, 6.28318530717958647692f - a), wc = fminf(c, 6.28318530717958647692f - c);
                d = (x >= lo[i] && x <= hi[i]) ? 0.f : fminf(wa, wc);
            }
            else
                d = fmaxf(fmaxf(lo[i] - x, x - hi[i]), 0.f);
            s = fmaf(d, d, s);
        }
    return s * (1.0f - 1e-5f);
}

// Cell search, one warp per query: the 32 lanes test 32 cells' boxes at a time and evaluate a needed
// cell's elements 32 at a time, so a warp visits only the cells its own query needs (a lane-per-query
// form, where a warp's 32 queries visit the union of their cells, kept about 10 of 32 lanes busy). The
// kept list is spread over the lanes (WarpList). Seed and thresholds as above: the own cell first, T
// from its k-th distance, then every other cell whose box is nearer than min(T, the list's last entry).
// One list per query (P = 1).
// The kept list spread over a warp: entry j = 32 s + lane in slot s of the lane (S = K_KEEP / 32
// rounded up slots), ascending, unused entries +inf / -1.
template <int K_KEEP>
struct WarpList
{
    static constexpr int S = (K_KEEP + 31) / 32;
    float d[S];
    int k[S];
    __device__ __forceinline__ void init()
    {
#pragma unroll
        for (int s = 0; s < S; ++s)
        {
            d[s] = __int_as_float(0x7f800000);
            k[s] = -1;
        }
    }
    // entry j of the list, in every lane
    __device__ __forceinline__ float at(int j) const
    {
        float v = d[0];
#pragma unroll
        for (int s = 1; s < S; ++s)
            if (j >> 5 == s)
                v = d[s];
        return __shfl_sync(0xffffffffu, v, j & 31);
    }
    __device__ __forceinline__ float last() const { return at(K_KEEP - 1); }
    // inserts (dd, kk) after the entries with a distance <= dd (those kept earlier stay first)
    __device__ __forceinline__ void insert(float dd, int kk, int lane)
    {
        int pos = 0;
#pragma unroll
        for (int s = 0; s < S; ++s)
            pos += __popc(__ballot_sync(0xffffffffu, 32 * s + lane < K_KEEP && d[s] <= dd));
        if (pos >= K_KEEP)
            return;
        float up_d[S];
        int up_k[S];
#pragma unroll
        for (int s = 0; s < S; ++s)
        {
            up_d[s] = __shfl_up_sync(0xffffffffu, d[s], 1);
            up_k[s] = __shfl_up_sync(0xffffffffu, k[s], 1);
            if (s > 0)
            {
                // lane 0 of slot s takes entry 32 s - 1: lane 31 of slot s - 1
                const float cd = __shfl_sync(0xffffffffu, d[s - 1], 31);
                const int ck = __shfl_sync(0xffffffffu, k[s - 1], 31);
                if (lane == 0)
                {
                    up_d[s] = cd;
                    up_k[s] = ck;
                }
            }
        }
#pragma unroll
        for (int s = 0; s < S; ++s)
        {
            const int j = 32 * s + lane;
            if (j >= pos && j < K_KEEP)
            {
                d[s] = j == pos ? dd : up_d[s];
                k[s] = j == pos ? kk : up_k[s];
            }
        }
    }
};

template <int KIND, int K_KEEP>
__global__ void __launch_bounds__(256) knn_bcell_warp_kernel(BoxCellArgs ci, SpaceParams sp, float eps,
                                                             const float *qf, int64_t nq, const int64_t *qorder,
                                                             const int *qcell, const int64_t *prefix, int k,
                                                             float *part_d, int64_t *part_k)
{
    const int lane = threadIdx.x & 31;
    const int64_t qs = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (qs >= nq)
        return;
    const int64_t qi = qorder[qs];
    if (prefix && qcell[qi] < ci.C)
        return;  // band 0 belongs to the prefix scan
    float qfe[8];
#pragma unroll
    for (int f = 0; f < 8; ++f)
        qfe[f] = f < sp.dim ? qf[(int64_t)f * nq + qi] : 0.f;
    const int64_t limit = prefix ? prefix[qi] : INT64_MAX;
    WarpList<K_KEEP> L;
    L.init();
    // one cell's eligible elements, 32 at a time; candidates below `cut` enter the list in lane order
    auto scan_cell = [&](int c, float T) {
        const int s0 = ci.start[c], s1 = ci.start[c + 1];
        for (int p0 = s0; p0 < s1; p0 += 32)
        {
            const int p = p0 + lane;
            float d = __int_as_float(0x7f800000);
            int key = -1;
            if (p < s1)
            {
                const int64_t kk = ci.skey[p];
                if (kk < limit)
                {
                    const float4 a = ci.pts8[2 * (int64_t)p], b = ci.pts8[2 * (int64_t)p + 1];
                    const float pf[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
                    d = box_dist2<KIND, 8>(pf, qfe, sp.dim);
                    key = (int)kk;
                }
            }
            const float last = L.last();
            unsigned m = __ballot_sync(0xffffffffu, d < last && d <= T);
            while (m)
            {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                const float dc = __shfl_sync(0xffffffffu, d, src);
                const int kc = __shfl_sync(0xffffffffu, key, src);
                if (dc < L.last())
                    L.insert(dc, kc, lane);
            }
        }
    };
    // seed: the query's own cell, then T from its k-th distance
    const int oc = qcell[qi] % ci.C;  // the query key is band * C + cell
    scan_cell(oc, __int_as_float(0x7f800000));
    float T = __int_as_float(0x7f800000);
    const float dkk = L.at(k - 1);
    if (dkk < __int_as_float(0x7f800000))
    {
        const float r = sqrtf(dkk) + 2.f * eps;
        T = r * r * (1.0f + 1e-5f);
    }
    for (int cb = 0; cb < ci.C; cb += 32)
    {
        const int c = cb + lane;
        float lb = __int_as_float(0x7f800000);
        if (c < ci.C && c != oc && ci.start[c] != ci.start[c + 1])
            lb = bcell_lb<KIND, 8>(ci.box + 4 * (int64_t)c, qfe, sp.dim);
        unsigned m = __ballot_sync(0xffffffffu, lb < fminf(T, L.last()));
        while (m)
        {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            // the list may have tightened since the cells were tested
            if (__shfl_sync(0xffffffffu, lb, src) < fminf(T, L.last()))
            {
                scan_cell(cb + src, T);
                // T follows the list's k-th distance (the final band only lies lower)
                const float dk = L.at(k - 1);
                if (dk < __int_as_float(0x7f800000))
                {
                    const float r = sqrtf(dk) + 2.f * eps;
                    T = fminf(T, r * r * (1.0f + 1e-5f));
                }
            }
        }
    }
#pragma unroll
    for (int s = 0; s < WarpList<K_KEEP>::S; ++s)
        if (32 * s + lane < K_KEEP)
        {
            part_d[qs * K_KEEP + 32 * s + lane] = L.d[s];
            part_k[qs * K_KEEP + 32 * s + lane] = L.k[s];
        }
}

int bcell_levels(int dim, int64_t n)
{
    // about 40 elements per cell, at most 65536 cells
    int L = 2;
    while (true)
    {
        int64_t c = 1;
        for (int d = 0; d < dim; ++d)
            c *= L + 1;
        if (c > 65536 || c * 40 > n)
            break;
        ++L;
    }
    return L;
}

static int grid_for(const LaunchCfg &lc, int64_t n)
{
    return (int)std::max<int64_t>(1, std::min<int64_t>((n + 255) / 256, (int64_t)lc.sm_count * 8));
}

void launch_bcell_build(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, int L, int C, int *cell,
                        int *count, int *start, int *fill, int64_t *skey, float4 *pts8, float4 *box)
{
    cudaMemsetAsync(count, 0, (size_t)C * sizeof(int), lc.stream);
    bcell_assign_kernel<<<grid_for(lc, nn.size), 256, 0, lc.stream>>>(sp, L, nn.feat32, nn.cap, nn.alive, nn.size,
                                                                      cell, count);
    bcell_scan_kernel<<<1, 1024, 0, lc.stream>>>(count, C, start, fill);
    bcell_scatter_kernel<<<grid_for(lc, nn.size), 256, 0, lc.stream>>>(cell, nn.size, start, fill, skey);
    bcell_gather_kernel<<<grid_for(lc, nn.size), 256, 0, lc.stream>>>(skey, start, C, nn.feat32, nn.cap, sp.dim,
                                                                      pts8);
    bcell_box_kernel<<<grid_for(lc, (int64_t)C * 32), 256, 0, lc.stream>>>(pts8, start, C, box);
    for (int i = 0; i < 5; ++i)
        note_launch();
}

void launch_bcell_query_order(const LaunchCfg &lc, const SpaceParams &sp, int L, int C, const float *qf, int64_t nq,
                              const int64_t *prefix, int64_t index_n, int bands, int *qcell, int *count, int *start,
                              int *fill, int64_t *qorder)
{
    const int keys = bands * C;
    cudaMemsetAsync(count, 0, (size_t)keys * sizeof(int), lc.stream);
    bcell_query_key_kernel<<<grid_for(lc, nq), 256, 0, lc.stream>>>(sp, L, C, qf, nq, prefix, index_n, bands, qcell,
                                                                    count);
    bcell_scan_kernel<<<1, 1024, 0, lc.stream>>>(count, keys, start, fill);
    bcell_scatter_kernel<<<grid_for(lc, nq), 256, 0, lc.stream>>>(qcell, nq, start, fill, qorder);
    for (int i = 0; i < 3; ++i)
        note_launch();
}

template <int KIND, int K_KEEP>
static void launch_bcell_t(const LaunchCfg &lc, const NNArgs &nn, const BoxCellArgs &ci, const SpaceParams &sp,
                           StatesView qv, const float *qf, int64_t nq, const int64_t *qorder, const int *qcell, int k,
                           const int64_t *prefix, int64_t *idx, double *dist, unsigned long long *fb_list,
                           unsigned long long *fb_n, RunCounters *ctr, float *part_d, int64_t *part_k)
{
    // one list per query (P = 1): the warp kernel visits every cell a query needs, and the prefix scan
    // of band 0 covers each of its queries' limits in one CTA
    const int qb = (int)((nq + 127) / 128), P = 1;
    knn_bcell_warp_kernel<KIND, K_KEEP><<<(int)((nq * 32 + 255) / 256), 256, 0, lc.stream>>>(
        ci, sp, nn.eps32, qf, nq, qorder, qcell, prefix, k, part_d, part_k);
    if (prefix)
    {
        // band 0 (limits below a quarter of the index) through the prefix scan, same P lists
        knn_scan_kernel<KIND, 8, K_KEEP><<<dim3(qb, P), 128, 0, lc.stream>>>(nn, sp, qf, nq, prefix,
                                                                            (nn.size + P - 1) / P, part_d, part_k,
                                                                            qorder, qcell, ci.C, nullptr);
        note_launch();
    }
    knn_finish_kernel<KIND, 8, K_KEEP><<<qb, 128, 0, lc.stream>>>(nn, sp, qv, nq, k, P, part_d, part_k, idx, dist,
                                                                 fb_list, fb_n, ctr, qorder);
    note_launch();
    note_launch();
}

bool launch_knn_bcell(const LaunchCfg &lc, const NNArgs &nn, const BoxCellArgs &ci, const SpaceParams &sp,
                      StatesView qv, const float *qf, int64_t nq, const int64_t *qorder, const int *qcell, int k,
                      const int64_t *prefix, int64_t *idx, double *dist, unsigned long long *fb_list,
                      unsigned long long *fb_n, RunCounters *ctr, float *part_d, int64_t *part_k)
{
    if (nq == 0 || sp.dim > 8 || k > knn_fp32_max_k(sp))
        return false;
#define GBO_BCELL_T(KIND, KK)                                                                                         \
    launch_bcell_t<KIND, KK>(lc, nn, ci, sp, qv, qf, nq, qorder, qcell, k, prefix, idx, dist, fb_list, fb_n, ctr,     \
                             part_d, part_k)
#define GBO_BCELL(KIND)                                                                                                \
    do                                                                                                                \
    {                                                                                                                 \
        if (k <= 12)                                                                                                  \
            GBO_BCELL_T(KIND, 16);                                                                                    \
        else if (k <= 20)                                                                                             \
            GBO_BCELL_T(KIND, 24);                                                                                    \
        else if (k <= 40)                                                                                             \
            GBO_BCELL_T(KIND, 48);                                                                                    \
        else                                                                                                          \
            GBO_BCELL_T(KIND, 72);                                                                                    \
    } while (0)
    if (sp.kind == GBO_SPACE_WRAP_L2)
        GBO_BCELL(GBO_SPACE_WRAP_L2);
    else if (sp.kind == GBO_SPACE_REAL_VECTOR)
        GBO_BCELL(GBO_SPACE_REAL_VECTOR);
    else
        return false;
#undef GBO_BCELL_T
#undef GBO_BCELL
    return true;
}


// ---------------------------------------------------------------- cell index for the chain metric
// Elements bucketed by the same key as the query order (the tip and middle-joint points, 8 levels per
// coordinate: kQueryKeys cells); per cell the elements' features (20 floats in five planes of float4,
// plane j holding features 4j..4j+3 of every sorted position, so that a warp's 32 elements read 512
// contiguous bytes per plane and the planes of links 4..9 form the search's hot set) and their box
// (per feature the minimum and maximum). The box bounds the chain distance from below:
// L * sum_i |(X_i, Y_i)(q) - box_i| <= L * sum_i |(X_i, Y_i)(q) - (X_i, Y_i)(e)| for every element e
// of the cell (scaled by 1 - 1e-5 against the rounding of both sides, which see the same features).
// The search is the warp-per-query one of the box kinds: own cell first (threshold seed), then the
// cells whose bound is below min(T, the list's last entry).
__global__ void ccell_gather_kernel(const int64_t *skey, const int *start, const int *count, const float *feat,
                                    int64_t cap, int F, int64_t n, float4 *sfeat)
{
    const int64_t total = (int64_t)start[kQueryKeys - 1] + count[kQueryKeys - 1];
    const int64_t m = min(n, total);
    for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < m; p += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t key = skey[p];
        float v[20];
#pragma unroll
        for (int f = 0; f < 20; ++f)
            v[f] = f < F ? feat[(int64_t)f * cap + key] : 0.f;
#pragma unroll
        for (int j = 0; j < 5; ++j)
            sfeat[(int64_t)j * n + p] = make_float4(v[4 * j], v[4 * j + 1], v[4 * j + 2], v[4 * j + 3]);
    }
}

// A chain box in 80 bytes: feature f's (minimum, maximum) as a half2 rounded outward (minimum down,
// maximum up, so that the half box contains the float one and every distance bound computed from it
// is still a lower bound; values beyond the half range become the largest finite half or infinity on
// the safe side), features 4j .. 4j+3 in uint4 j.
__device__ __forceinline__ uint4 pack_box4(float4 lo, float4 hi)
{
    auto pk = [](float l, float h) {
        const __half2 v = __halves2half2(__float2half_rd(l), __float2half_ru(h));
        return *(const unsigned *)&v;
    };
    return make_uint4(pk(lo.x, hi.x), pk(lo.y, hi.y), pk(lo.z, hi.z), pk(lo.w, hi.w));
}

// box of cell c: five uint4 (pack_box4) (warp per cell)
__global__ void ccell_box_kernel(const float4 *sfeat, int64_t fs, const int *start, const int *count, uint4 *box)
{
    const int lane = threadIdx.x & 31;
    for (int c = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); c < kQueryKeys;
         c += (int)((gridDim.x * blockDim.x) >> 5))
    {
        float mn[20], mx[20];
#pragma unroll
        for (int f = 0; f < 20; ++f)
        {
            mn[f] = __int_as_float(0x7f800000);
            mx[f] = -__int_as_float(0x7f800000);
        }
        for (int p = start[c] + lane; p < start[c] + count[c]; p += 32)
        {
#pragma unroll
            for (int j = 0; j < 5; ++j)
            {
                const float4 a = sfeat[(int64_t)j * fs + p];
                const float v[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
                for (int t = 0; t < 4; ++t)
                {
                    mn[4 * j + t] = fminf(mn[4 * j + t], v[t]);
                    mx[4 * j + t] = fmaxf(mx[4 * j + t], v[t]);
                }
            }
        }
#pragma unroll
        for (int f = 0; f < 20; ++f)
            for (int o = 16; o > 0; o >>= 1)
            {
                mn[f] = fminf(mn[f], __shfl_xor_sync(0xffffffffu, mn[f], o));
                mx[f] = fmaxf(mx[f], __shfl_xor_sync(0xffffffffu, mx[f], o));
            }
        if (lane < 5)
        {
            const float *m0 = mn + 0, *m1 = mx + 0;
            float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
#pragma unroll
            for (int j = 0; j < 5; ++j)
                if (j == lane)
                {
                    lo = make_float4(m0[4 * j], m0[4 * j + 1], m0[4 * j + 2], m0[4 * j + 3]);
                    hi = make_float4(m1[4 * j], m1[4 * j + 1], m1[4 * j + 2], m1[4 * j + 3]);
                }
            box[5 * (int64_t)c + lane] = pack_box4(lo, hi);
        }
    }
}

// Inside a cell, elements are ordered by a Morton code of two more joints (levels 0..31 of x and y of joints
// dim/4 and 3 dim/4, bits interleaved), then by key, so that runs of kChunk consecutive elements
// ("chunks") are close in those joints and their boxes bound the distance more tightly than the cell's. One
// CTA per cell sorts (code, key) pairs in shared memory (bitonic sort); cells of more than kSortMax
// elements keep the scatter's order (still exact, the chunk boxes are only looser).
constexpr int kSortMax = 16384;
constexpr int kChunk = 32;  // elements per chunk: one chunk per warp step (16 per chunk, two chunks a step,
                            // visited fewer elements but took 10% longer)

__device__ __forceinline__ unsigned ccell_code(const SpaceParams &sp, const float *feat, int64_t cap, int64_t key)
{
    const int joints[2] = {sp.dim / 4, (3 * sp.dim) / 4};
    unsigned lv[4];
#pragma unroll
    for (int t = 0; t < 2; ++t)
    {
        const float r = 2.5f * sqrtf(0.5f * (float)(joints[t] + 1));
#pragma unroll
        for (int c = 0; c < 2; ++c)
        {
            const float v = feat[(int64_t)(2 * joints[t] + c) * cap + key];
            int l = (int)floorf((v + r) * (32.0f / (2.0f * r)));
            lv[2 * t + c] = (unsigned)(l < 0 ? 0 : (l > 31 ? 31 : l));
        }
    }
    unsigned code = 0;
#pragma unroll
    for (int b = 4; b >= 0; --b)
#pragma unroll
        for (int t = 0; t < 4; ++t)
            code = (code << 1) | ((lv[t] >> b) & 1u);
    return code;
}

__global__ void __launch_bounds__(512) ccell_sort_kernel(SpaceParams sp, const float *feat, int64_t cap,
                                                         const int *start, const int *count, int64_t *skey)
{
    extern __shared__ unsigned long long sv[];
    const int c = blockIdx.x, n = count[c], s0 = start[c];
    if (n < 2 || n > kSortMax)
        return;
    int np = 1;
    while (np < n)
        np <<= 1;
    for (int i = threadIdx.x; i < np; i += blockDim.x)
    {
        unsigned long long v = ~0ull;
        if (i < n)
        {
            const int64_t key = skey[s0 + i];
            v = ((unsigned long long)ccell_code(sp, feat, cap, key) << 32) | (unsigned long long)(unsigned)key;
        }
        sv[i] = v;
    }
    __syncthreads();
    for (int k = 2; k <= np; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1)
        {
            for (int i = threadIdx.x; i < np; i += blockDim.x)
            {
                const int ixj = i ^ j;
                if (ixj > i)
                {
                    const unsigned long long a = sv[i], b = sv[ixj];
                    if ((a > b) == ((i & k) == 0))
                    {
                        sv[i] = b;
                        sv[ixj] = a;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x)
        skey[s0 + i] = (int64_t)(unsigned)(sv[i] & 0xffffffffull);
}

// first chunk of each cell: exclusive scan of ceil(count / kChunk) over the 4096 cells (one CTA of 1024)
__global__ void __launch_bounds__(1024) ccell_chunk_scan_kernel(const int *count, int *cstart)
{
    __shared__ int part[1024];
    const int i0 = threadIdx.x * 4;
    int v[4], sum = 0;
#pragma unroll
    for (int t = 0; t < 4; ++t)
    {
        v[t] = (count[i0 + t] + kChunk - 1) / kChunk;
        sum += v[t];
    }
    part[threadIdx.x] = sum;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1)
    {
        const int x = threadIdx.x >= o ? part[threadIdx.x - o] : 0;
        __syncthreads();
        part[threadIdx.x] += x;
        __syncthreads();
    }
    int run = part[threadIdx.x] - sum;
#pragma unroll
    for (int t = 0; t < 4; ++t)
    {
        cstart[i0 + t] = run;
        run += v[t];
    }
    if (threadIdx.x == 1023)
        cstart[kQueryKeys] = part[1023];
}

// box of each chunk (warp per chunk, lane per element): five uint4 (pack_box4)
__global__ void ccell_chunk_box_kernel(const float4 *sfeat, int64_t fs, const int *start, const int *count,
                                       const int *cstart, uint4 *cbox)
{
    const int lane = threadIdx.x & 31;
    const int nchunks = cstart[kQueryKeys];
    for (int ch = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); ch < nchunks;
         ch += (int)((gridDim.x * blockDim.x) >> 5))
    {
        // the cell of chunk ch: the last c with cstart[c] <= ch (binary search)
        int lo = 0, hi = kQueryKeys - 1;
        while (lo < hi)
        {
            const int mid = (lo + hi + 1) >> 1;
            if (cstart[mid] <= ch)
                lo = mid;
            else
                hi = mid - 1;
        }
        const int c = lo;
        const int p0 = start[c] + kChunk * (ch - cstart[c]), p1 = min(p0 + kChunk, start[c] + count[c]);
        const int p = p0 + lane;
        float v[20];
#pragma unroll
        for (int j = 0; j < 5; ++j)
        {
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f);
            if (p < p1)
                a = sfeat[(int64_t)j * fs + p];
            v[4 * j] = a.x;
            v[4 * j + 1] = a.y;
            v[4 * j + 2] = a.z;
            v[4 * j + 3] = a.w;
        }
        float mn[20], mx[20];
#pragma unroll
        for (int f = 0; f < 20; ++f)
        {
            mn[f] = p < p1 ? v[f] : __int_as_float(0x7f800000);
            mx[f] = p < p1 ? v[f] : -__int_as_float(0x7f800000);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1)
            {
                mn[f] = fminf(mn[f], __shfl_xor_sync(0xffffffffu, mn[f], o));
                mx[f] = fmaxf(mx[f], __shfl_xor_sync(0xffffffffu, mx[f], o));
            }
        }
        if (lane < 5)
        {
            float4 lo = make_float4(0.f, 0.f, 0.f, 0.f), hi = lo;
#pragma unroll
            for (int j = 0; j < 5; ++j)
                if (j == lane)
                {
                    lo = make_float4(mn[4 * j], mn[4 * j + 1], mn[4 * j + 2], mn[4 * j + 3]);
                    hi = make_float4(mx[4 * j], mx[4 * j + 1], mx[4 * j + 2], mx[4 * j + 3]);
                }
            cbox[5 * (int64_t)ch + lane] = pack_box4(lo, hi);
        }
    }
}

void launch_ccell_build(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, int *key, int *count,
                        int *start, int *fill, int64_t *skey, float4 *sfeat, uint4 *box, int *cstart, uint4 *cbox)
{
    const int grid = grid_for(lc, nn.size);
    cudaMemsetAsync(count, 0, kQueryKeys * sizeof(int), lc.stream);
    query_key_kernel<<<grid, 256, 0, lc.stream>>>(sp, nn.feat32, nn.cap, nn.size, nn.alive, key, count);
    query_scan_kernel<<<1, 1024, 0, lc.stream>>>(count, start, fill);
    query_scatter_kernel<<<grid, 256, 0, lc.stream>>>(key, nn.size, start, fill, skey);
    const int smem = kSortMax * (int)sizeof(unsigned long long);
    cudaFuncSetAttribute(ccell_sort_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    ccell_sort_kernel<<<kQueryKeys, 512, smem, lc.stream>>>(sp, nn.feat32, nn.cap, start, count, skey);
    ccell_gather_kernel<<<grid, 256, 0, lc.stream>>>(skey, start, count, nn.feat32, nn.cap, 2 * sp.dim, nn.size,
                                                     sfeat);
    ccell_box_kernel<<<(kQueryKeys * 32 + 255) / 256, 256, 0, lc.stream>>>(sfeat, nn.size, start, count, box);
    ccell_chunk_scan_kernel<<<1, 1024, 0, lc.stream>>>(count, cstart);
    ccell_chunk_box_kernel<<<lc.sm_count * 8, 256, 0, lc.stream>>>(sfeat, nn.size, start, count, cstart, cbox);
    for (int i = 0; i < 8; ++i)
        note_launch();
}

// chain distance from query features q to a cell's or chunk's box (pack_box4 layout), before the scale by
// the link length
__device__ __forceinline__ float ccell_lb(const uint4 *b, const float *q, int dim)
{
    float s = 0.f;
#pragma unroll
    for (int j = 0; j < 5; ++j)
    {
        const uint4 w = b[j];
        const unsigned u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int t = 0; t < 4; t += 2)
        {
            const int i = (4 * j + t) / 2;  // link
            if (i < dim)
            {
                const float2 bx = __half22float2(*(const __half2 *)&u[t]);      // (min, max) of x
                const float2 by = __half22float2(*(const __half2 *)&u[t + 1]);  // (min, max) of y
                const float dx = fmaxf(fmaxf(bx.x - q[4 * j + t], q[4 * j + t] - bx.y), 0.f);
                const float dy = fmaxf(fmaxf(by.x - q[4 * j + t + 1], q[4 * j + t + 1] - by.y), 0.f);
                s += sqrt_approx(fmaf(dx, dx, dy * dy));
            }
        }
    }
    return s;
}

// 3 CTAs per SM: 80 registers without spills (the default choice, 64 registers for 4 CTAs, spilled)
template <int K_KEEP>
__global__ void __launch_bounds__(256, 3) knn_ccell_warp_kernel(ChainCellArgs ci, SpaceParams sp, float eps,
                                                             const float *qf, int64_t nq, const int64_t *qorder,
                                                             const int *qkey, int k, float *part_d, int64_t *part_k,
                                                             RunCounters *ctr)
{
    const int lane = threadIdx.x & 31;
    const int64_t qs = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (qs >= nq)
        return;
    const int64_t qi = qorder[qs];
    const int F = 2 * sp.dim;
    float qfe[20];
#pragma unroll
    for (int f = 0; f < 20; ++f)
        qfe[f] = f < F ? qf[(int64_t)f * nq + qi] : 0.f;
    const float link = (float)sp.link;
    WarpList<K_KEEP> L;
    L.init();
    unsigned long long nbytes = 0;  // feature and box bytes read for this query (lane 0)
    // Elements whose outer-link partial passes wait in a per-warp ring of 64 (position and partial) until
    // 32 are queued (or the cell ends); their inner links are then read and summed one element per lane,
    // so that this stage runs with full warps instead of for the few passing lanes of every chunk. A
    // queued element is tested again against the list and T of the moment, which only lie lower.
    __shared__ int wq_pos[8][64];
    __shared__ float wq_outer[8][64];
    int *qp = wq_pos[threadIdx.x >> 5];
    float *qo = wq_outer[threadIdx.x >> 5];
    int qhead = 0, qn = 0;  // warp-uniform
    auto flush = [&](int cnt, float T) {
        __syncwarp();  // the queued entries are written
        const int slot = (qhead + lane) & 63;
        const int p = lane < cnt ? qp[slot] : 0;
        const float outer = lane < cnt ? qo[slot] : 0.f;
        __syncwarp();  // and read before later chunks reuse their slots
        qhead += cnt;
        qn -= cnt;
        float d = __int_as_float(0x7f800000);
        int key = -1;
        const float last = L.last();
        if (lane < cnt && outer * link < last && outer * link <= T)
        {
            float pf[8];
#pragma unroll
            for (int j = 0; j < 2; ++j)
            {
                const float4 a = ci.sfeat[(int64_t)j * ci.fs + p];
                pf[4 * j] = a.x;
                pf[4 * j + 1] = a.y;
                pf[4 * j + 2] = a.z;
                pf[4 * j + 3] = a.w;
            }
            float inner = 0.f;
#pragma unroll
            for (int i = 0; i < 4; ++i)
                if (i < sp.dim)
                {
                    const float dx = pf[2 * i] - qfe[2 * i], dy = pf[2 * i + 1] - qfe[2 * i + 1];
                    inner += sqrt_approx(fmaf(dx, dx, dy * dy));
                }
            d = (inner + outer) * link;
            key = (int)ci.skey[p];
        }
        unsigned m = __ballot_sync(0xffffffffu, d < last && d <= T);
        while (m)
        {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            const float dc = __shfl_sync(0xffffffffu, d, src);
            const int kc = __shfl_sync(0xffffffffu, key, src);
            if (dc < L.last())
                L.insert(dc, kc, lane);
        }
    };
    // the elements of one chunk (positions p0 .. s1 - 1, at most 32), one lane each: links 4.. first
    // (features 8-19), whose terms are the largest; the rest (features 0-7) is read only when the element
    // can still enter the list (flush). Terms are non-negative and FP32 addition is monotone, so the full
    // sum is at least the partial one.
    auto scan_chunk = [&](int p0, int s1, float T) {
        const int p = p0 + lane;
        const float last = L.last();
        float outer = 0.f;
        bool pass = false;
        if (p < s1)
        {
            float pf[20];
#pragma unroll
            for (int j = 2; j < 5; ++j)
            {
                const float4 a = ci.sfeat[(int64_t)j * ci.fs + p];
                pf[4 * j] = a.x;
                pf[4 * j + 1] = a.y;
                pf[4 * j + 2] = a.z;
                pf[4 * j + 3] = a.w;
            }
#pragma unroll
            for (int i = 4; i < 10; ++i)
                if (i < sp.dim)
                {
                    const float dx = pf[2 * i] - qfe[2 * i], dy = pf[2 * i + 1] - qfe[2 * i + 1];
                    outer += sqrt_approx(fmaf(dx, dx, dy * dy));
                }
            pass = outer * link < last && outer * link <= T;
        }
        const unsigned pm = __ballot_sync(0xffffffffu, pass);
        if (pass)
        {
            const int slot = (qhead + qn + __popc(pm & ((1u << lane) - 1u))) & 63;
            qp[slot] = p;
            qo[slot] = outer;
        }
        qn += __popc(pm);
        if (qn >= 32)
            flush(32, T);
    };
    // a cell: its chunks' boxes (lanes over chunks), then the elements of the chunks whose bound is below
    // min(T, the list's last entry), rechecked against the bound of the moment
    auto scan_cell = [&](int c, float T) {
        const int s0 = ci.start[c], s1 = s0 + ci.count[c];
        const int c0 = ci.cstart[c], c1 = ci.cstart[c + 1];
        for (int cb = c0; cb < c1; cb += 32)
        {
            const int ch = cb + lane;
            float lb = __int_as_float(0x7f800000);
            if (ch < c1)
                lb = ccell_lb(ci.cbox + 5 * (int64_t)ch, qfe, sp.dim) * link * (1.0f - 1e-5f);
            nbytes += 80ull * (unsigned)min(32, c1 - cb);
            unsigned m = __ballot_sync(0xffffffffu, lb < fminf(T, L.last()));
            while (m)
            {
                const int src = __ffs(m) - 1;
                m &= m - 1;
                if (__shfl_sync(0xffffffffu, lb, src) < fminf(T, L.last()))
                {
                    const int p0 = s0 + kChunk * (cb + src - c0), p1 = min(p0 + kChunk, s1);
                    nbytes += 48ull * (unsigned)(p1 - p0);  // links 4.. of each element (inner links not counted)
                    scan_chunk(p0, p1, T);
                }
            }
        }
        if (qn > 0)
            flush(qn, T);
    };
    const int own = qkey[qi];
    scan_cell(own, __int_as_float(0x7f800000));
    float T = __int_as_float(0x7f800000);
    // T follows the list's k-th distance (the final band only lies lower)
    auto tighten = [&]() {
        const float dk = L.at(k - 1);
        if (dk < __int_as_float(0x7f800000))
            T = fminf(T, (dk + 2.f * eps) * (1.0f + 1e-5f));
    };
    tighten();
    // key digits (3 bits each): tip x, tip y, middle x, middle y; the 80 cells next to the own cell in
    // that grid come next, so that the list holds near neighbours before the pass over all cells
    auto near_own = [&](int c) {
        bool nb = true;
#pragma unroll
        for (int t = 0; t < 4; ++t)
        {
            const int dl = ((c >> (3 * t)) & 7) - ((own >> (3 * t)) & 7);
            nb &= dl >= -1 && dl <= 1;
        }
        return nb;
    };
    auto visit = [&](int c, bool ok) {
        float lb = __int_as_float(0x7f800000);
        if (ok && ci.count[c] > 0)
            lb = ccell_lb(ci.box + 5 * (int64_t)c, qfe, sp.dim) * link * (1.0f - 1e-5f);
        nbytes += 80ull * __popc(__ballot_sync(0xffffffffu, lb < __int_as_float(0x7f800000)));
        unsigned m = __ballot_sync(0xffffffffu, lb < fminf(T, L.last()));
        while (m)
        {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            if (__shfl_sync(0xffffffffu, lb, src) < fminf(T, L.last()))
            {
                scan_cell(__shfl_sync(0xffffffffu, c, src), T);
                tighten();
            }
        }
    };
    for (int j0 = 0; j0 < 81; j0 += 32)
    {
        // offset j in base 3: digit t in {0, 1, 2} moves digit t of the key by -1, 0, +1
        const int j = j0 + lane;
        int c = 0, rem = j;
        bool ok = j < 81 && j != 40;  // 40: no move (the own cell)
#pragma unroll
        for (int t = 0; t < 4; ++t)
        {
            const int l = ((own >> (3 * t)) & 7) + (rem % 3) - 1;
            rem /= 3;
            ok &= l >= 0 && l < 8;
            c |= (l & 7) << (3 * t);
        }
        visit(ok ? c : 0, ok);
    }
    for (int cb = 0; cb < kQueryKeys; cb += 32)
    {
        const int c = cb + lane;
        float lb = __int_as_float(0x7f800000);
        if (!near_own(c) && ci.count[c] > 0)
            lb = ccell_lb(ci.box + 5 * (int64_t)c, qfe, sp.dim) * link * (1.0f - 1e-5f);
        nbytes += 80ull * __popc(__ballot_sync(0xffffffffu, lb < __int_as_float(0x7f800000)));
        unsigned m = __ballot_sync(0xffffffffu, lb < fminf(T, L.last()));
        while (m)
        {
            const int src = __ffs(m) - 1;
            m &= m - 1;
            if (__shfl_sync(0xffffffffu, lb, src) < fminf(T, L.last()))
            {
                scan_cell(cb + src, T);
                tighten();
            }
        }
    }
#pragma unroll
    for (int s = 0; s < WarpList<K_KEEP>::S; ++s)
        if (32 * s + lane < K_KEEP)
        {
            part_d[qs * K_KEEP + 32 * s + lane] = L.d[s];
            part_k[qs * K_KEEP + 32 * s + lane] = L.k[s];
        }
    if (lane == 0 && ctr)
        atomicAdd(&ctr->bytes, nbytes);
}

bool launch_knn_ccell(const LaunchCfg &lc, const NNArgs &nn, const ChainCellArgs &ci, const SpaceParams &sp,
                      StatesView qv, const float *qf, int64_t nq, const int64_t *qorder, const int *qkey, int k,
                      int64_t *idx, double *dist, unsigned long long *fb_list, unsigned long long *fb_n,
                      RunCounters *ctr, float *part_d, int64_t *part_k)
{
    if (nq == 0 || sp.kind != GBO_SPACE_KINEMATIC_CHAIN || sp.dim > 10 || k > 20)
        return false;
    const int qb = (int)((nq + 127) / 128), wg = (int)((nq * 32 + 255) / 256);
    if (k <= 12)
    {
        knn_ccell_warp_kernel<16><<<wg, 256, 0, lc.stream>>>(ci, sp, nn.eps32, qf, nq, qorder, qkey, k, part_d, part_k,
                                                             ctr);
        knn_finish_kernel<GBO_SPACE_KINEMATIC_CHAIN, 10, 16><<<qb, 128, 0, lc.stream>>>(
            nn, sp, qv, nq, k, 1, part_d, part_k, idx, dist, fb_list, fb_n, ctr, qorder);
    }
    else
    {
        knn_ccell_warp_kernel<24><<<wg, 256, 0, lc.stream>>>(ci, sp, nn.eps32, qf, nq, qorder, qkey, k, part_d, part_k,
                                                             ctr);
        knn_finish_kernel<GBO_SPACE_KINEMATIC_CHAIN, 10, 24><<<qb, 128, 0, lc.stream>>>(
            nn, sp, qv, nq, k, 1, part_d, part_k, idx, dist, fb_list, fb_n, ctr, qorder);
    }
    note_launch();
    note_launch();
    return true;
}

}  // namespace gbo
