// Nearest-neighbour kernels behind NearestNeighbors<T>::nearestK / nearestR.
//
// Result order is (FP64 distance, key), key = insertion index: the order NearestNeighborsLinear
// produces (NearestNeighborsLinear.h:119-142) whenever distances are distinct, with ties resolved by
// insertion order. distance is evaluated as distance(element, query) (ElemSort, :159-172).
//
//   knn_exact_kernel  FP64, one warp per query: lanes scan keys lane, lane+32, ... keeping a sorted
//                     register top-k; the warp then merges the 32 lists with shuffle argmin rounds.
//   knn_fp32_kernel   FP32 bulk, one thread per query, element features staged in shared memory
//                     tiles; keeps the best K_KEEP by FP32 distance. Every kept element within
//                     2*eps of the k-th FP32 distance is re-evaluated in FP64 and the final order is
//                     decided in FP64. If more than K_KEEP elements fall in that band the query is
//                     queued for knn_exact_kernel (FP64 scan).
//   radius kernels    FP64 count / fill (CSR), sorted by (distance, key).
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
template <int K, class T>
__device__ __forceinline__ void topk_insert(T *dk, int64_t *ik, T d, int64_t key)
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
        const double d = distance64<MAXD>(sp, x, q);
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
// cumulative link-direction sums (X_1..X_n, Y_1..Y_n), F = 2 dim, so that
// distance = L * sum_i |(X_i(a) - X_i(b), Y_i(a) - Y_i(b))|.
template <int KIND, int MAXF>
__device__ __forceinline__ float dist32_sq_or_d(const float *a, const float *b, int dim, float &lower)
{
    if constexpr (KIND == GBO_SPACE_KINEMATIC_CHAIN)
    {
        // lower bound sum_i (|dx_i| + |dy_i|) / sqrt(2) <= sum_i |(dx_i, dy_i)| (no sqrt needed)
        float l1 = 0.f;
#pragma unroll
        for (int i = 0; i < MAXF / 2; ++i)
            if (i < dim)
                l1 += fabsf(a[i] - b[i]) + fabsf(a[i + dim] - b[i + dim]);
        lower = l1;
        return 0.f;
    }
    else
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
        lower = s;
        return s;
    }
}

__device__ __forceinline__ float sqrt_approx(float x)
{
    float r;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}

template <int KIND, int MAXF>
__device__ __forceinline__ float chain_dist32(const float *a, const float *b, int dim)
{
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < MAXF / 2; ++i)
        if (i < dim)
        {
            const float dx = a[i] - b[i], dy = a[i + dim] - b[i + dim];
            s += sqrt_approx(fmaf(dx, dx, dy * dy));
        }
    return s;
}

template <int KIND, int MAXD, int MAXF, int K_KEEP>
__global__ void __launch_bounds__(128) knn_fp32_kernel(NNArgs nn, SpaceParams sp, StatesView qv, const float *qf,
                                                       int64_t nq, int k, const int64_t *prefix, int64_t *idx,
                                                       double *dist, unsigned long long *fb_list,
                                                       unsigned long long *fb_n, RunCounters *ctr)
{
    constexpr int TILE = 128;
    __shared__ float tile[MAXF][TILE];
    __shared__ unsigned char tile_alive[TILE];
    __shared__ int64_t s_limit;
    const int F = KIND == GBO_SPACE_KINEMATIC_CHAIN ? 2 * sp.dim : sp.dim;
    const int64_t qi = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool active = qi < nq;
    float qfe[MAXF];
#pragma unroll
    for (int f = 0; f < MAXF; ++f)
        qfe[f] = (active && f < F) ? qf[(int64_t)f * nq + qi] : 0.f;
    int64_t limit = nn.size;
    if (active && prefix)
        limit = min(limit, prefix[qi]);
    if (threadIdx.x == 0)
        s_limit = 0;
    __syncthreads();
    if (active)
        atomicMax((unsigned long long *)&s_limit, (unsigned long long)limit);
    __syncthreads();
    const int64_t block_limit = s_limit;

    float dk[K_KEEP];
    int64_t ik[K_KEEP];
#pragma unroll
    for (int j = 0; j < K_KEEP; ++j)
    {
        dk[j] = __int_as_float(0x7f800000);
        ik[j] = -1;
    }
    const float lb_scale = KIND == GBO_SPACE_KINEMATIC_CHAIN ? 0.70710678f * (1.0f - 1e-5f) : 1.0f;
    for (int64_t base = 0; base < block_limit; base += TILE)
    {
        __syncthreads();
        for (int t = threadIdx.x; t < TILE; t += blockDim.x)
        {
            const int64_t key = base + t;
            const bool in = key < block_limit;
            tile_alive[t] = in ? nn.alive[key] : 0;
#pragma unroll
            for (int f = 0; f < MAXF; ++f)
                if (f < F)
                    tile[f][t] = in ? nn.feat32[(int64_t)f * nn.cap + key] : 0.f;
        }
        __syncthreads();
        if (!active)
            continue;
        const int tn = (int)min((int64_t)TILE, limit - base);
        for (int t = 0; t < tn; ++t)
        {
            if (!tile_alive[t])
                continue;
            float pf[MAXF];
#pragma unroll
            for (int f = 0; f < MAXF; ++f)
                pf[f] = f < F ? tile[f][t] : 0.f;
            float lower;
            float d = dist32_sq_or_d<KIND, MAXF>(pf, qfe, sp.dim, lower);
            if constexpr (KIND == GBO_SPACE_KINEMATIC_CHAIN)
            {
                if (lower * lb_scale * (float)sp.link >= dk[K_KEEP - 1])
                    continue;
                d = chain_dist32<KIND, MAXF>(pf, qfe, sp.dim) * (float)sp.link;
            }
            if (d < dk[K_KEEP - 1])
                topk_insert<K_KEEP>(dk, ik, d, base + t);
        }
    }
    if (!active)
        return;
    // Re-check band in FP64. For squared-distance kinds the band is applied on squared values.
    const float eps = nn.eps32;
    const float kth = dk[k - 1 < K_KEEP ? k - 1 : K_KEEP - 1];
    float band;
    if constexpr (KIND == GBO_SPACE_KINEMATIC_CHAIN)
        band = kth + 2.f * eps;
    else
    {
        const float r = sqrtf(kth) + 2.f * eps;
        band = r * r * (1.0f + 1e-6f);
    }
    const int64_t live = min(limit, (int64_t)nn.size);  // upper bound on candidates
    (void)live;
    if (k < K_KEEP && !(dk[K_KEEP - 1] > band) && ik[K_KEEP - 1] >= 0)
    {
        // more than K_KEEP elements may lie in the band: exact scan
        const unsigned long long pos = atomicAdd(fb_n, 1ull);
        fb_list[pos] = (unsigned long long)qi;
        atomicAdd(&ctr->fallbacks, 1ull);
        return;
    }
    double q64[MAXD];
    load_query<MAXD>(qv, qi, sp.dim, q64);
    double d64[K_KEEP];
    int64_t k64[K_KEEP];
    int nc = 0;
#pragma unroll
    for (int j = 0; j < K_KEEP; ++j)
    {
        d64[j] = __longlong_as_double(0x7ff0000000000000ll);
        k64[j] = INT64_MAX;
    }
#pragma unroll
    for (int j = 0; j < K_KEEP; ++j)
        if (ik[j] >= 0 && (j < k || dk[j] <= band))
        {
            double x[MAXD];
            load_point<MAXD>(nn.pts64, nn.cap, sp.dim, ik[j], x);
            const double d = distance64<MAXD>(sp, x, q64);
            // insertion into (d, key) order
            double cd = d;
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
    for (int j = 0; j < k; ++j)
    {
        const bool have = j < K_KEEP && k64[j] != INT64_MAX;
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
            out[(int64_t)d * ld_out + i] = X;
            out[(int64_t)(d + sp.dim) * ld_out + i] = Y;
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
                d = distance64<MAXD>(sp, x, q);
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

template <int KIND, int MAXD, int MAXF>
static void launch_fp32_t(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, const float *qf,
                          int64_t nq, int k, const int64_t *prefix, int64_t *idx, double *dist,
                          unsigned long long *fb_list, unsigned long long *fb_n, RunCounters *ctr)
{
    const int grid = (int)((nq + 127) / 128);
    if (k <= 12)
        knn_fp32_kernel<KIND, MAXD, MAXF, 16><<<grid, 128, 0, lc.stream>>>(nn, sp, qv, qf, nq, k, prefix, idx, dist,
                                                                           fb_list, fb_n, ctr);
    else
        knn_fp32_kernel<KIND, MAXD, MAXF, 24><<<grid, 128, 0, lc.stream>>>(nn, sp, qv, qf, nq, k, prefix, idx, dist,
                                                                           fb_list, fb_n, ctr);
    note_launch();
}

bool launch_knn_fp32(const LaunchCfg &lc, const NNArgs &nn, const SpaceParams &sp, StatesView qv, const float *qf,
                     int64_t nq, int k, const int64_t *prefix, int64_t *idx, double *dist, unsigned long long *fb_list,
                     unsigned long long *fb_n, RunCounters *ctr)
{
    if (k > 20 || nq == 0)
        return false;
    if (sp.kind == GBO_SPACE_KINEMATIC_CHAIN && sp.dim <= 10)
        launch_fp32_t<GBO_SPACE_KINEMATIC_CHAIN, 10, 20>(lc, nn, sp, qv, qf, nq, k, prefix, idx, dist, fb_list, fb_n,
                                                          ctr);
    else if (sp.kind == GBO_SPACE_WRAP_L2 && sp.dim <= 8)
        launch_fp32_t<GBO_SPACE_WRAP_L2, 8, 8>(lc, nn, sp, qv, qf, nq, k, prefix, idx, dist, fb_list, fb_n, ctr);
    else if (sp.kind == GBO_SPACE_REAL_VECTOR && sp.dim <= 8)
        launch_fp32_t<GBO_SPACE_REAL_VECTOR, 8, 8>(lc, nn, sp, qv, qf, nq, k, prefix, idx, dist, fb_list, fb_n, ctr);
    else
        return false;
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

}  // namespace gbo
