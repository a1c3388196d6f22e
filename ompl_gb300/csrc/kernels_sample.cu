// State sampling: RealVectorStateSampler::sampleUniform / sampleUniformNear and SO2StateSampler
// (RealVectorStateSpace.cpp:45-65, SO2StateSpace.cpp:46-56) over one sampler's RNG stream.
//
// The stream is OMPL's RNG (RandomNumbers.h:66-76): std::mt19937 -> libstdc++
// generate_canonical<double, 53> (two 32-bit draws w0, w1: (w0 + w1 * 2^32) / 2^64, values >= 1
// replaced by the largest double below 1) -> uniformReal(lo, hi) = (hi - lo) * U + lo.
// mt19937 (Matsumoto & Nishimura 1998) is sequential across 624-word blocks, so one CTA owns one
// stream: the block regeneration runs in the three dependency-free chunks [0,227), [227,454),
// [454,623) plus word 623, then all threads temper and convert the block's words.
#include "kernels_nn.cuh"

namespace gbo
{

__device__ __forceinline__ unsigned temper(unsigned y)
{
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
}

__device__ __forceinline__ unsigned twist_word(unsigned cur, unsigned next, unsigned far)
{
    const unsigned y = (cur & 0x80000000u) | (next & 0x7fffffffu);
    return far ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}

__device__ void regenerate(unsigned *mt)
{
    const int t = threadIdx.x;
    // chunk 1: k in [0, 227): mt[k + 397] still old
    unsigned v = 0;
    if (t < 227)
        v = twist_word(mt[t], mt[t + 1], mt[t + 397]);
    __syncthreads();
    if (t < 227)
        mt[t] = v;
    __syncthreads();
    // chunk 2: k in [227, 454): mt[k - 227] new (chunk 1), mt[k + 1] old
    if (t < 227)
        v = twist_word(mt[t + 227], mt[t + 228], mt[t]);
    __syncthreads();
    if (t < 227)
        mt[t + 227] = v;
    __syncthreads();
    // chunk 3: k in [454, 623): mt[k - 227] new (chunk 2), mt[k + 1] old
    if (t < 169)
        v = twist_word(mt[t + 454], mt[t + 455], mt[t + 227]);
    __syncthreads();
    if (t < 169)
        mt[t + 454] = v;
    __syncthreads();
    if (t == 0)
        mt[623] = twist_word(mt[623], mt[0], mt[396]);
    __syncthreads();
}

__device__ __forceinline__ double canonical53(unsigned w0, unsigned w1)
{
    double sum = (double)w0;
    sum = __dadd_rn(sum, __dmul_rn((double)w1, 4294967296.0));
    double r = __dmul_rn(sum, 5.421010862427522170037264e-20);  // / 2^64 (exact power of two)
    if (r >= 1.0)
        r = 0.99999999999999988897769753748;                   // nextafter(1, 0)
    return r;
}

// One CTA: n states of sp.dim values, value v = (state v / dim, coordinate v % dim) drawn from the
// word pair (2v, 2v+1) of the stream continuing at st->pos.
__global__ void __launch_bounds__(256) sample_kernel(SamplerState *st, SpaceParams sp, StatesView nearv, int use_near,
                                                     double distance, int64_t n, MutStatesView out)
{
    __shared__ unsigned mt[624];
    __shared__ unsigned tw[624];
    __shared__ unsigned s_pending;
    __shared__ int s_has_pending;
    for (int i = threadIdx.x; i < 624; i += blockDim.x)
        mt[i] = st->mt[i];
    unsigned pos = st->pos;
    if (threadIdx.x == 0)
        s_has_pending = 0;
    __syncthreads();
    const int64_t total = n * sp.dim;
    int64_t v0 = 0;  // next value index
    while (v0 < total)
    {
        if (pos >= 624)
        {
            regenerate(mt);
            pos = 0;
        }
        for (int i = threadIdx.x; i < 624; i += blockDim.x)
            tw[i] = temper(mt[i]);
        __syncthreads();
        // words [pos, 624) of this block; a pending word from the previous block pairs with tw[pos]
        int start = pos;
        const int has_pending = s_has_pending;
        const unsigned pending = s_pending;
        if (has_pending)
            start += 1;
        const int avail_pairs = (624 - start) / 2;
        const int64_t nv = min((int64_t)avail_pairs + (has_pending ? 1 : 0), total - v0);
        for (int64_t m = threadIdx.x; m < nv; m += blockDim.x)
        {
            unsigned w0, w1;
            if (has_pending && m == 0)
            {
                w0 = pending;
                w1 = tw[pos];
            }
            else
            {
                const int off = start + 2 * (int)(m - (has_pending ? 1 : 0));
                w0 = tw[off];
                w1 = tw[off + 1];
            }
            const double U = canonical53(w0, w1);
            const int64_t v = v0 + m;
            const int64_t i = v / sp.dim;
            const int d = (int)(v - i * sp.dim);
            double lo, hi;
            if (use_near)
            {
                const double c = nearv(i, d);
                if (sp.kind == GBO_SPACE_SO2)
                {
                    lo = __dsub_rn(c, distance);
                    hi = __dadd_rn(c, distance);
                }
                else
                {
                    lo = fmax(sp.low[d], __dsub_rn(c, distance));
                    hi = fmin(sp.high[d], __dadd_rn(c, distance));
                }
            }
            else
            {
                lo = sp.low[d];
                hi = sp.high[d];
            }
            double x = __dadd_rn(__dmul_rn(__dsub_rn(hi, lo), U), lo);
            if (use_near && sp.kind == GBO_SPACE_SO2)
            {
                // SO2StateSpace::enforceBounds (SO2StateSpace.cpp:79-87)
                double y = fmod(x, 2.0 * kPi);
                if (y < -kPi)
                    y = __dadd_rn(y, 2.0 * kPi);
                else if (y >= kPi)
                    y = __dsub_rn(y, 2.0 * kPi);
                x = y;
            }
            out(i, d) = x;
        }
        // advance the stream position
        int used = 2 * (int)nv - (has_pending ? 1 : 0);
        const int newpos = pos + used;
        __syncthreads();
        if (threadIdx.x == 0)
        {
            s_has_pending = 0;
            if (v0 + nv < total && newpos == 623)
            {
                s_pending = tw[623];
                s_has_pending = 1;
            }
        }
        __syncthreads();
        v0 += nv;
        pos = s_has_pending ? 624 : newpos;
    }
    __syncthreads();
    for (int i = threadIdx.x; i < 624; i += blockDim.x)
        st->mt[i] = mt[i];
    if (threadIdx.x == 0)
        st->pos = pos;
}

void launch_sample_uniform(const LaunchCfg &lc, SamplerState *st, const SpaceParams &sp, const double *near,
                           StatesView nearv, double distance, int64_t n, MutStatesView out)
{
    if (n == 0)
        return;
    sample_kernel<<<1, 256, 0, lc.stream>>>(st, sp, nearv, near != nullptr, distance, n, out);
    note_launch();
}

// FP32 FMA throughput probe: independent FMA chains, no memory traffic in the loop.
__global__ void __launch_bounds__(256) fma_peak_kernel(float *sink, int iters, float seed)
{
    float a0 = seed + threadIdx.x, a1 = a0 + 1.f, a2 = a0 + 2.f, a3 = a0 + 3.f, a4 = a0 + 4.f, a5 = a0 + 5.f,
          a6 = a0 + 6.f, a7 = a0 + 7.f;
    const float b = 0.999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i)
    {
#pragma unroll
        for (int j = 0; j < 16; ++j)
        {
            a0 = fmaf(a0, b, c);
            a1 = fmaf(a1, b, c);
            a2 = fmaf(a2, b, c);
            a3 = fmaf(a3, b, c);
            a4 = fmaf(a4, b, c);
            a5 = fmaf(a5, b, c);
            a6 = fmaf(a6, b, c);
            a7 = fmaf(a7, b, c);
        }
    }
    const float r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 12345.678f)
        sink[0] = r;
}

__global__ void sincos32_kernel(const double *theta, int64_t n, float *c, float *s)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        sincos_ff(split_double(theta[i]), c[i], s[i]);
}

void launch_sincos32(const LaunchCfg &lc, const double *theta, int64_t n, float *c, float *s)
{
    if (n == 0)
        return;
    sincos32_kernel<<<(int)((n + 255) / 256), 256, 0, lc.stream>>>(theta, n, c, s);
    note_launch();
}

__global__ void __launch_bounds__(256) dfma_peak_kernel(double *sink, int iters, double seed)
{
    double a0 = seed + threadIdx.x, a1 = a0 + 1.0, a2 = a0 + 2.0, a3 = a0 + 3.0;
    const double b = 0.999999, c = 1e-7;
    for (int i = 0; i < iters; ++i)
    {
#pragma unroll
        for (int j = 0; j < 8; ++j)
        {
            a0 = fma(a0, b, c);
            a1 = fma(a1, b, c);
            a2 = fma(a2, b, c);
            a3 = fma(a3, b, c);
        }
    }
    const double r = a0 + a1 + a2 + a3;
    if (r == 12345.678)
        sink[0] = r;
}

double measure_fp64_peak(const LaunchCfg &lc)
{
    double *sink = nullptr;
    cudaMalloc(&sink, 16);
    const int blocks = lc.sm_count * 8, iters = 256;
    dfma_peak_kernel<<<blocks, 256, 0, lc.stream>>>(sink, 8, 1.0);
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventRecord(e0, lc.stream);
    dfma_peak_kernel<<<blocks, 256, 0, lc.stream>>>(sink, iters, 1.0);
    cudaEventRecord(e1, lc.stream);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    note_launch();
    note_launch();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return ms > 0.f ? 2.0 * 4 * 8 * (double)iters * blocks * 256 / (ms * 1e-3) : 0.0;
}

double measure_fp32_peak(const LaunchCfg &lc)
{
    float *sink = nullptr;
    cudaMalloc(&sink, 16);
    const int blocks = lc.sm_count * 8, iters = 4096;
    fma_peak_kernel<<<blocks, 256, 0, lc.stream>>>(sink, 64, 1.f);  // warm-up
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    double best = 0.0;
    for (int rep = 0; rep < 3; ++rep)
    {
        cudaEventRecord(e0, lc.stream);
        fma_peak_kernel<<<blocks, 256, 0, lc.stream>>>(sink, iters, 1.f);
        cudaEventRecord(e1, lc.stream);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        const double flops = 2.0 * 8 * 16 * (double)iters * blocks * 256;
        if (ms > 0.f && flops / (ms * 1e-3) > best)
            best = flops / (ms * 1e-3);
    }
    note_launch();
    note_launch();
    note_launch();
    note_launch();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(sink);
    return best;
}

}  // namespace gbo
