// State sampling: RealVectorStateSampler::sampleUniform / sampleUniformNear and SO2StateSampler
// (RealVectorStateSpace.cpp:45-65, SO2StateSpace.cpp:46-56) over one sampler's RNG stream.
//
// The stream is OMPL's RNG (RandomNumbers.h:66-76): std::mt19937 -> libstdc++
// generate_canonical<double, 53> (two 32-bit draws w0, w1: (w0 + w1 * 2^32) / 2^64, values >= 1
// replaced by the largest double below 1) -> uniformReal(lo, hi) = (hi - lo) * U + lo.
// mt19937 (Matsumoto & Nishimura 1998) is sequential across 624-word blocks, so one CTA produces a
// sampler's word stream (mt_words_kernel) and the whole GPU converts word pairs into coordinates
// (words_to_states_kernel); large calls alternate the two over chunks of the stream.
#include <algorithm>

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

__device__ __forceinline__ double canonical53(unsigned w0, unsigned w1)
{
    double sum = (double)w0;
    sum = __dadd_rn(sum, __dmul_rn((double)w1, 4294967296.0));
    double r = __dmul_rn(sum, 5.421010862427522170037264e-20);  // / 2^64 (exact power of two)
    if (r >= 1.0)
        r = 0.99999999999999988897769753748;                   // nextafter(1, 0)
    return r;
}

// The word stream: one CTA continues the stream at st->pos and writes its next W tempered words to
// out, then saves the generator. A block's regeneration runs in the three dependency-free chunks
// [0,227), [227,454), [454,623) and word 623 into a second buffer (4 barriers per block), and each
// word is tempered and stored as soon as its chunk produces it.
__global__ void __launch_bounds__(256) mt_words_kernel(SamplerState *st, int64_t W, unsigned *out)
{
    __shared__ unsigned buf[2][624];
    unsigned *cur = buf[0], *nxt = buf[1];
    const int t = threadIdx.x;
    for (int i = t; i < 624; i += blockDim.x)
        cur[i] = st->mt[i];
    int pos = (int)st->pos;  // next unused word of cur (624: none)
    __syncthreads();
    int64_t w = min((int64_t)(624 - pos), W);  // the rest of the current block
    for (int i = t; i < (int)w; i += blockDim.x)
        out[i] = temper(cur[pos + i]);
    pos += (int)w;
    while (w < W)
    {
        const int m = (int)min((int64_t)624, W - w);  // words of the new block that are used
        unsigned *o = out + w;
        if (t < 227)
        {
            const unsigned v = twist_word(cur[t], cur[t + 1], cur[t + 397]);
            nxt[t] = v;
            if (t < m)
                o[t] = temper(v);
        }
        __syncthreads();
        if (t < 227)
        {
            const unsigned v = twist_word(cur[t + 227], cur[t + 228], nxt[t]);
            nxt[t + 227] = v;
            if (t + 227 < m)
                o[t + 227] = temper(v);
        }
        __syncthreads();
        if (t < 169)
        {
            const unsigned v = twist_word(cur[t + 454], cur[t + 455], nxt[t + 227]);
            nxt[t + 454] = v;
            if (t + 454 < m)
                o[t + 454] = temper(v);
        }
        __syncthreads();
        if (t == 0)
        {
            const unsigned v = twist_word(cur[623], nxt[0], nxt[396]);
            nxt[623] = v;
            if (623 < m)
                o[623] = temper(v);
        }
        __syncthreads();
        unsigned *tmp = cur;
        cur = nxt;
        nxt = tmp;
        w += m;
        pos = m;
    }
    for (int i = t; i < 624; i += blockDim.x)
        st->mt[i] = cur[i];
    if (t == 0)
        st->pos = (unsigned)pos;
}

// Values v0 .. v0 + nv - 1 of a sampling call (value v = coordinate v % dim of state v / dim) from the
// word pairs (2m, 2m + 1), m = v - v0, of the word stream: generate_canonical<double, 53> and
// uniformReal (or the near bounds), across the whole GPU.
__global__ void __launch_bounds__(256) words_to_states_kernel(const unsigned *words, int64_t v0, int64_t nv,
                                                              SpaceParams sp, StatesView nearv, int use_near,
                                                              double distance, MutStatesView out)
{
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < nv; m += (int64_t)gridDim.x * blockDim.x)
    {
        const double U = canonical53(words[2 * m], words[2 * m + 1]);
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
}

void launch_sample_uniform(const LaunchCfg &lc, SamplerState *st, const SpaceParams &sp, const double *near,
                           StatesView nearv, double distance, int64_t n, MutStatesView out, unsigned *words,
                           int64_t cap_words)
{
    const int64_t total = n * sp.dim, chunk = cap_words / 2;
    for (int64_t v0 = 0; v0 < total; v0 += chunk)
    {
        const int64_t nv = std::min(chunk, total - v0);
        mt_words_kernel<<<1, 256, 0, lc.stream>>>(st, 2 * nv, words);
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((nv + 255) / 256, (int64_t)lc.sm_count * 8));
        words_to_states_kernel<<<grid, 256, 0, lc.stream>>>(words, v0, nv, sp, nearv, near != nullptr, distance, out);
        note_launch();
        note_launch();
    }
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
