// State sampling: RealVectorStateSampler::sampleUniform / sampleUniformNear and SO2StateSampler
// (RealVectorStateSpace.cpp:45-65, SO2StateSpace.cpp:46-56) over one sampler's RNG stream.
//
// The stream is OMPL's RNG (RandomNumbers.h:66-76): std::mt19937 -> libstdc++
// generate_canonical<double, 53> (two 32-bit draws w0, w1: (w0 + w1 * 2^32) / 2^64, values >= 1
// replaced by the largest double below 1) -> uniformReal(lo, hi) = (hi - lo) * U + lo.
// mt19937 (Matsumoto & Nishimura 1998) is sequential across 624-word blocks. Calls of fewer than 2^18
// stream words run on one CTA that produces the sampler's word stream (mt_words_kernel) while the
// whole GPU converts word pairs into coordinates (words_to_states_kernel); larger calls cut their
// stretch of the stream into segments that start from jump-ahead windows and run side by side (below).
// sampleGaussian (further below) draws its polar candidates' words the same two ways.
#include <algorithm>
#include <cmath>

#include "crlog.cuh"
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
// kRaw (speculative draws): the words are stored untempered, every new block is stored whole (up to
// W + 623 words) and the generator is left unchanged, so that any prefix of the stream can later be
// committed by copying the block that holds its last word (gauss_advance_kernel).
template <bool kRaw>
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
        out[i] = kRaw ? cur[pos + i] : temper(cur[pos + i]);
    pos += (int)w;
    while (w < W)
    {
        const int m = kRaw ? 624 : (int)min((int64_t)624, W - w);  // words of the new block that are stored
        unsigned *o = out + w;
        if (t < 227)
        {
            const unsigned v = twist_word(cur[t], cur[t + 1], cur[t + 397]);
            nxt[t] = v;
            if (t < m)
                o[t] = kRaw ? v : temper(v);
        }
        __syncthreads();
        if (t < 227)
        {
            const unsigned v = twist_word(cur[t + 227], cur[t + 228], nxt[t]);
            nxt[t + 227] = v;
            if (t + 227 < m)
                o[t + 227] = kRaw ? v : temper(v);
        }
        __syncthreads();
        if (t < 169)
        {
            const unsigned v = twist_word(cur[t + 454], cur[t + 455], nxt[t + 227]);
            nxt[t + 454] = v;
            if (t + 454 < m)
                o[t + 454] = kRaw ? v : temper(v);
        }
        __syncthreads();
        if (t == 0)
        {
            const unsigned v = twist_word(cur[623], nxt[0], nxt[396]);
            nxt[623] = v;
            if (623 < m)
                o[623] = kRaw ? v : temper(v);
        }
        __syncthreads();
        unsigned *tmp = cur;
        cur = nxt;
        nxt = tmp;
        w += m;
        pos = m;
    }
    if (kRaw)
        return;
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
        mt_words_kernel<false><<<1, 256, 0, lc.stream>>>(st, 2 * nv, words);
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((nv + 255) / 256, (int64_t)lc.sm_count * 8));
        words_to_states_kernel<<<grid, 256, 0, lc.stream>>>(words, v0, nv, sp, nearv, near != nullptr, distance, out);
        note_launch();
        note_launch();
    }
}

// ---------------------------------------------------------------- segmented stream (jump-ahead)
// Calls of many values cut their stretch of the stream, words [0, W) counted from the sampler's next
// word T0, into segments of L words (L even, so no value's word pair is split): segment s starts from
// the generator window at T0 - 1 + s L (position 1 of that window: its word 0 only carries its top
// bit). Window 0 is the sampler's own state. Window s >= 1 is A^(sL) applied to the window at T0 - 1
// (mt_jump.cu): with p = x^(sL) mod phi, its word w is the XOR over the set coefficients i of p of
// u_(i+w), u_t = x_(T0-1+t). One CTA per segment then runs the recurrence over its words and converts
// them to coordinates, so the call runs at the width of the GPU instead of one CTA's recurrence.

// RN(w1 * 2^32 + w0) / 2^64 (generate_canonical's value) in integer arithmetic: the same double as
// canonical53, including the largest double below 1 for sums that round up to 2^64.
__device__ __forceinline__ double canonical53_int(unsigned w0, unsigned w1)
{
    const unsigned long long w = ((unsigned long long)w1 << 32) | w0;
    if (w == 0)
        return 0.0;
    const int z = __clzll(w);
    const unsigned long long m = w << z;  // leading one at bit 63
    unsigned long long mant = m >> 11;    // 53 bits
    const unsigned rem = (unsigned)(m & 0x7ffu);
    mant += (rem > 0x400u || (rem == 0x400u && (mant & 1ull))) ? 1ull : 0ull;
    unsigned long long e = 1022ull - (unsigned long long)z;  // value in [2^(-1-z), 2^-z)
    if (mant >> 53)
    {
        mant >>= 1;
        e += 1;
    }
    if (e >= 1023ull)
        return 0.99999999999999988897769753748;  // rounded to 1: nextafter(1, 0)
    return __longlong_as_double((long long)((e << 52) | (mant & 0xFFFFFFFFFFFFFull)));
}

// Coordinate d of state i of a call from generate_canonical's U.
__device__ __forceinline__ void emit_uniform_id(int64_t i, int d, double U, const SpaceParams &sp, const double *span,
                                                StatesView nearv, int use_near, double distance, MutStatesView out)
{
    double x;
    if (use_near)
    {
        const double c = nearv(i, d);
        double lo, hi;
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
        x = __dadd_rn(__dmul_rn(__dsub_rn(hi, lo), U), lo);
        if (sp.kind == GBO_SPACE_SO2)
        {
            // SO2StateSpace::enforceBounds (SO2StateSpace.cpp:79-87)
            double y = fmod(x, 2.0 * kPi);
            if (y < -kPi)
                y = __dadd_rn(y, 2.0 * kPi);
            else if (y >= kPi)
                y = __dsub_rn(y, 2.0 * kPi);
            x = y;
        }
    }
    else
        x = __dadd_rn(__dmul_rn(span[d], U), sp.low[d]);
    out(i, d) = x;
}

// The next 624 raw words (nxt) after block cur: the recurrence in its three dependency-free chunks,
// word 623 with the last one. Every thread of the CTA (at least 227) calls it.
__device__ __forceinline__ void twist_block(const unsigned *cur, unsigned *nxt)
{
    const int t = threadIdx.x;
    if (t < 227)
        nxt[t] = twist_word(cur[t], cur[t + 1], cur[t + 397]);
    __syncthreads();
    if (t < 227)
        nxt[t + 227] = twist_word(cur[t + 227], cur[t + 228], nxt[t]);
    __syncthreads();
    if (t < 169)
        nxt[t + 454] = twist_word(cur[t + 454], cur[t + 455], nxt[t + 227]);
    else if (t == 169)
        nxt[623] = twist_word(cur[623], nxt[0], nxt[396]);
    __syncthreads();
}

constexpr int64_t kJumpU = 19968 + 704;  // u words the jumps read (coefficients < 19968, words < 640 + 64)

// u_t = x_(T0-1+t) for t < n (one CTA), and states[0] = the sampler's block and position.
__global__ void __launch_bounds__(256) mt_window_seq_kernel(const SamplerState *st, int64_t n, unsigned *u,
                                                            unsigned *state0)
{
    __shared__ unsigned buf[2][624];
    unsigned *cur = buf[0], *nxt = buf[1];
    const int t = threadIdx.x;
    for (int i = t; i < 624; i += blockDim.x)
    {
        cur[i] = st->mt[i];
        state0[i] = cur[i];
    }
    const int pos = (int)st->pos;  // 1..624
    if (t == 0)
        state0[624] = (unsigned)pos;
    __syncthreads();
    int64_t w = 625 - pos;  // u_0 .. u_(624-pos) are cur[pos-1 .. 623]
    for (int i = t; i < w && i < n; i += blockDim.x)
        u[i] = cur[pos - 1 + i];
    while (w < n)
    {
        twist_block(cur, nxt);
        for (int i = t; i < 624 && w + i < n; i += blockDim.x)
            u[w + i] = nxt[i];
        unsigned *tmp = cur;
        cur = nxt;
        nxt = tmp;
        w += 624;
        __syncthreads();
    }
}

// Windows 1..K by table lookup ("four Russians"): coefficients are taken 5 at a time (group g covers
// i = 5g .. 5g + 4), and for each window word w the 32 XOR combinations of u[5g + w .. 5g + w + 4] are
// tabulated once per group and shared by every window: window k adds the entry its 5 coefficient bits
// select. A CTA of NW warps covers 8 NW window words and one range of groups for up to 32 NW windows
// (one thread per window, 8 NW accumulators each). Entry (w, h) sits at word 33 w + h: a reader's
// address is its h plus a constant per w, and the 32 readers of one column hit 32 banks or the same
// word; lane (c, q) of warp p builds entries 8q .. 8q + 7 of column 8p + c, and a warp's stores of one
// step cover 32 banks. Partial results go to states[1..K] by atomicXor (zeroed before).
constexpr int kJG = 5;                                 // coefficients per lookup
constexpr int kJGroups = (19937 + kJG - 1) / kJG;      // 3988 groups (bits past 19936 are zero)

// grid: (window-word chunks, ranges of qper groups, window chunks); dynamic shared memory holds the
// range's u words (5 qper + 8 NW + 5)
template <int NW>
__global__ void __launch_bounds__(32 * NW) mt_jump_kernel(const unsigned *u, const unsigned *polys, int K, int qper,
                                                          unsigned *states)
{
    constexpr int TW = 8 * NW, KP = 32 * NW, GB = NW <= 5 ? 4 : 2;  // GB groups tabulated per phase
    extern __shared__ unsigned us[];
    __shared__ unsigned tab[2][GB][33 * TW];
    const int w0 = blockIdx.x * TW;
    const int g0 = blockIdx.y * qper, g1 = min(g0 + qper, kJGroups);
    const int k0 = blockIdx.z * KP;
    const int t = threadIdx.x, nk = min(KP, K - k0);
    const int sl = kJG * qper + TW + kJG;
    const int ubase = kJG * g0 + w0;
    for (int j = t; j < sl; j += blockDim.x)
        us[j] = ubase + j < kJumpU ? u[ubase + j] : 0u;  // words past kJumpU are never used
    __syncthreads();
    const int lane = t & 31, bw = 8 * (t >> 5) + (lane & 7), bq = lane >> 3;
    // tables of groups ga .. ga + GB - 1 (those below g1) into set (ga / GB) & 1
    auto build = [&](int ga) {
#pragma unroll
        for (int e = 0; e < GB; ++e)
        {
            const int g = ga + e;
            if (g >= g1)
                break;
            unsigned *T = tab[((ga - g0) / GB) & 1][e] + 33 * bw + 8 * bq;
            const unsigned *x = us + kJG * (g - g0) + bw;
            const unsigned x0 = x[0], x1 = x[1], x2 = x[2];
            const unsigned base = ((bq & 1) ? x[3] : 0u) ^ ((bq & 2) ? x[4] : 0u);
#pragma unroll
            for (int j = 0; j < 8; ++j)
                T[j] = base ^ ((j & 1) ? x0 : 0u) ^ ((j & 2) ? x1 : 0u) ^ ((j & 4) ? x2 : 0u);
        }
    };
    unsigned acc[TW];
#pragma unroll
    for (int w = 0; w < TW; ++w)
        acc[w] = 0u;
    // this window's coefficient words qa, qa + 1 (zero past word 623), advanced as the groups move on
    const unsigned *crow = polys + (size_t)(k0 + min(t, nk - 1)) * 624;
    int qa = (kJG * g0) >> 5;
    unsigned c_lo = crow[qa], c_hi = qa + 1 < 624 ? crow[qa + 1] : 0u;
    if (g0 < g1)
        build(g0);
    __syncthreads();
#pragma unroll 1
    for (int ga = g0; ga < g1; ga += GB)
    {
        if (ga + GB < g1)
            build(ga + GB);
        const unsigned(*set)[33 * TW] = tab[((ga - g0) / GB) & 1];
#pragma unroll
        for (int e = 0; e < GB; ++e)
        {
            const int g = ga + e;
            if (g >= g1)
                break;
            const int b = kJG * g, q = b >> 5, sh = b & 31;
            if (q != qa)
            {
                qa = q;
                c_lo = c_hi;
                c_hi = qa + 1 < 624 ? crow[qa + 1] : 0u;
            }
            if (t < nk)
            {
                unsigned v = c_lo >> sh;
                if (sh > 32 - kJG)
                    v |= c_hi << (32 - sh);
                const unsigned *T = set[e] + (v & 31u);
#pragma unroll
                for (int w = 0; w < TW; ++w)
                    acc[w] ^= T[33 * w];
            }
        }
        __syncthreads();
    }
    if (t < nk)
    {
        unsigned *o = states + (size_t)(k0 + t + 1) * 625 + w0;
#pragma unroll
        for (int w = 0; w < TW; ++w)
            if (w0 + w < 624)
                atomicXor(o + w, acc[w]);
    }
}

template <int NW>
static void launch_jump_t(const LaunchCfg &lc, const unsigned *u, const uint32_t *polys, int K, unsigned *states)
{
    // two CTAs per SM: the ranges of groups split the rest of the grid over 2 x SM count (four per SM
    // measured the same: the lookups are bound by shared-memory wavefronts, not by latency)
    const int wchunks = (624 + 8 * NW - 1) / (8 * NW), kchunks = (K + 32 * NW - 1) / (32 * NW);
    const int ranges = std::max(1, std::min(kJGroups, (2 * lc.sm_count + wchunks * kchunks / 2) / (wchunks * kchunks)));
    const int qper = (kJGroups + ranges - 1) / ranges;
    const size_t smem = (size_t)(kJG * qper + 8 * NW + kJG) * sizeof(unsigned);
    if (smem > 48 * 1024)
        cudaFuncSetAttribute(mt_jump_kernel<NW>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    mt_jump_kernel<NW><<<dim3(wchunks, (kJGroups + qper - 1) / qper, kchunks), 32 * NW, smem, lc.stream>>>(
        u, polys, K, qper, states);
}

static void launch_jump(const LaunchCfg &lc, const unsigned *u, const uint32_t *polys, int K, unsigned *states)
{
    switch (std::min(8, (K + 31) / 32))
    {
    case 1: launch_jump_t<1>(lc, u, polys, K, states); break;
    case 2: launch_jump_t<2>(lc, u, polys, K, states); break;
    case 3: launch_jump_t<3>(lc, u, polys, K, states); break;
    case 4: launch_jump_t<4>(lc, u, polys, K, states); break;
    case 5: launch_jump_t<5>(lc, u, polys, K, states); break;
    case 6: launch_jump_t<6>(lc, u, polys, K, states); break;
    case 7: launch_jump_t<7>(lc, u, polys, K, states); break;
    default: launch_jump_t<8>(lc, u, polys, K, states); break;
    }
}

// One CTA per segment s: words [s L, min((s + 1) L, W)) of the call from window s, tempered and stored
// as the recurrence produces them (word j of the call at words[j]); the last segment leaves its
// generator in st. kRaw: the words are stored untempered and st is left unchanged (sampleGaussian's
// speculative draws, committed afterwards).
template <bool kRaw>
__global__ void __launch_bounds__(256) mt_segment_kernel(SamplerState *st, const unsigned *states, int64_t L,
                                                         int64_t W, int nseg, unsigned *words)
{
    __shared__ unsigned buf[2][624];
    unsigned *cur = buf[0], *nxt = buf[1];
    const int t = threadIdx.x, s = blockIdx.x;
    const unsigned *src = states + (size_t)s * 625;
    for (int i = t; i < 624; i += blockDim.x)
        cur[i] = src[i];
    int pos = s == 0 ? (int)src[624] : 1;
    const int64_t begin = (int64_t)s * L, len = min(begin + L, W) - begin;
    unsigned *o = words + begin;
    __syncthreads();
    int64_t w = min((int64_t)(624 - pos), len);  // the rest of the first block
    for (int i = t; i < (int)w; i += blockDim.x)
        o[i] = kRaw ? cur[pos + i] : temper(cur[pos + i]);
    pos += (int)w;
#pragma unroll 1
    while (w < len)
    {
        const int m = (int)min((int64_t)624, len - w);  // words of the new block that belong to the segment
        unsigned *ob = o + w;
        if (t < 227)
        {
            const unsigned v = twist_word(cur[t], cur[t + 1], cur[t + 397]);
            nxt[t] = v;
            if (t < m)
                ob[t] = kRaw ? v : temper(v);
        }
        __syncthreads();
        if (t < 227)
        {
            const unsigned v = twist_word(cur[t + 227], cur[t + 228], nxt[t]);
            nxt[t + 227] = v;
            if (t + 227 < m)
                ob[t + 227] = kRaw ? v : temper(v);
        }
        __syncthreads();
        if (t < 170)
        {
            const unsigned v = t < 169 ? twist_word(cur[t + 454], cur[t + 455], nxt[t + 227])
                                       : twist_word(cur[623], nxt[0], nxt[396]);
            nxt[t + 454] = v;
            if (t + 454 < m)
                ob[t + 454] = kRaw ? v : temper(v);
        }
        __syncthreads();
        unsigned *tmp = cur;
        cur = nxt;
        nxt = tmp;
        w += m;
        pos = m;
    }
    if (!kRaw && s == nseg - 1)
    {
        for (int i = t; i < 624; i += blockDim.x)
            st->mt[i] = cur[i];
        if (t == 0)
            st->pos = (unsigned)pos;
    }
}

// Values v0 .. v0 + nv - 1 of the call from the stored word pairs (2m, 2m + 1), m = v - v0:
// generate_canonical in integer arithmetic, then uniformReal (or the near bounds). state = v / dim by a
// multiply-high with magic = ceil(2^40 / dim) (exact for v < 2^31 and dim <= 256).
__global__ void __launch_bounds__(256) pairs_to_states_kernel(const uint2 *pairs, int64_t nv, SpaceParams sp,
                                                              unsigned long long magic, StatesView nearv,
                                                              int use_near, double distance, MutStatesView out)
{
    __shared__ double span[GBO_MAXD];
    for (int d = threadIdx.x; d < sp.dim; d += blockDim.x)
        span[d] = __dsub_rn(sp.high[d], sp.low[d]);
    __syncthreads();
    for (int64_t m = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; m < nv; m += (int64_t)gridDim.x * blockDim.x)
    {
        const uint2 w = pairs[m];
        const unsigned long long v = (unsigned long long)m;
        const int64_t i = (int64_t)__umul64hi(v << 24, magic);
        emit_uniform_id(i, (int)(v - (unsigned long long)i * sp.dim), canonical53_int(w.x, w.y), sp, span, nearv,
                        use_near, distance, out);
    }
}

int64_t sample_jump_words(int64_t nseg, int64_t W)
{
    return kJumpU + nseg * 625 + 4 + W;
}

void launch_sample_uniform_jump(const LaunchCfg &lc, SamplerState *st, const SpaceParams &sp, const double *near,
                                StatesView nearv, double distance, int64_t n, MutStatesView out, unsigned *scratch,
                                const uint32_t *polys, int64_t L, int nseg)
{
    const int64_t values = n * sp.dim, W = 2 * values;
    unsigned *u = scratch, *states = scratch + kJumpU, *words = states + (size_t)nseg * 625;
    words += (4 - ((uintptr_t)words / 4) % 4) % 4;  // 16-byte aligned
    const int K = nseg - 1;
    if (K > 0)
        cudaMemsetAsync(states + 625, 0, (size_t)K * 625 * sizeof(unsigned), lc.stream);
    mt_window_seq_kernel<<<1, 256, 0, lc.stream>>>(st, kJumpU, u, states);
    note_launch();
    if (K > 0)
    {
        launch_jump(lc, u, (const unsigned *)polys, K, states);
        note_launch();
    }
    mt_segment_kernel<false><<<nseg, 256, 0, lc.stream>>>(st, states, L, W, nseg, words);
    const unsigned long long magic = ((1ull << 40) + (unsigned long long)sp.dim - 1) / (unsigned long long)sp.dim;
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((values + 255) / 256, (int64_t)lc.sm_count * 16));
    pairs_to_states_kernel<<<grid, 256, 0, lc.stream>>>((const uint2 *)words, values, sp, magic, nearv, near != nullptr,
                                                        distance, out);
    note_launch();
    note_launch();
}

// The next W raw (untempered) words of the stream after the sampler's next word into raw[0 .. W), the
// generator unchanged: the segmented generation of sampleUniform without the conversion.
static void launch_raw_words_jump(const LaunchCfg &lc, const SamplerState *st, int64_t W, unsigned *raw,
                                  unsigned *scratch, const uint32_t *polys, int64_t L)
{
    const int nseg = (int)((W + L - 1) / L);
    unsigned *u = scratch, *states = scratch + kJumpU;
    const int K = nseg - 1;
    if (K > 0)
        cudaMemsetAsync(states + 625, 0, (size_t)K * 625 * sizeof(unsigned), lc.stream);
    mt_window_seq_kernel<<<1, 256, 0, lc.stream>>>(st, kJumpU, u, states);
    if (K > 0)
    {
        launch_jump(lc, u, polys, K, states);
        note_launch();
    }
    mt_segment_kernel<true><<<nseg, 256, 0, lc.stream>>>(nullptr, states, L, W, nseg, raw);
    note_launch();
    note_launch();
}

// ---------------------------------------------------------------- sampleGaussian
// RealVectorStateSampler::sampleGaussian (RealVectorStateSpace.cpp:67-82: per coordinate
// rng_.gaussian(mean, stdDev) clamped to the bounds) and SO2StateSampler::sampleGaussian
// (SO2StateSpace.cpp:58-62: wrapped by enforceBounds). RNG::gaussian (RandomNumbers.h:98-101) is
// libstdc++'s normal_distribution, the polar method of Marsaglia and Bray (1964) with a cached pair:
// a candidate takes two uniform01 draws (4 stream words), x = 2U - 1, y = 2V - 1, r2 = x^2 + y^2, and is
// rejected while r2 > 1 or r2 == 0; an accepted one gives mult = sqrt(-2 log(r2) / r2) and the values
// y * mult (returned) then x * mult (cached for the next draw of the same RNG, across calls).
// Every operation is the same IEEE double operation except log, which is log_rn (crlog.cuh, rounded
// to nearest); glibc's log differs from the correctly rounded value in the last bit for a small
// fraction of arguments, and only the values of those pairs differ (by an ulp or two).
//
// Stream consumption is data dependent, so a chunk draws a bounded surplus of candidates
// speculatively (raw words, generator unchanged), evaluates every accepted candidate's pair once
// (gauss_pairs_kernel), ranks the CTAs' counts (gauss_scan_kernel), places the pairs the call needs
// (gauss_emit_kernel) and then commits exactly the words used (gauss_advance[_seg]_kernel).
constexpr int kGaussPerCta = 1024;  // candidates per CTA: 256 threads x 4

// 2U - 1 rounded to nearest for a generate_canonical value U in [0, 1): 2U by the exponent (exact; U is
// 0 or at least 2^-64), then one FP64 subtraction.
__device__ __forceinline__ double two_u_minus_1(double U)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(U);
    return __dsub_rn(__longlong_as_double((long long)(b ? b + (1ull << 52) : 0ull)), 1.0);
}

// The polar method's candidate from four stream words: generate_canonical in integer arithmetic (the
// same doubles as canonical53), and the rejection test r2 > 1 || r2 == 0 on the bits (r2 >= +0).
__device__ __forceinline__ bool polar_candidate(uint4 w, double &x, double &y, double &r2)
{
    x = two_u_minus_1(canonical53_int(temper(w.x), temper(w.y)));
    y = two_u_minus_1(canonical53_int(temper(w.z), temper(w.w)));
    r2 = __dadd_rn(__dmul_rn(x, x), __dmul_rn(y, y));
    const unsigned long long rb = (unsigned long long)__double_as_longlong(r2);
    return rb != 0ull && rb <= 0x3FF0000000000000ull;
}

// a < b for doubles as IEEE compares them, on the integer pipe (the FP64 pipe is this kernel's bound):
// false when either is NaN or both are zeros, else the order of the sign-magnitude bit patterns.
__device__ __forceinline__ bool dlt_bits(double a, double b)
{
    const long long ia = __double_as_longlong(a), ib = __double_as_longlong(b);
    const unsigned long long ma = (unsigned long long)ia & 0x7fffffffffffffffull;
    const unsigned long long mb = (unsigned long long)ib & 0x7fffffffffffffffull;
    if (ma > 0x7ff0000000000000ull || mb > 0x7ff0000000000000ull || (ma | mb) == 0ull)
        return false;
    return (ia ^ ((ia >> 63) & 0x7fffffffffffffffll)) < (ib ^ ((ib >> 63) & 0x7fffffffffffffffll));
}

// Value v of the call (coordinate v % dim of state v / dim) from a standard normal value g:
// normal_distribution's g * 1 + 0 (which only turns -0 into +0: done on the bits), then * stdDev + mean
// and the bounds.
__device__ __forceinline__ void gauss_emit(const SpaceParams &sp, StatesView mean, double stddev, MutStatesView out,
                                           int64_t v, double g)
{
    const int64_t i = v / sp.dim;
    const int d = (int)(v - i * sp.dim);
    const double g0 = __double_as_longlong(g) == (long long)0x8000000000000000ull ? 0.0 : g;
    double z = __dadd_rn(__dmul_rn(g0, stddev), mean(i, d));
    if (sp.kind == GBO_SPACE_SO2)
    {
        // SO2StateSpace::enforceBounds (SO2StateSpace.cpp:79-87)
        double r = fmod(z, 2.0 * kPi);
        if (r < -kPi)
            r = __dadd_rn(r, 2.0 * kPi);
        else if (r >= kPi)
            r = __dsub_rn(r, 2.0 * kPi);
        z = r;
    }
    else if (dlt_bits(z, sp.low[d]))
        z = sp.low[d];
    else if (dlt_bits(sp.high[d], z))
        z = sp.high[d];
    out(i, d) = z;
}

// Value 0 of a call from the cached value of the previous call.
__global__ void gauss_saved_kernel(SamplerState *st, SpaceParams sp, StatesView mean, double stddev, MutStatesView out)
{
    if (threadIdx.x == 0)
    {
        gauss_emit(sp, mean, stddev, out, 0, st->saved);
        st->has_saved = 0;
    }
}

// The pairs of CTA b's 1,024 candidates (k = 1024 b .. 1024 b + 1023): its threads rank the accepted
// candidates in stream order with ballots and keep their (x, y) compacted in shared memory, then
// evaluate consecutive pairs with no lane idle on a rejected candidate: accepted candidate q of the CTA
// gives pair[1024 b + q] = (y mult, x mult), mult = sqrt(-2 log(r2) / r2), and kidx[1024 b + q] = its
// candidate index within the CTA; cnt[b] = the CTA's accepted count. The pairs whose log the plain-FP64
// evaluation cannot round (about 3 %) are listed (b << 10 | q, one global atomic per CTA) for
// gauss_slow_kernel, which runs the double-double evaluation for all of them across the GPU; done here
// at the end of each CTA, it held the CTA's other warps in a long serial tail. gauss_emit_kernel places
// the pairs.
__global__ void __launch_bounds__(256) gauss_pairs_kernel(const uint4 *cand, int64_t G, long long *cnt,
                                                          double2 *pair, unsigned short *kidx, unsigned *slowlist,
                                                          GaussChunk *ctl)
{
    __shared__ double2 sxy[kGaussPerCta];          // accepted (x, y) by local pair index
    __shared__ double sr2[kGaussPerCta];           // and their x^2 + y^2
    __shared__ unsigned short slow[kGaussPerCta];  // local pair indices left to log_cr
    __shared__ int wcnt[4][8];
    __shared__ int nslow;
    __shared__ long long slow0;  // this CTA's first entry in slowlist
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    if (t == 0)
        nslow = 0;
    const int64_t base = (int64_t)blockIdx.x * kGaussPerCta;
    double xs[4], ys[4], rs[4];
    unsigned bal[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
    {
        const int64_t k = base + r * 256 + t;
        bool acc = false;
        xs[r] = ys[r] = rs[r] = 0.0;
        if (k < G)
            acc = polar_candidate(cand[k], xs[r], ys[r], rs[r]);
        bal[r] = __ballot_sync(0xffffffffu, acc);
        if (lane == 0)
            wcnt[r][warp] = __popc(bal[r]);
    }
    __syncthreads();
    int np = 0;  // accepted candidates of this CTA in earlier rounds
#pragma unroll
    for (int r = 0; r < 4; ++r)
    {
        int before = 0, all = 0;
#pragma unroll
        for (int w = 0; w < 8; ++w)
        {
            before += w < warp ? wcnt[r][w] : 0;
            all += wcnt[r][w];
        }
        if ((bal[r] >> lane) & 1u)
        {
            const int q = np + before + __popc(bal[r] & ((1u << lane) - 1u));
            sxy[q] = make_double2(xs[r], ys[r]);
            sr2[q] = rs[r];
            kidx[base + q] = (unsigned short)(r * 256 + t);
        }
        np += all;
    }
    if (t == 0)
        cnt[blockIdx.x] = np;
    __syncthreads();
#pragma unroll 1
    for (int q = t; q < np; q += 256)
    {
        const double2 p = sxy[q];
        const double r2 = sr2[q];
        double lg;
        if (log_fast(r2, lg))
        {
            const double mult = __dsqrt_rn(__ddiv_rn(__dmul_rn(-2.0, lg), r2));
            pair[base + q] = make_double2(__dmul_rn(p.y, mult), __dmul_rn(p.x, mult));
        }
        else
            slow[atomicAdd(&nslow, 1)] = (unsigned short)q;
    }
    __syncthreads();
    const int ns = nslow;
    if (ns == 0)
        return;
    if (t == 0)
        slow0 = atomicAdd((unsigned long long *)&ctl->slow, (unsigned long long)ns);
    __syncthreads();
    for (int i = t; i < ns; i += 256)
        slowlist[slow0 + i] = (unsigned)blockIdx.x << 10 | slow[i];
}

// Pair v = b << 10 | q of the chunk from its candidate (formed again from its words) and lg = log(r2).
__device__ __forceinline__ void gauss_listed_pair(const uint4 *cand, const unsigned short *kidx, double2 *pair,
                                                  unsigned v, bool cr, unsigned *crlist, GaussChunk *ctl)
{
    const int64_t base = (int64_t)(v >> 10) * kGaussPerCta;
    const int q = (int)(v & 1023u);
    double x, y, r2, lg;
    polar_candidate(cand[base + kidx[base + q]], x, y, r2);
    if (cr)
        lg = log_cr(r2);
    else if (!log_med(r2, lg))
    {
        // left to gauss_cr_kernel (about 2 % of the list): one atomic per warp
        const unsigned act = __activemask(), lane = threadIdx.x & 31u;
        const unsigned lead = __ffs(act) - 1;
        unsigned long long at = 0;
        if (lane == lead)
            at = atomicAdd((unsigned long long *)&ctl->slow_cr, (unsigned long long)__popc(act));
        at = __shfl_sync(act, at, lead);
        crlist[at + __popc(act & ((1u << lane) - 1u))] = v;
        return;
    }
    const double mult = __dsqrt_rn(__ddiv_rn(__dmul_rn(-2.0, lg), r2));
    pair[base + q] = make_double2(__dmul_rn(y, mult), __dmul_rn(x, mult));
}

// The pairs gauss_pairs_kernel listed, with log_med; those it cannot round go to crlist.
__global__ void __launch_bounds__(256) gauss_slow_kernel(const uint4 *cand, const unsigned short *kidx,
                                                         const unsigned *slowlist, unsigned *crlist,
                                                         GaussChunk *ctl, double2 *pair)
{
    const long long n = ctl->slow;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        gauss_listed_pair(cand, kidx, pair, slowlist[e], false, crlist, ctl);
}

// The pairs gauss_slow_kernel left, with log_cr.
__global__ void __launch_bounds__(256) gauss_cr_kernel(const uint4 *cand, const unsigned short *kidx,
                                                       const unsigned *crlist, GaussChunk *ctl, double2 *pair)
{
    const long long n = ctl->slow_cr;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x)
        gauss_listed_pair(cand, kidx, pair, crlist[e], true, nullptr, ctl);
}

// Exclusive scan of the per-CTA counts in place (one CTA of 1024 threads); the total goes to ctl.
__global__ void __launch_bounds__(1024) gauss_scan_kernel(long long *cnt, int nb, GaussChunk *ctl)
{
    __shared__ long long part[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long run = 0;
    for (int b0 = 0; b0 < nb; b0 += 1024)
    {
        const int b = b0 + (int)threadIdx.x;
        const long long v = b < nb ? cnt[b] : 0;
        long long x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1)
        {
            const long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o)
                x += y;
        }
        if (lane == 31)
            part[warp] = x;
        __syncthreads();
        if (warp == 0)
        {
            long long p = part[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1)
            {
                const long long y = __shfl_up_sync(0xffffffffu, p, o);
                if (lane >= o)
                    p += y;
            }
            part[lane] = p;
        }
        __syncthreads();
        if (b < nb)
            cnt[b] = run + (warp ? part[warp - 1] : 0) + x - v;
        run += part[31];
        __syncthreads();
    }
    if (threadIdx.x == 0)
    {
        ctl->accepted = run;
        ctl->consumed = -1;
    }
}

struct GaussArgs
{
    const double2 *pair;         // pairs of each CTA's accepted candidates (gauss_pairs_kernel)
    const unsigned short *kidx;  // their candidate indices within the CTA
    const long long *off;        // accepted candidates before each CTA
    int nb;                      // CTAs of the chunk
    int64_t need;                // pairs the call still needs
    int64_t v0;                  // value index of the chunk's first pair
    int64_t M;                   // values of the call
    double stddev;
    SpaceParams sp;
    StatesView mean;
    MutStatesView out;
    SamplerState *st;
    GaussChunk *ctl;
};

// Accepted candidate j of the chunk (in stream order) becomes pair j: values v0 + 2j and v0 + 2j + 1;
// the value past the call's end is cached. The words through the last needed candidate are the
// chunk's consumption.
__global__ void __launch_bounds__(256) gauss_emit_kernel(const __grid_constant__ GaussArgs a)
{
    const int b = blockIdx.x;
    const long long rank0 = a.off[b];
    if (rank0 >= a.need)
        return;  // the call's pairs all come from earlier candidates
    const long long next = b + 1 < a.nb ? a.off[b + 1] : a.ctl->accepted;
    const int np = (int)(min(next, (long long)a.need) - rank0);  // at most 1,024
    const int64_t base = (int64_t)b * kGaussPerCta;
#pragma unroll 1
    for (int q = threadIdx.x; q < np; q += 256)
    {
        const double2 g = a.pair[base + q];
        const int64_t j = rank0 + q, v = a.v0 + 2 * j;
        gauss_emit(a.sp, a.mean, a.stddev, a.out, v, g.x);
        if (v + 1 < a.M)
            gauss_emit(a.sp, a.mean, a.stddev, a.out, v + 1, g.y);
        else
        {
            a.st->saved = g.y;
            a.st->has_saved = 1;
        }
        if (j == a.need - 1)
            a.ctl->consumed = 4 * (base + a.kidx[base + q] + 1);
    }
}

// Commits the words the chunk used: K = ctl->consumed (or all W words when the chunk fell short).
// raw holds the rest of the generator's current block (r = 624 - pos words) and then whole blocks,
// untempered, so the generator after word K is the block holding word K - 1.
__global__ void __launch_bounds__(256) gauss_advance_kernel(SamplerState *st, const unsigned *raw, int64_t W,
                                                            const GaussChunk *ctl)
{
    const long long c = ctl->consumed;
    const int64_t K = c >= 0 ? c : W;
    const int64_t r = 624 - (int64_t)st->pos;
    __syncthreads();  // every thread has read pos
    if (K <= r)
    {
        if (threadIdx.x == 0)
            st->pos = (unsigned)(624 - r + K);
        return;
    }
    const int64_t start = r + 624 * ((K - r - 1) / 624);
    for (int i = threadIdx.x; i < 624; i += blockDim.x)
        st->mt[i] = raw[start + i];
    if (threadIdx.x == 0)
        st->pos = (unsigned)(K - start);
}

// The same commit when raw holds exactly the words after the sampler's next one (segmented form): the
// generator after word K is the window of the 624 words before it (position 624), taken from the old
// block for the part before raw[0].
__global__ void __launch_bounds__(256) gauss_advance_seg_kernel(SamplerState *st, const unsigned *raw, int64_t W,
                                                                const GaussChunk *ctl)
{
    __shared__ unsigned old[624];
    const long long c = ctl->consumed;
    const int64_t K = c >= 0 ? c : W;
    const int pos = (int)st->pos;
    for (int i = threadIdx.x; i < 624; i += blockDim.x)
        old[i] = st->mt[i];
    __syncthreads();  // every thread has read pos and the block
    const int64_t r = 624 - pos;
    if (K <= r)
    {
        if (threadIdx.x == 0)
            st->pos = (unsigned)(pos + K);
        return;
    }
    for (int i = threadIdx.x; i < 624; i += blockDim.x)
    {
        const int64_t m = K - 624 + i;  // word m of raw (m < 0: the old block's word pos + m)
        st->mt[i] = m < 0 ? old[pos + m] : raw[m];
    }
    if (threadIdx.x == 0)
        st->pos = 624u;
}

int64_t launch_sample_gaussian(const LaunchCfg &lc, SamplerState *st, bool has_saved, const SpaceParams &sp,
                               StatesView meanv, double stddev, int64_t n, MutStatesView out, unsigned *words,
                               int64_t cap_words, GaussChunk *ctl, long long *cnt, double2 *pair,
                               unsigned short *kidx, unsigned *slowlist, unsigned *jump_scratch,
                               const uint32_t *polys, int64_t L)
{
    const int64_t M = n * sp.dim;
    if (M == 0)
        return 0;
    int64_t v = 0;
    if (has_saved)
    {
        gauss_saved_kernel<<<1, 32, 0, lc.stream>>>(st, sp, meanv, stddev, out);
        note_launch();
        v = 1;
    }
    int64_t need = (M - v + 1) / 2, chunks = 0;
    const int64_t gmax = (cap_words - 624) / 4;
    while (need > 0)
    {
        // acceptance pi/4: the expected count plus 8 standard deviations of the candidates needed
        const double mu = (double)need / 0.7853981633974483;
        const int64_t G = std::max<int64_t>(1, std::min<int64_t>(gmax, (int64_t)std::ceil(mu + 8.0 * std::sqrt(mu) + 64.0)));
        const int nb = (int)((G + kGaussPerCta - 1) / kGaussPerCta);
        // segmented (jump-ahead) generation of the candidates' words when the chunk is large
        const bool seg = polys && 4 * G >= ((int64_t)1 << 18);
        if (seg)
            launch_raw_words_jump(lc, st, 4 * G, words, jump_scratch, polys, L);
        else
            mt_words_kernel<true><<<1, 256, 0, lc.stream>>>(st, 4 * G, words);
        cudaMemsetAsync(&ctl->slow, 0, 2 * sizeof(long long), lc.stream);  // slow and slow_cr
        unsigned *crlist = slowlist + gauss_pair_slots(cap_words);
        gauss_pairs_kernel<<<nb, 256, 0, lc.stream>>>((const uint4 *)words, G, cnt, pair, kidx, slowlist, ctl);
        gauss_slow_kernel<<<lc.sm_count * 8, 256, 0, lc.stream>>>((const uint4 *)words, kidx, slowlist, crlist, ctl,
                                                                  pair);
        gauss_cr_kernel<<<lc.sm_count, 256, 0, lc.stream>>>((const uint4 *)words, kidx, crlist, ctl, pair);
        gauss_scan_kernel<<<1, 1024, 0, lc.stream>>>(cnt, nb, ctl);
        GaussArgs a{pair, kidx, cnt, nb, need, v, M, stddev, sp, meanv, out, st, ctl};
        gauss_emit_kernel<<<nb, 256, 0, lc.stream>>>(a);
        if (seg)
            gauss_advance_seg_kernel<<<1, 256, 0, lc.stream>>>(st, words, 4 * G, ctl);
        else
            gauss_advance_kernel<<<1, 256, 0, lc.stream>>>(st, words, 4 * G, ctl);
        for (int i = 0; i < 7; ++i)
            note_launch();
        GaussChunk h{};
        if (cudaMemcpyAsync(&h, ctl, sizeof(h), cudaMemcpyDeviceToHost, lc.stream) != cudaSuccess ||
            cudaStreamSynchronize(lc.stream) != cudaSuccess)
            return -1;
        const int64_t got = std::min<int64_t>(h.accepted, need);
        if (got <= 0)  // >= 64 candidates without one accepted: the stream is broken, not unlucky
            return -1;
        v += 2 * got;
        need -= got;
        ++chunks;
    }
    return chunks;
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

__global__ void log_rn_kernel(const double *x, int64_t n, double *out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        out[i] = log_rn(x[i]);
}

void launch_log_rn(const LaunchCfg &lc, const double *x, int64_t n, double *out)
{
    if (n == 0)
        return;
    log_rn_kernel<<<(int)((n + 255) / 256), 256, 0, lc.stream>>>(x, n, out);
    note_launch();
}

}  // namespace gbo
