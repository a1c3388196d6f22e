// Warp-cooperative FP32 evaluation of the kinematic-chain checker (demos/KinematicChain.h:209-276)
// and metric (:105-121) with no FP64 instruction on the bulk path.
//
// One warp evaluates one state. Lane k owns link k: the joint angle is split exactly into a
// float-float pair with integer operations, theta_k = q_0 + ... + q_k is an inclusive warp scan in
// float-float arithmetic (error ~1e-13), reduced modulo 2*pi with an exact three-part constant,
// and cos/sin come from sincosf of the high part plus a first-order correction with the low part.
// Segment endpoints are a warp scan of the link vectors. The 45 link-link and 11*W link-world
// segment tests are then spread over the 32 lanes, 32 tests per round in the order self pairs,
// then world segments; a round with a definite intersection ends the evaluation (ballot). Every
// comparison is classified with the error bounds of the guarded FP32 test (checkers.cuh).
#pragma once
#include "checkers.cuh"

namespace gbo
{

struct ff
{
    float hi, lo;
};

__device__ __forceinline__ ff two_sum(float a, float b)
{
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}

__device__ __forceinline__ ff fast_two_sum(float a, float b)
{
    const float s = a + b;
    return {s, b - (s - a)};
}

__device__ __forceinline__ ff ff_add(ff a, ff b)
{
    const ff s = two_sum(a.hi, b.hi);
    return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}

// Exact split of a double into hi + lo floats using integer operations only (|x| >= 2^-100 or 0;
// smaller magnitudes become 0). hi keeps the top 24 significand bits, lo the next 24.
__device__ __forceinline__ ff split_double(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e < -100)
        return {0.f, 0.f};
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    const float hi = __int_as_float((int)(sign | ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29)));
    const unsigned rem = (unsigned)(m & 0x1FFFFFFFull);                    // 29 low bits, weight 2^(e-52)
    const float lo_abs = e >= -74 ? __uint2float_rz(rem) * __int_as_float((e - 52 + 127) << 23) : 0.f;
    return {hi, sign ? -lo_abs : lo_abs};
}

// 2*pi = C1 + C2 + C3: C1 has 8 significant bits and C2 20, so k*C1 and k*C2 are exact for |k| < 2^11.
__device__ __forceinline__ ff reduce_2pi(ff t)
{
    constexpr float C1 = 6.28125f;
    constexpr float C2 = 519505.0f / 268435456.0f;         // 2*pi - C1 rounded to 20 bits (exact)
    constexpr float C3 = 2.4308403e-10f;                   // 2*pi - C1 - C2 (residual ~5e-18)
    const float k = rintf(t.hi * 0.15915494309189535f);
    const float r1 = fmaf(-k, C1, t.hi);                   // exact
    const ff s = two_sum(r1, -k * C2);                      // k*C2 exact
    return fast_two_sum(s.hi, s.lo + fmaf(-k, C3, t.lo));
}

// cos/sin of a reduced float-float angle: sincosf(hi) corrected to first order in lo.
__device__ __forceinline__ void sincos_ff(ff r, float &c, float &s)
{
    float s0, c0;
    sincosf(r.hi, &s0, &c0);
    c = fmaf(-s0, r.lo, c0);
    s = fmaf(c0, r.lo, s0);
}

// Inclusive warp scan of a float-float value over lanes [0, 32).
__device__ __forceinline__ ff warp_scan_ff(ff v, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const float h = __shfl_up_sync(0xffffffffu, v.hi, o);
        const float l = __shfl_up_sync(0xffffffffu, v.lo, o);
        if (lane >= o)
            v = ff_add(v, {h, l});
    }
    return v;
}

__device__ __forceinline__ float warp_scan_f(float v, int lane)
{
#pragma unroll
    for (int o = 1; o < 32; o <<= 1)
    {
        const float h = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o)
            v += h;
    }
    return v;
}

__device__ __forceinline__ float warp_sum_f(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Per-CTA test tables: tests [0, n_self) are link-link pairs (a, b), tests [n_self, n_self + 11*W)
// link-world pairs; entry = a | (b << 8) for self pairs and link | (world << 8) otherwise.
struct ChainTables
{
    int n_self;
    int n_tests;
};

__device__ __forceinline__ void build_chain_tables(int n_links, int nw, unsigned *tab, ChainTables &t)
{
    const int m = n_links + 1;  // segments incl. the tip
    int n_self = 0;
    for (int i = 0; i < m; ++i)
        for (int j = i + 2; j < m; ++j)
            ++n_self;
    t.n_self = n_self;
    t.n_tests = n_self + m * nw;
    for (int idx = threadIdx.x; idx < t.n_tests; idx += blockDim.x)
    {
        unsigned e;
        if (idx < n_self)
        {
            int r = idx, i = 0;
            while (r >= m - (i + 2))
            {
                r -= m - (i + 2);
                ++i;
            }
            e = (unsigned)i | ((unsigned)(i + 2 + r) << 8);
        }
        else
        {
            const int r = idx - n_self;
            e = (unsigned)(r % m) | ((unsigned)(r / m) << 8);  // world-major: 11 links of a segment adjacent
        }
        tab[idx] = e;
    }
}

// Link directions of one state: lane k < n holds joint k as float-float (zero elsewhere).
// Returns, in lane k <= n, the segment vector V_k and start point P_k (lane n = tip segment).
__device__ __forceinline__ void chain_segments32(ff q, int lane, int n, float L, float &vx, float &vy, float &px,
                                                 float &py)
{
    const ff th = reduce_2pi(warp_scan_ff(q, lane));
    float c, s;
    sincos_ff(th, c, s);
    // tip segment (lane n) uses the last link's direction with length 0.001
    const float cl = __shfl_sync(0xffffffffu, c, n > 0 ? n - 1 : 0);
    const float sl = __shfl_sync(0xffffffffu, s, n > 0 ? n - 1 : 0);
    const bool tip = lane == n;
    vx = lane < n ? c * L : (tip ? cl * 0.001f : 0.f);
    vy = lane < n ? s * L : (tip ? sl * 0.001f : 0.f);
    // end point of segment k = sum_{m<=k} V_m ; start point = end point of segment k-1
    const float ex = warp_scan_f(vx, lane), ey = warp_scan_f(vy, lane);
    px = __shfl_up_sync(0xffffffffu, ex, 1);
    py = __shfl_up_sync(0xffffffffu, ey, 1);
    if (lane == 0)
    {
        px = 0.f;
        py = 0.f;
    }
}

// Warp-cooperative guarded state test. Returns kInvalid, kValid or kAmbiguous (same in all lanes).
__device__ __forceinline__ int chain_state_warp32(int lane, float vx, float vy, float px, float py,
                                                  const ChainSegF32 *w, const unsigned *tab, const ChainTables &t,
                                                  const ChainGuard &g)
{
    bool amb = false;
    for (int base = 0; base < t.n_tests; base += 32)
    {
        const int idx = base + lane;
        int r = kValid;
        const unsigned e = idx < t.n_tests ? tab[idx] : 0u;
        const int a = (int)(e & 0xff), b = (int)(e >> 8);
        const float ax = __shfl_sync(0xffffffffu, vx, a), ay = __shfl_sync(0xffffffffu, vy, a);
        const float apx = __shfl_sync(0xffffffffu, px, a), apy = __shfl_sync(0xffffffffu, py, a);
        const bool self = idx < t.n_self;
        const float bvx = __shfl_sync(0xffffffffu, vx, b & 31), bvy = __shfl_sync(0xffffffffu, vy, b & 31);
        const float bpx = __shfl_sync(0xffffffffu, px, b & 31), bpy = __shfl_sync(0xffffffffu, py, b & 31);
        if (idx < t.n_tests)
        {
            if (self)
                r = seg_intersect32(ax, ay, bvx, bvy, apx - bpx, apy - bpy, g.self_den, g.self_s, g.self_t, g.self_u,
                                    g.self_v);
            else
            {
                const ChainSegF32 ws = w[b];
                r = seg_intersect32(ax, ay, ws.sx, ws.sy, apx - ws.x0, apy - ws.y0, ws.e_den, ws.e_s, ws.e_t, ws.e_u,
                                    ws.e_v);
            }
        }
        if (__any_sync(0xffffffffu, r == kInvalid))
            return kInvalid;
        amb |= __any_sync(0xffffffffu, r == kAmbiguous);
    }
    return amb ? kAmbiguous : kValid;
}

// Workspace distance of two states (lane k < n holds joint k of each) and the FP32 segment count.
// Returns the segment count, or -1 when ceil(distance / lvs) is not decided by the error bound.
__device__ __forceinline__ int chain_segment_count_warp(ff qa, ff qb, int lane, int n, float L, float inv_lvs,
                                                        float e_dist, unsigned factor)
{
    float c1, s1, c2, s2;
    sincos_ff(reduce_2pi(warp_scan_ff(qa, lane)), c1, s1);
    sincos_ff(reduce_2pi(warp_scan_ff(qb, lane)), c2, s2);
    const float dx = warp_scan_f(lane < n ? c1 - c2 : 0.f, lane);
    const float dy = warp_scan_f(lane < n ? s1 - s2 : 0.f, lane);
    const float dist = warp_sum_f(lane < n ? sqrtf(fmaf(dx, dx, dy * dy)) : 0.f) * L;
    const float lo = (dist - e_dist) * inv_lvs * (1.0f - 4.0f * 5.96e-8f);
    const float hi = (dist + e_dist) * inv_lvs * (1.0f + 4.0f * 5.96e-8f);
    const float cl = ceilf(lo), ch = ceilf(hi);
    if (cl == ch && lo > 0.f)
        return (int)(factor * (unsigned)cl);
    return -1;
}

}  // namespace gbo
