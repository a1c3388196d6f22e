// Warp-cooperative kinematic-chain state test (uses the guarded segment test of checkers.cuh and
// the FP32 arithmetic of chain_warp.cuh).
#pragma once
#include "checkers.cuh"

namespace gbo
{

__device__ __forceinline__ int chain_test_count(int n_links, int nw, int &n_self)
{
    const int m = n_links + 1;  // segments incl. the tip
    n_self = (m - 1) * (m - 2) / 2;
    return n_self + m * nw;
}

// Fields of a default-order test entry: link a (bits 0-7), second segment b (bits 8-30: a link for a
// link-link pair, else a world segment), link-link flag (bit 31).
__host__ __device__ __forceinline__ int chain_test_a(unsigned e)
{
    return (int)(e & 0xffu);
}
__host__ __device__ __forceinline__ int chain_test_b(unsigned e)
{
    return (int)((e >> 8) & 0x7fffffu);
}

// Default order: self pairs row by row, then world-major link-world pairs.
__host__ __device__ inline unsigned chain_test_entry(int idx, int n_links, int nw)
{
    const int m = n_links + 1;
    const int n_self = (m - 1) * (m - 2) / 2;
    if (idx < n_self)
    {
        int r = idx, i = 0;
        while (r >= m - (i + 2))
        {
            r -= m - (i + 2);
            ++i;
        }
        return (unsigned)i | ((unsigned)(i + 2 + r) << 8) | 0x80000000u;
    }
    const int r = idx - n_self;
    return (unsigned)(r % m) | ((unsigned)(r / m) << 8);
}

// Segments of one state from its absolute link angles: lane k < n holds theta_k = q_0 + ... + q_k as
// float-float. Returns, in lane k <= n, the segment vector V_k and start point P_k (lane n = tip segment).
__device__ __forceinline__ void chain_segments32_theta(ff theta, int lane, int n, float L, float &vx, float &vy,
                                                       float &px, float &py)
{
    float c, s;
    sincos_ff(theta, c, s);
    // tip segment (lane n) uses the last link's direction with length 0.001
    const float cl = __shfl_sync(0xffffffffu, c, n > 0 ? n - 1 : 0);
    const float sl = __shfl_sync(0xffffffffu, s, n > 0 ? n - 1 : 0);
    const bool tip = lane == n;
    vx = lane < n ? c * L : (tip ? cl * 0.001f : 0.f);
    vy = lane < n ? s * L : (tip ? sl * 0.001f : 0.f);
    // end point of segment k = sum_{m<=k} V_m ; start point = end point of segment k-1
    const float ex = warp_scan_f16(vx, lane, n + 1), ey = warp_scan_f16(vy, lane, n + 1);
    px = __shfl_up_sync(0xffffffffu, ex, 1);
    py = __shfl_up_sync(0xffffffffu, ey, 1);
    if (lane == 0)
    {
        px = 0.f;
        py = 0.f;
    }
}

// The same from the joints: lane k < n holds joint k as float-float (zero elsewhere).
__device__ __forceinline__ void chain_segments32(ff q, int lane, int n, float L, float &vx, float &vy, float &px,
                                                 float &py)
{
    chain_segments32_theta(warp_scan_ff(q, lane), lane, n, L, vx, vy, px, py);
}

// FP64 segments of one state in the reference's operation order (KinematicChain.h:214-228): theta
// and the end points accumulate sequentially (lane m's values reach every lane by shuffle), cos/sin
// are evaluated lane-parallel. Lane k <= n receives segment k (lane n: the 0.001 tip segment).
__device__ __forceinline__ void chain_segments64_warp(double q, int lane, int n, double L, double &x0, double &y0,
                                                      double &x1, double &y1)
{
    double th = 0.0, mine = 0.0;
    for (int m = 0; m < n; ++m)
    {
        th = dadd(th, __shfl_sync(0xffffffffu, q, m));
        if (m == lane)
            mine = th;
    }
    double sn, cs;
    sincos_cr(mine, &sn, &cs);
    double x = 0.0, y = 0.0, cl = 1.0, sl = 0.0;
    x0 = y0 = x1 = y1 = 0.0;
    for (int m = 0; m < n; ++m)
    {
        cl = __shfl_sync(0xffffffffu, cs, m);
        sl = __shfl_sync(0xffffffffu, sn, m);
        if (m == lane)
        {
            x0 = x;
            y0 = y;
        }
        x = dadd(x, dmul(cl, L));
        y = dadd(y, dmul(sl, L));
        if (m == lane)
        {
            x1 = x;
            y1 = y;
        }
    }
    if (lane == n)
    {
        x0 = x;
        y0 = y;
        x1 = dadd(x, dmul(cl, 0.001));
        y1 = dadd(y, dmul(sl, 0.001));
    }
}

// One-ulp hazard bound and counter of the running launch, set by the warp kernels' setup (kept in shared
// memory so that the FP32 loops carry no registers for them).
__shared__ double chain_hz_pos;
__shared__ unsigned long long *chain_hz;

// Definite-intersection bitmap of one state over all tests in default order (no early exit).
__device__ __forceinline__ void chain_state_hits32(int lane, float vx, float vy, float px, float py,
                                                   const ChainSegF32 *w, int n_links, int nw, int n_tests,
                                                   ChainGuard g, unsigned *bits)
{
    for (int base = 0; base < n_tests; base += 32)
    {
        const int idx = base + lane;
        const unsigned e = idx < n_tests ? chain_test_entry(idx, n_links, nw) : 0u;
        const int a = chain_test_a(e), b = chain_test_b(e);
        const float ax = __shfl_sync(0xffffffffu, vx, a), ay = __shfl_sync(0xffffffffu, vy, a);
        const float apx = __shfl_sync(0xffffffffu, px, a), apy = __shfl_sync(0xffffffffu, py, a);
        const float bvx = __shfl_sync(0xffffffffu, vx, b & 31), bvy = __shfl_sync(0xffffffffu, vy, b & 31);
        const float bpx = __shfl_sync(0xffffffffu, px, b & 31), bpy = __shfl_sync(0xffffffffu, py, b & 31);
        int r = kValid;
        if (idx < n_tests)
        {
            if (e & 0x80000000u)
                r = seg_intersect32(ax, ay, bvx, bvy, apx - bpx, apy - bpy, g.self_lo, g.self_hi, g.self_den);
            else
            {
                const ChainSegF32 ws = w[b];
                r = seg_intersect32(ax, ay, ws.sx, ws.sy, apx - ws.x0, apy - ws.y0, ws.lo, ws.hi, ws.e_den);
            }
        }
        const unsigned m = __ballot_sync(0xffffffffu, r == kInvalid);
        if (lane == 0)
            bits[base / 32] = m;
    }
}

// Workspace distance of two states given their absolute link angles (lane k < n: theta_k of each, as
// from warp_scan_ff of the joints) and the FP32 segment count. Returns the segment count, or -1 when
// ceil(distance / lvs) is not decided by the error bound.
__device__ __forceinline__ int chain_segment_count_warp(ff ta, ff tb, int lane, int n, float L, float inv_lvs,
                                                        float e_dist, unsigned factor)
{
    float c1, s1, c2, s2;
    sincos_ff(ta, c1, s1);
    sincos_ff(tb, c2, s2);
    const float dx = warp_scan_f16(lane < n ? c1 - c2 : 0.f, lane, n);
    const float dy = warp_scan_f16(lane < n ? s1 - s2 : 0.f, lane, n);
    const float dist = warp_sum_f16(lane < n ? sqrtf(fmaf(dx, dx, dy * dy)) : 0.f, n) * L;
    const float lo = (dist - e_dist) * inv_lvs * (1.0f - 4.0f * 5.96e-8f);
    const float hi = (dist + e_dist) * inv_lvs * (1.0f + 4.0f * 5.96e-8f);
    if (!(lo > 0.f) || !(hi < 4.0e6f))
        return -1;
    float cl = rint_add(lo), ch = rint_add(hi);
    cl += cl < lo ? 1.f : 0.f;  // ceil
    ch += ch < hi ? 1.f : 0.f;
    if (cl == ch)
        return (int)(factor * (unsigned)int_of(cl));
    return -1;
}

}  // namespace gbo
