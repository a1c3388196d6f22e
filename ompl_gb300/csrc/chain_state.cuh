// Warp-cooperative kinematic-chain state test (uses the guarded segment test of checkers.cuh and
// the FP32 arithmetic of chain_warp.cuh).
#pragma once
#include "checkers.cuh"

namespace gbo
{

// Per-CTA test tables: one entry per segment test, a | (b << 8) with bit 31 set for a link-link pair
// (a, b) and clear for link a vs world segment b.
struct ChainTables
{
    int n_self;
    int n_tests;
};

__device__ __forceinline__ int chain_test_count(int n_links, int nw, int &n_self)
{
    const int m = n_links + 1;  // segments incl. the tip
    n_self = (m - 1) * (m - 2) / 2;
    return n_self + m * nw;
}

// Fields of a table entry: link a (bits 0-7), second segment b (bits 8-30: a link for a link-link
// pair, else a world segment), link-link flag (bit 31).
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

// Per-warp tables in shared memory: `order` (device, optional) is a permutation of the default entries
// chosen on the host so that likely intersections come first (bit 31 marks a link-link pair). Warp q's
// table resolves every test to the indices of its two records in the CTA's record array (world
// segments at [0, nw), warp q's links at [lb_q, lb_q + n_links + 1)): first | (second << 16). The
// record array lives in shared memory (at most 7,264 records of 32 bytes), so 16 bits hold an index.
__device__ __forceinline__ void build_chain_tables(int n_links, int nw, const unsigned *order, unsigned *tabs,
                                                   int n_warps, ChainTables &t)
{
    int n_self;
    t.n_tests = chain_test_count(n_links, nw, n_self);
    t.n_self = n_self;
    const int total = n_warps * t.n_tests;
    for (int k = threadIdx.x; k < total; k += blockDim.x)
    {
        const int q = k / t.n_tests, idx = k - q * t.n_tests;
        const unsigned e = order ? order[idx] : chain_test_entry(idx, n_links, nw);
        const int lb = nw + q * (n_links + 1);
        const int ia = lb + chain_test_a(e);
        const int ib = (e & 0x80000000u) ? lb + chain_test_b(e) : chain_test_b(e);
        tabs[k] = (unsigned)ia | ((unsigned)ib << 16);
    }
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
    const float ex = warp_scan_f(vx, lane), ey = warp_scan_f(vy, lane);
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
    sincos(mine, &sn, &cs);  // CUDA's FP64 sincos: one-ulp hazards are counted with its bound
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

// Per-warp link records: the CTA's shared memory holds, after the world's segments, one block of
// n_links + 1 ChainSegF32 records per warp, laid out like a world segment (start point, vector,
// then the link-link error bounds), so that a link-link test reads its second segment exactly as a
// link-world test reads a world segment. The bounds are written once per CTA; the start point and
// vector are rewritten for every state the warp evaluates.
__device__ __forceinline__ void init_chain_links(ChainSegF32 *links, int count, const ChainGuard &g)
{
    for (int k = threadIdx.x; k < count; k += blockDim.x)
        links[k] = ChainSegF32{0.f, 0.f, 0.f, 0.f, g.self_lo, g.self_hi, g.self_den, 0.f};
}

// FP64 re-evaluation of the tests of one round whose FP32 result is ambiguous (reference operation
// order): builds the state's FP64 segments from q = joint `lane` in FP64 and reruns the lanes whose
// r is kAmbiguous. Warp-collective. Out of line so that the FP32 loop carries no FP64 values.
// e: the lane's table entry (record indices, see build_chain_tables); nw, lb: world size and the
// warp's first link record.
// One-ulp hazard bound and counter of the running launch, set by the warp kernels' setup (kept in shared
// memory so that the FP32 loops carry no registers for them).
__shared__ double chain_hz_pos;
__shared__ unsigned long long *chain_hz;

static __device__ __noinline__ int chain_round64(int lane, int n, double L64, double q, unsigned e, int nw, int lb,
                                                 int r, const double *w64)
{
    const double hz_pos = chain_hz_pos;
    unsigned long long *hz = chain_hz;
    double sx0, sy0, sx1, sy1;
    chain_segments64_warp(q, lane, n, L64, sx0, sy0, sx1, sy1);
    const int ib = (int)(e >> 16);
    const bool link = ib >= nw;
    const int a = (int)(e & 0xffffu) - lb, b = link ? ib - lb : ib;
    const double ax0 = __shfl_sync(0xffffffffu, sx0, a), ay0 = __shfl_sync(0xffffffffu, sy0, a);
    const double ax1 = __shfl_sync(0xffffffffu, sx1, a), ay1 = __shfl_sync(0xffffffffu, sy1, a);
    const double bx0 = __shfl_sync(0xffffffffu, sx0, b & 31), by0 = __shfl_sync(0xffffffffu, sy0, b & 31);
    const double bx1 = __shfl_sync(0xffffffffu, sx1, b & 31), by1 = __shfl_sync(0xffffffffu, sy1, b & 31);
    if (r != kAmbiguous)
        return r;
    bool hit;
    if (link)
        hit = seg_intersect64_hz(ax0, ay0, ax1, ay1, bx0, by0, bx1, by1, hz_pos, hz_pos, hz);
    else
    {
        const double *o = w64 + 4 * (size_t)b;
        hit = seg_intersect64_hz(ax0, ay0, ax1, ay1, o[0], o[1], o[2], o[3], hz_pos, 0.0, hz);
    }
    return hit ? kInvalid : kValid;
}

// Warp-cooperative state test: kInvalid or kValid (same in all lanes). Lane k <= n holds segment k
// of the state (vector vx, vy; start px, py). `w` is the CTA's shared record array: the world's
// segments at [0, nw), this warp's link records at [lb, lb + n + 1); `tab` is this warp's table of
// record indices. Tests run 32 per round in table order; a round with an ambiguous FP32 result
// re-evaluates those tests with the FP64 reference code (chain_round64) from q64(lane) = joint `lane`
// of the state in FP64. `rechecked` counts states that needed FP64.
template <class Q64>
__device__ __forceinline__ int chain_state_warp32(int lane, int n, double L64, float vx, float vy, float px,
                                                  float py, ChainSegF32 *w, int nw, int lb, const double *w64,
                                                  const unsigned *tab, ChainTables t, Q64 q64, unsigned &rechecked)
{
    __syncwarp();  // the previous state's records are no longer read
    if (lane <= n)
        *(float4 *)&w[lb + lane] = make_float4(px, py, vx, vy);
    __syncwarp();
    bool have64 = false;
    for (int base = 0; base < t.n_tests; base += 32)
    {
        const int idx = base + lane;
        int r = kValid;
        unsigned e = 0u;
        if (idx < t.n_tests)
        {
            e = tab[idx];
            const float4 A = *(const float4 *)&w[e & 0xffffu];
            const ChainSegF32 B = w[e >> 16];
            r = seg_intersect32(A.z, A.w, B.sx, B.sy, A.x - B.x0, A.y - B.y0, B.lo, B.hi, B.e_den);
        }
        if (__ballot_sync(0xffffffffu, r != kValid))
        {
            if (__any_sync(0xffffffffu, r == kAmbiguous))
            {
                if (!have64)
                {
                    have64 = true;
                    ++rechecked;
                }
                r = chain_round64(lane, n, L64, q64(lane), e, nw, lb, r, w64);
            }
            if (__any_sync(0xffffffffu, r == kInvalid))
                return kInvalid;
        }
    }
    return kValid;
}

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
    const float dx = warp_scan_f(lane < n ? c1 - c2 : 0.f, lane);
    const float dy = warp_scan_f(lane < n ? s1 - s2 : 0.f, lane);
    const float dist = warp_sum_f(lane < n ? sqrtf(fmaf(dx, dx, dy * dy)) : 0.f) * L;
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
