// Kinematic-chain state test of the warp kernels: two segment tests per lane in packed FP32 (f32x2)
// arithmetic, world segments held in registers, one ballot per round of 64 tests.
//
// The segment test of demos/KinematicChain.h:251-276 reports a collision of link a (start p, vector
// v) and segment b (start b0, vector s) exactly when |denom| >= DBL_EPSILON and, for denom > 0, all of
//   c1 = s_numer - F >= 0,  c2 = t_numer - F >= 0,  c3 = -F - (s_numer - denom) >= 0,
//   c4 = F - (t_numer - denom) >= 0
// hold (F = FLT_EPSILON), and for denom < 0 when all four are < 0. With sigma = sign(denom) and
// d_i = sigma c_i, a collision therefore needs min_i d_i >= 0 (> 0 for denom < 0). The FP32 values
// are those of the guarded test of checkers.cuh (same products, same roundings; the host bound e of
// a world segment covers |x32 - x64| <= e/2 for every numerator x, e_den likewise for denom), so:
//   |denom32| <= e_den                       ambiguous (sign or zero test undecided)
//   min d32 > e                              definite collision
//   min d32 < -e                             definitely none
//   otherwise                                ambiguous
// (fl(x - F) > e implies x - F > e (1 - 2^-24), hence x64 - F > e/2 - 2^-24 e > 0; symmetrically for
// < -e.) An ambiguous test is settled by the FP64 reference-order test; the boolean of every state
// equals the FP64 one.
//
// Layout in shared memory (per CTA): world segments in pairs, 48 bytes each ({x0, y0}, {sx, sy},
// {e, e_den} as pairs of floats); per warp, link records LB[k] = {(px, px), (py, py)}, {(vx, vx),
// (-vy, -vy)} (the link as broadcast pairs) and link-pair records LP[r] in the world-pair format for
// segments (r + 2, r + 3) (the last one pairs the tip segment with a null segment), then a null
// record. A null segment (far away, zero vector, e tiny, e_den -1) is definitely clear of everything.
//
// Rounds ("units"), in an order chosen at checker creation (likely collisions first):
//   world unit (c, lr): lane l tests link a = lr + R * (l >> 4) (R = ceil(segments / 2)) against the
//     two world segments of pair (l & 15) of chunk c (32 world segments per chunk), held in registers;
//   self unit s: lane l tests entry 32 s + l of the self table, (link a, link pair record r): the
//     link-link pairs (a, b), b >= a + 2 (adjacent segments never meet in the reference's arithmetic).
#pragma once
#include "chain_state.cuh"
#include "kernels.cuh"

namespace gbo
{

typedef unsigned long long f2;  // two floats: first in the low word

__device__ __forceinline__ f2 f2_pack(float a, float b)
{
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 r, float &a, float &b)
{
    asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r));
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b)
{
    f2 d;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b)
{
    f2 d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b)
{
    f2 d;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c)
{
    f2 d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ float fmin3(float a, float b, float c)
{
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}

// Second segment of a packed pair test: two segments with start (X0, Y0), negated x and plain y of the
// vector (NSX, SY), bounds (E, ED).
struct SegPair
{
    f2 X0, Y0, NSX, SY, E, ED;
};

__device__ __forceinline__ SegPair load_seg_pair(const ulonglong2 *rec)
{
    const ulonglong2 r0 = rec[0], r1 = rec[1], r2 = rec[2];
    return SegPair{r0.x, r0.y, r1.x, r1.y, r2.x, r2.y};
}

// Classification of one FP32 test from its quantities (one half): returns 2 bits: bit 0 = not
// definitely clear (a collision or an ambiguous test), bit 1 = definite collision. c2n is -c2.
__device__ __forceinline__ unsigned classify_half(float den, float c1, float c2n, float c3, float c4, float e, float ed)
{
    const unsigned s = __float_as_uint(den) & 0x80000000u;
    const float d1 = __uint_as_float(__float_as_uint(c1) ^ s);
    const float d2 = __uint_as_float(__float_as_uint(c2n) ^ s ^ 0x80000000u);
    const float d3 = __uint_as_float(__float_as_uint(c3) ^ s), d4 = __uint_as_float(__float_as_uint(c4) ^ s);
    const float m = fminf(fmin3(d1, d2, d3), d4);
    const bool den_undecided = fabsf(den) <= ed;
    const bool bad = den_undecided || !(m < -e);
    const bool hit = !den_undecided && m > e;
    return (bad ? 1u : 0u) | (hit ? 2u : 0u);
}

// Two tests of link (PX2, PY2, VX2, VY2) against a segment pair: 2 bits per test (bits 0-1: first,
// 2-3: second), see classify_half. The products and roundings are those of seg_intersect32
// (checkers.cuh), written with negated operands where that is exact:
//   den = fma(vx, sy, (-sx) vy),  s_numer = fma(vx, cy, vy (-cx)),  -t_numer = fma(-sx, cy, sy cx)
// with c = p - b0; then c1 = s_numer - F, -c2 = -t_numer + F, c3 = -F - (s_numer - den),
// c4 = F + (-t_numer + den) = F - (t_numer - den).
__device__ __forceinline__ unsigned pair_test(f2 PX2, f2 PY2, f2 VX2, f2 VY2, const SegPair &b)
{
    constexpr float F = 1.1920928955078125e-07f;
    const f2 F2 = f2_pack(F, F), NF2 = f2_pack(-F, -F);
    const f2 CX = f2_sub(PX2, b.X0), NCX = f2_sub(b.X0, PX2), CY = f2_sub(PY2, b.Y0);
    const f2 DEN = f2_fma(VX2, b.SY, f2_mul(b.NSX, VY2));
    const f2 SN = f2_fma(VX2, CY, f2_mul(VY2, NCX));
    const f2 NTN = f2_fma(b.NSX, CY, f2_mul(b.SY, CX));
    const f2 C1 = f2_sub(SN, F2), C3 = f2_sub(NF2, f2_sub(SN, DEN));
    const f2 C2N = f2_add(NTN, F2), C4 = f2_add(F2, f2_add(NTN, DEN));
    float den0, den1, a0, a1, b0, b1, c0, c1, d0, d1, e0, e1, ed0, ed1;
    f2_unpack(DEN, den0, den1);
    f2_unpack(C1, a0, a1);
    f2_unpack(C2N, b0, b1);
    f2_unpack(C3, c0, c1);
    f2_unpack(C4, d0, d1);
    f2_unpack(b.E, e0, e1);
    f2_unpack(b.ED, ed0, ed1);
    return classify_half(den0, a0, b0, c0, d0, e0, ed0) | (classify_half(den1, a1, b1, c1, d1, e1, ed1) << 2);
}

// The warp kernels' dynamic shared memory (kernels_chain.cu lays it out).
extern __shared__ __align__(128) unsigned char chain_smem[];

// Byte offsets into chain_smem of a warp's chain data (32-bit, so that they take one register each).
struct ChainWarp
{
    unsigned lb;        // warp: link records (2 ulonglong2 each), segments 0..m-1
    unsigned lp;        // warp: link-pair records (3 ulonglong2 each), r = 0..m-2 (m-2: null)
    unsigned self_tab;  // CTA: self table, entries a | (r << 8), padded to whole rounds
    unsigned units;     // CTA: round order (u16)
    int m, R;
};

__device__ __forceinline__ const ulonglong2 *chain_rec(unsigned off)
{
    return (const ulonglong2 *)(chain_smem + off);
}

// Writes the state's link records: lane k < m holds segment k (start px, py; vector vx, vy).
// Warp-collective.
__device__ __forceinline__ void write_link_records(const ChainWarp &cw, int lane, float vx, float vy, float px,
                                                   float py)
{
    const float nx = __shfl_down_sync(0xffffffffu, px, 1), ny = __shfl_down_sync(0xffffffffu, py, 1);
    const float nvx = __shfl_down_sync(0xffffffffu, vx, 1), nvy = __shfl_down_sync(0xffffffffu, vy, 1);
    __syncwarp();  // the previous state's records are no longer read
    if (lane < cw.m)
    {
        ulonglong2 *r = (ulonglong2 *)(chain_smem + cw.lb) + 2 * lane;
        r[0] = make_ulonglong2(f2_pack(px, px), f2_pack(py, py));
        r[1] = make_ulonglong2(f2_pack(vx, vx), f2_pack(vy, vy));
    }
    if (lane >= 2 && lane < cw.m)
    {
        const bool tip = lane == cw.m - 1;
        ulonglong2 *r = (ulonglong2 *)(chain_smem + cw.lp) + 3 * (lane - 2);
        r[0] = make_ulonglong2(f2_pack(px, tip ? kNullCoord : nx), f2_pack(py, tip ? kNullCoord : ny));
        r[1] = make_ulonglong2(f2_pack(-vx, tip ? 0.f : -nvx), f2_pack(vy, tip ? 0.f : nvy));
    }
    __syncwarp();
}

// FP64 re-check of the ambiguous tests of one round (warp-collective; out of line so that the FP32
// loop carries no FP64 state): `amb` holds the lane's ambiguous halves (bit 0: first, bit 1: second),
// a the link, b the first segment of the pair (a world segment index, or a link index when link is
// set; the second is b + 1). Builds the state's FP64 segments in the reference's order from joint
// `lane` (q), counts one-ulp hazards (chain_hz). Returns true when one of them collides.
static __device__ __noinline__ bool chain_resolve64(int lane, int n, double L64, double q, unsigned amb, int a, int b,
                                                    bool link, const double *w64)
{
    const double hz_pos = chain_hz_pos;
    unsigned long long *hz = chain_hz;
    double sx0, sy0, sx1, sy1;
    chain_segments64_warp(q, lane, n, L64, sx0, sy0, sx1, sy1);
    const double ax0 = __shfl_sync(0xffffffffu, sx0, a & 31), ay0 = __shfl_sync(0xffffffffu, sy0, a & 31);
    const double ax1 = __shfl_sync(0xffffffffu, sx1, a & 31), ay1 = __shfl_sync(0xffffffffu, sy1, a & 31);
    bool hit = false;
    for (int h = 0; h < 2; ++h)
    {
        const int bb = b + h;
        const double bx0 = __shfl_sync(0xffffffffu, sx0, bb & 31), by0 = __shfl_sync(0xffffffffu, sy0, bb & 31);
        const double bx1 = __shfl_sync(0xffffffffu, sx1, bb & 31), by1 = __shfl_sync(0xffffffffu, sy1, bb & 31);
        if (amb >> h & 1u)
        {
            if (link)
                hit |= seg_intersect64_hz(ax0, ay0, ax1, ay1, bx0, by0, bx1, by1, hz_pos, hz_pos, hz);
            else
            {
                const double *o = w64 + 4 * (size_t)bb;
                hit |= seg_intersect64_hz(ax0, ay0, ax1, ay1, o[0], o[1], o[2], o[3], hz_pos, 0.0, hz);
            }
        }
    }
    return __any_sync(0xffffffffu, hit);
}

// Warp-cooperative state test after write_link_records: kInvalid, kValid or (RESOLVE false) kAmbiguous,
// the same in all lanes. `mine` is the lane's world pair of chunk `chunk` (reloaded here when a unit of
// another chunk comes up). Without RESOLVE, a round whose tests are clear or ambiguous but not
// definitely colliding ends the test with kAmbiguous (the caller defers the edge or state to the
// resolving pass); with RESOLVE, its ambiguous tests are re-evaluated in FP64 (q64(lane) gives joint
// `lane` of the state in FP64) and `rechecked` counts the states that needed it.
template <bool RESOLVE, class Q64>
__device__ __forceinline__ int chain_state_test(const ChainWarp &cw, const WorldArgs &wa, int lane, int n,
                                                double L64, SegPair &mine, int &chunk, Q64 q64, unsigned &rechecked)
{
    bool have64 = false;
    const int g = lane >> 4, p = lane & 15;
    const unsigned short *units = (const unsigned short *)(chain_smem + cw.units);
    for (int k = 0; k < wa.n_units; ++k)
    {
        const int u = units[k];
        int a, b;
        bool link;
        unsigned cls;
        if (u < wa.n_self_units)
        {
            const unsigned e = ((const unsigned *)(chain_smem + cw.self_tab))[32 * u + lane];
            a = (int)(e & 0xffu);
            const int r = (int)(e >> 8);
            const ulonglong2 *l = chain_rec(cw.lb) + 2 * a;
            const ulonglong2 l0 = l[0], l1 = l[1];
            cls = pair_test(l0.x, l0.y, l1.x, l1.y, load_seg_pair(chain_rec(cw.lp) + 3 * r));
            b = r + 2;
            link = true;
        }
        else
        {
            const int w = u - wa.n_self_units, c = w / cw.R, lr = w - c * cw.R;
            if (c != chunk)
            {
                chunk = c;
                const int pi = c * 16 + p;
                mine = load_seg_pair(chain_rec(0) + 3 * (pi < wa.n_pairs ? pi : wa.n_pairs));
            }
            a = lr + cw.R * g;
            const bool live = a < cw.m;
            a = live ? a : 0;
            const ulonglong2 *l = chain_rec(cw.lb) + 2 * a;
            const ulonglong2 l0 = l[0], l1 = l[1];
            cls = pair_test(l0.x, l0.y, l1.x, l1.y, mine);
            cls = live ? cls : 0u;
            b = 32 * c + 2 * p;
            link = false;
        }
        if (__ballot_sync(0xffffffffu, (cls & 5u) != 0u))
        {
            if (__any_sync(0xffffffffu, (cls & 10u) != 0u))
                return kInvalid;
            if constexpr (!RESOLVE)
                return kAmbiguous;
            else
            {
                const unsigned amb = (cls & 1u) | ((cls >> 1) & 2u);  // ambiguous halves (bad, no definite hit)
                if (!have64)
                {
                    have64 = true;
                    ++rechecked;
                }
                if (chain_resolve64(lane, n, L64, q64(lane), amb, a, b, link, (const double *)wa.data64))
                    return kInvalid;
            }
        }
    }
    return kValid;
}

}  // namespace gbo
