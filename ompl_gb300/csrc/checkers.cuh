// Validity predicates on the device.
//
// FP64 forms reproduce the reference's arithmetic operation for operation (exact _rn intrinsics):
//   circles          tests/resources/circles2D.h:141-151
//   kinematic chain  demos/KinematicChain.h:209-276
//   DH sphere arm    no OMPL counterpart: standard DH forward kinematics, spheres evenly spaced along
//                    each link, a pair collides when |c_robot - c_world|^2 < (r_robot + r_world)^2
//                    (kernels.cuh: dh_valid64 fixes the operation order)
//
// FP32_GUARDED forms evaluate every comparison in FP32 together with a bound E on
// |value_fp32 - value_fp64_reference| and classify it as definitely-true, definitely-false or
// ambiguous (|value - threshold| <= E). A state whose outcome depends on an ambiguous comparison is
// re-evaluated with the FP64 form, so the returned boolean always equals the FP64 one.
#pragma once
#include "common.cuh"
#include "chain_warp.cuh"

namespace gbo
{

enum : int
{
    kInvalid = 0,
    kValid = 1,
    kAmbiguous = 2
};

// ---------------------------------------------------------------- circles (FP64)
// world layout in memory: n rows of (x, y, r*r) doubles (r*r formed in FP64 on the host, as circles2D.h:51).
__device__ __forceinline__ bool circles_valid64(const double *w, int n, double x, double y)
{
    for (int i = 0; i < n; ++i)
    {
        double dx = dsub(w[3 * i + 0], x);
        double dy = dsub(w[3 * i + 1], y);
        if (dadd(dmul(dx, dx), dmul(dy, dy)) < w[3 * i + 2])
            return false;
    }
    return true;
}

// ---------------------------------------------------------------- kinematic chain (FP64)
// Segment intersection of demos/KinematicChain.h:251-276.
__device__ __forceinline__ bool seg_intersect64(double ax0, double ay0, double ax1, double ay1, double bx0, double by0,
                                                double bx1, double by1)
{
    double s10_x = dsub(ax1, ax0);
    double s10_y = dsub(ay1, ay0);
    double s32_x = dsub(bx1, bx0);
    double s32_y = dsub(by1, by0);
    double denom = dsub(dmul(s10_x, s32_y), dmul(s32_x, s10_y));
    if (fabs(denom) < kDblEps)
        return false;
    bool denomPositive = denom > 0;
    double s02_x = dsub(ax0, bx0);
    double s02_y = dsub(ay0, by0);
    double s_numer = dsub(dmul(s10_x, s02_y), dmul(s10_y, s02_x));
    if ((s_numer < kFltEps) == denomPositive)
        return false;
    double t_numer = dsub(dmul(s32_x, s02_y), dmul(s32_y, s02_x));
    if ((t_numer < kFltEps) == denomPositive)
        return false;
    if (((dsub(s_numer, denom) > -kFltEps) == denomPositive) || ((dsub(t_numer, denom) > kFltEps) == denomPositive))
        return false;
    return true;
}

// ---------------------------------------------------------------- one-ulp hazards of the FP64 forms
// The FP64 forms evaluate the reference's arithmetic on the same doubles, except that the sines and
// cosines of the forward kinematics are correctly rounded (crtrig.cuh) where the reference calls the C
// library, whose results differ from the correctly rounded ones by one ulp on a small fraction of
// arguments. A decision is a hazard when a comparison lies so close to its threshold that inputs moved
// by that much could change it: the kernels count those in RunCounters::hazards, so a run with no
// hazard took every FP64 decision as the reference does, whatever its C library returned.
//
// Bound on |x'y' - xy| + roundings for inputs moved by at most dx, dy: zero when nothing moved
// (identical inputs give identical results).
__device__ __forceinline__ double prod_move(double x, double y, double dx, double dy)
{
    if (dx == 0.0 && dy == 0.0)
        return 0.0;
    return dx * fabs(y) + fabs(x) * dy + dx * dy + 0x1p-52 * fabs(x * y);
}

// Hazard test of the segment test of demos/KinematicChain.h:251-276 for segment a (endpoints moved by at
// most pa per coordinate) and segment b (pb): `stage` is how far the reference's branch sequence got
// (0: |denom| test, 1: + s_numer test, 2: + t_numer test, 3: + first final clause, 4: + second); a
// hazard is counted on *hz. Comparisons farther than 1e-9 from their thresholds are never hazards here
// (the bounds are below 1e-12 for coordinates of magnitude <= 4), so callers form the bounds only for
// close comparisons.
static __device__ __noinline__ void seg_hazard64(double ax0, double ay0, double ax1, double ay1, double bx0,
                                                double by0, double bx1, double by1, int stage, double pa, double pb,
                                                unsigned long long *hz)
{
    const double s10x = dsub(ax1, ax0), s10y = dsub(ay1, ay0);
    const double s32x = dsub(bx1, bx0), s32y = dsub(by1, by0);
    const double denom = dsub(dmul(s10x, s32y), dmul(s32x, s10y));
    const double s02x = dsub(ax0, bx0), s02y = dsub(ay0, by0);
    const double sn = dsub(dmul(s10x, s02y), dmul(s10y, s02x));
    const double tn = dsub(dmul(s32x, s02y), dmul(s32y, s02x));
    const double u2 = 0x1p-52;
    const double d10x = pa > 0.0 ? 2.0 * pa + u2 * fabs(s10x) : 0.0, d10y = pa > 0.0 ? 2.0 * pa + u2 * fabs(s10y) : 0.0;
    const double d32x = pb > 0.0 ? 2.0 * pb + u2 * fabs(s32x) : 0.0, d32y = pb > 0.0 ? 2.0 * pb + u2 * fabs(s32y) : 0.0;
    const double pp = pa + pb;
    const double d02x = pp > 0.0 ? pp + u2 * fabs(s02x) : 0.0, d02y = pp > 0.0 ? pp + u2 * fabs(s02y) : 0.0;
    auto moved = [&](double m, double v) { return m == 0.0 ? 0.0 : 2.0 * (m + u2 * fabs(v)); };
    const double e_den = moved(prod_move(s10x, s32y, d10x, d32y) + prod_move(s32x, s10y, d32x, d10y), denom);
    const double e_s = moved(prod_move(s10x, s02y, d10x, d02y) + prod_move(s10y, s02x, d10y, d02x), sn);
    const double e_t = moved(prod_move(s32x, s02y, d32x, d02y) + prod_move(s32y, s02x, d32y, d02x), tn);
    bool h = fabs(fabs(denom) - kDblEps) <= e_den || fabs(denom) <= e_den;
    h |= stage >= 1 && fabs(sn - kFltEps) <= e_s;
    h |= stage >= 2 && fabs(tn - kFltEps) <= e_t;
    h |= stage >= 3 && fabs(dsub(sn, denom) + kFltEps) <= moved(e_s + e_den, sn - denom);
    h |= stage >= 4 && fabs(dsub(tn, denom) - kFltEps) <= moved(e_t + e_den, tn - denom);
    if (h)
        atomicAdd(hz, 1ull);
}

// seg_intersect64 that also counts a hazard (atomicAdd on *hz) when one of the comparisons it evaluated
// lies within 1e-9 of its threshold and within the moved-input bound (seg_hazard64, out of line).
__device__ __forceinline__ bool seg_intersect64_hz(double ax0, double ay0, double ax1, double ay1, double bx0,
                                                   double by0, double bx1, double by1, double pa, double pb,
                                                   unsigned long long *hz)
{
    const double s10_x = dsub(ax1, ax0), s10_y = dsub(ay1, ay0);
    const double s32_x = dsub(bx1, bx0), s32_y = dsub(by1, by0);
    const double denom = dsub(dmul(s10_x, s32_y), dmul(s32_x, s10_y));
    const double s02_x = dsub(ax0, bx0), s02_y = dsub(ay0, by0);
    const double s_numer = dsub(dmul(s10_x, s02_y), dmul(s10_y, s02_x));
    const double t_numer = dsub(dmul(s32_x, s02_y), dmul(s32_y, s02_x));
    bool result = true;
    int stage = 0;
    const bool denomPositive = denom > 0;
    if (fabs(denom) < kDblEps)
        result = false;
    else if (stage = 1, (s_numer < kFltEps) == denomPositive)
        result = false;
    else if (stage = 2, (t_numer < kFltEps) == denomPositive)
        result = false;
    else if (stage = 3, (dsub(s_numer, denom) > -kFltEps) == denomPositive)
        result = false;
    else if (stage = 4, (dsub(t_numer, denom) > kFltEps) == denomPositive)
        result = false;
    const double near = 1e-9;
    const bool close = fabs(fabs(denom) - kDblEps) <= near || fabs(denom) <= near ||
                       (stage >= 1 && fabs(s_numer - kFltEps) <= near) || (stage >= 2 && fabs(t_numer - kFltEps) <= near) ||
                       (stage >= 3 && fabs(s_numer - denom + kFltEps) <= near) ||
                       (stage >= 4 && fabs(t_numer - denom - kFltEps) <= near);
    if (hz && close)
        seg_hazard64(ax0, ay0, ax1, ay1, bx0, by0, bx1, by1, stage, pa, pb, hz);
    return result;
}

// Adjacent chain segments (i, i+1) share an endpoint, so in FP64 s02 == -s10 exactly, s_numer == +0 and
// t_numer == denom bitwise; every branch of the test above then reports "no collision". Both forms
// therefore skip adjacent pairs without changing any result.

// FK of demos/KinematicChain.h:214-228 into n+2 points (n links plus the 0.001 tip segment).
template <int MAXD>
__device__ __forceinline__ void chain_points64(const SpaceParams &s, const double *q, double *X, double *Y)
{
    double theta = 0., x = 0., y = 0., c = 1.0, sn = 0.0;
    X[0] = 0.;
    Y[0] = 0.;
#pragma unroll
    for (int i = 0; i < MAXD; ++i)
        if (i < s.dim)
        {
            theta = dadd(theta, q[i]);
            sincos_cr(theta, &sn, &c);
            x = dadd(x, dmul(c, s.link));
            y = dadd(y, dmul(sn, s.link));
            X[i + 1] = x;
            Y[i + 1] = y;
        }
#pragma unroll
    for (int i = 0; i <= MAXD; ++i)
        if (i == s.dim)
        {
            X[i + 1] = dadd(x, dmul(c, 0.001));
            Y[i + 1] = dadd(y, dmul(sn, 0.001));
        }
}

// world: n rows of (x0, y0, x1, y1) doubles. hz_pos bounds how far a joint position can move when
// every sine and cosine moves by one ulp; hazards are counted on *hz (nullable).
template <int MAXD>
__device__ bool chain_valid64(const SpaceParams &s, const double *q, const double *w, int nw, double hz_pos = 0.0,
                              unsigned long long *hz = nullptr)
{
    double X[MAXD + 2], Y[MAXD + 2];
    chain_points64<MAXD>(s, q, X, Y);
    const int m = s.dim + 1;  // segments
#pragma unroll
    for (int i = 0; i < MAXD + 1; ++i)
#pragma unroll
        for (int j = i + 2; j < MAXD + 1; ++j)
            if (j < m)
                if (seg_intersect64_hz(X[i], Y[i], X[i + 1], Y[i + 1], X[j], Y[j], X[j + 1], Y[j + 1], hz_pos, hz_pos,
                                       hz))
                    return false;
#pragma unroll
    for (int i = 0; i < MAXD + 1; ++i)
        if (i < m)
            for (int j = 0; j < nw; ++j)
                if (seg_intersect64_hz(X[i], Y[i], X[i + 1], Y[i + 1], w[4 * j], w[4 * j + 1], w[4 * j + 2],
                                       w[4 * j + 3], hz_pos, 0.0, hz))
                    return false;
    return true;
}

// ---------------------------------------------------------------- kinematic chain (FP32, guarded)
// Per world segment, FP32 data plus its error bounds (filled by the host, see chain_bounds in capi.cu),
// 32 bytes = two 16-byte loads:
//   x0, y0, sx, sy : start point and direction vector (s32) rounded to FP32
//   lo, hi         : FLT_EPSILON - e and FLT_EPSILON + e rounded outward, e a bound on |fp32 - fp64| of
//                    s_numer, t_numer, s_numer - denom and t_numer - denom for a link vs this segment
//   e_den          : bound on |fp32 - fp64| of denom
struct __align__(16) ChainSegF32
{
    float x0, y0, sx, sy, lo, hi, e_den, pad;
};

struct ChainGuard
{
    float eps_dir;                      // bound on |cos/sin fp32 - fp64| of one link direction
    float self_lo, self_hi, self_den;   // lo, hi, e_den of link-vs-link tests
};

// Guarded segment test: returns kInvalid (definite collision), kValid (definite none) or kAmbiguous.
// Branch-free: every clause of demos/KinematicChain.h:267-274 ("(cmp) == denomPositive => no
// collision") is classified, then combined: one clause that definitely holds decides "no
// collision" whatever the others are, a collision needs all four to fail definitely, and an
// undecided zero or sign test of the denominator is undecided. With |x32 - x64| <= e/2 for every
// numerator x (the bounds carry a safety factor of 2), "x < FLT_EPSILON" is definitely true when
// x32 < lo = FLT_EPSILON - e and definitely false when x32 >= hi = FLT_EPSILON + e; the clauses on
// s_numer - denom and t_numer - denom compare against -FLT_EPSILON (thresholds -lo, -hi) and
// +FLT_EPSILON.
__device__ __forceinline__ int seg_intersect32(float s10x, float s10y, float s32x, float s32y, float s02x, float s02y,
                                               float lo, float hi, float e_den)
{
    const float den = fmaf(s10x, s32y, -s32x * s10y);
    const float sn = fmaf(s10x, s02y, -s10y * s02x);
    const float tn = fmaf(s32x, s02y, -s32y * s02x);
    const float un = sn - den, vn = tn - den;
    const bool P = den > 0.f;
    // definite truth (x_t) and definite falsehood (x_f) of each comparison
    const bool s_t = sn < lo, s_f = sn >= hi;
    const bool t_t = tn < lo, t_f = tn >= hi;
    const bool u_t = un > -lo, u_f = un <= -hi;
    const bool v_t = vn > hi, v_f = vn <= lo;
    const bool holds = P ? (s_t || t_t || u_t || v_t) : (s_f || t_f || u_f || v_f);
    const bool undecided = !(s_t || s_f) || !(t_t || t_f) || !(u_t || u_f) || !(v_t || v_f);
    const bool den_undecided = fabsf(den) <= e_den;
    return den_undecided ? kAmbiguous : (holds ? kValid : (undecided ? kAmbiguous : kInvalid));
}

// FP32 link directions from an FP64 angle (thread-per-state forms): the angle is split exactly into
// a float-float pair and evaluated with sincos_ff (chain_warp.cuh); |error| <= 1.3e-7 per component.
__device__ __forceinline__ void dir32(double theta, float &c, float &s)
{
    sincos_ff(split_double(theta), c, s);
}

template <int MAXD>
__device__ int chain_valid32(const SpaceParams &s, const double *q, const ChainSegF32 *w, int nw, const ChainGuard &g)
{
    float X[MAXD + 2], Y[MAXD + 2], VX[MAXD + 1], VY[MAXD + 1];
    const float L = (float)s.link;
    double theta = 0.;
    float x = 0.f, y = 0.f, c = 1.f, sn = 0.f;
    X[0] = 0.f;
    Y[0] = 0.f;
#pragma unroll
    for (int i = 0; i < MAXD; ++i)
        if (i < s.dim)
        {
            theta = dadd(theta, q[i]);
            dir32(theta, c, sn);
            VX[i] = c * L;
            VY[i] = sn * L;
            x = fmaf(c, L, x);
            y = fmaf(sn, L, y);
            X[i + 1] = x;
            Y[i + 1] = y;
        }
#pragma unroll
    for (int i = 0; i <= MAXD; ++i)
        if (i == s.dim)
        {
            VX[i] = c * 0.001f;
            VY[i] = sn * 0.001f;
            X[i + 1] = fmaf(c, 0.001f, x);
            Y[i + 1] = fmaf(sn, 0.001f, y);
        }
    const int m = s.dim + 1;
    bool amb = false;
#pragma unroll
    for (int i = 0; i < MAXD + 1; ++i)
#pragma unroll
        for (int j = i + 2; j < MAXD + 1; ++j)
            if (j < m)
            {
                int r = seg_intersect32(VX[i], VY[i], VX[j], VY[j], X[i] - X[j], Y[i] - Y[j], g.self_lo, g.self_hi,
                                        g.self_den);
                if (r == kInvalid)
                    return kInvalid;
                amb |= (r == kAmbiguous);
            }
    for (int j = 0; j < nw; ++j)
    {
        const ChainSegF32 ws = w[j];
#pragma unroll
        for (int i = 0; i < MAXD + 1; ++i)
            if (i < m)
            {
                int r = seg_intersect32(VX[i], VY[i], ws.sx, ws.sy, X[i] - ws.x0, Y[i] - ws.y0, ws.lo, ws.hi,
                                        ws.e_den);
                if (r == kInvalid)
                    return kInvalid;
                amb |= (r == kAmbiguous);
            }
    }
    return amb ? kAmbiguous : kValid;
}

}  // namespace gbo
