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
            sincos(theta, &sn, &c);
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

// world: n rows of (x0, y0, x1, y1) doubles.
template <int MAXD>
__device__ bool chain_valid64(const SpaceParams &s, const double *q, const double *w, int nw)
{
    double X[MAXD + 2], Y[MAXD + 2];
    chain_points64<MAXD>(s, q, X, Y);
    const int m = s.dim + 1;  // segments
#pragma unroll
    for (int i = 0; i < MAXD + 1; ++i)
#pragma unroll
        for (int j = i + 2; j < MAXD + 1; ++j)
            if (j < m)
                if (seg_intersect64(X[i], Y[i], X[i + 1], Y[i + 1], X[j], Y[j], X[j + 1], Y[j + 1]))
                    return false;
#pragma unroll
    for (int i = 0; i < MAXD + 1; ++i)
        if (i < m)
            for (int j = 0; j < nw; ++j)
                if (seg_intersect64(X[i], Y[i], X[i + 1], Y[i + 1], w[4 * j], w[4 * j + 1], w[4 * j + 2],
                                    w[4 * j + 3]))
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
