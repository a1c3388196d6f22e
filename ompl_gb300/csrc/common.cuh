// Shared device definitions: layouts, space parameters, FP64 arithmetic in OMPL's exact operation
// order (explicit _rn intrinsics, which the compiler never fuses into FMA), and FP32 helpers.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/gbompl.h"
#include "crtrig.cuh"

#define GBO_MAXD 16
#define GBO_PI 3.141592653589793238462643383279502884

namespace gbo
{

struct SpaceParams
{
    int kind;
    int dim;
    unsigned factor;
    double lvs;
    double link;        // KINEMATIC_CHAIN link length
    double low[GBO_MAXD];
    double high[GBO_MAXD];
};

// Batch view of states: value (i, d) at p[i * si + d * sd].
struct StatesView
{
    const double *p;
    int64_t si, sd;
    __host__ __device__ double operator()(int64_t i, int d) const
    {
        return p[i * si + (int64_t)d * sd];
    }
};

inline StatesView make_view(const double *p, int64_t ld, int layout)
{
    StatesView v;
    v.p = p;
    if (layout == GBO_LAYOUT_SOA)
    {
        v.si = 1;
        v.sd = ld;
    }
    else
    {
        v.si = ld;
        v.sd = 1;
    }
    return v;
}

struct MutStatesView
{
    double *p;
    int64_t si, sd;
    __device__ double &operator()(int64_t i, int d) const
    {
        return p[i * si + (int64_t)d * sd];
    }
};

// ---------------------------------------------------------------- exact FP64 (no contraction)
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double ddiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ double dsqrt(double a) { return __dsqrt_rn(a); }

constexpr double kPi = GBO_PI;
constexpr double kTwoPi = 2.0 * GBO_PI;  // exact doubling of the double pi, as 2.0 * pi in OMPL
constexpr double kDblEps = 2.220446049250313080847263336181640625e-16;
constexpr double kFltEps = 1.1920928955078125e-07;

// distance(a, b) in OMPL's operation order for each space kind.
//   REAL_VECTOR: RealVectorStateSpace.cpp:230-242; SO2: SO2StateSpace.cpp:114-126;
//   KINEMATIC_CHAIN: demos/KinematicChain.h:105-121; WRAP_L2: L2 of per-joint wrapped differences.
// CR: sines and cosines correctly rounded (sincos_cr); otherwise CUDA's FP64 sincos (within 2 ulp, far
// cheaper on GB300's FP64 pipe), used by the re-check paths of the FP32 forms.
template <int MAXD, bool CR = true>
__device__ double distance64(const SpaceParams &s, const double *a, const double *b)
{
    const int n = s.dim;
    if (s.kind == GBO_SPACE_SO2)
    {
        double d = fabs(dsub(a[0], b[0]));
        return (d > kPi) ? dsub(kTwoPi, d) : d;
    }
    if (s.kind == GBO_SPACE_KINEMATIC_CHAIN)
    {
        double t1 = 0., t2 = 0., dx = 0., dy = 0., dist = 0.;
#pragma unroll
        for (int i = 0; i < MAXD; ++i)
            if (i < n)
            {
                t1 = dadd(t1, a[i]);
                t2 = dadd(t2, b[i]);
                double s1, c1, s2, c2;
                if (CR)
                {
                    sincos_cr(t1, &s1, &c1);
                    sincos_cr(t2, &s2, &c2);
                }
                else
                {
                    sincos(t1, &s1, &c1);
                    sincos(t2, &s2, &c2);
                }
                dx = dadd(dx, dsub(c1, c2));
                dy = dadd(dy, dsub(s1, s2));
                dist = dadd(dist, dsqrt(dadd(dmul(dx, dx), dmul(dy, dy))));
            }
        return dmul(dist, s.link);
    }
    double sum = 0.0;
#pragma unroll
    for (int i = 0; i < MAXD; ++i)
        if (i < n)
        {
            double d = dsub(a[i], b[i]);
            if (s.kind == GBO_SPACE_WRAP_L2)
            {
                d = fabs(d);
                if (d > kPi)
                    d = dsub(kTwoPi, d);
            }
            sum = dadd(sum, dmul(d, d));
        }
    return dsqrt(sum);
}

// One joint of the shortest-arc interpolation of SO2StateSpace.cpp:134-153 / KinematicChain.h:150-176.
__device__ __forceinline__ double interp_angle64(double from, double to, double t)
{
    double diff = dsub(to, from);
    if (fabs(diff) <= kPi)
        return dadd(from, dmul(diff, t));
    diff = diff > 0.0 ? dsub(kTwoPi, diff) : dsub(-kTwoPi, diff);
    double v = dsub(from, dmul(diff, t));
    if (v > kPi)
        v = dsub(v, kTwoPi);
    else if (v < -kPi)
        v = dadd(v, kTwoPi);
    return v;
}

// interpolate(from, to, t) (RealVectorStateSpace.cpp:257-265 or per-joint shortest arc).
template <int MAXD>
__device__ void interpolate64(const SpaceParams &s, const double *from, const double *to, double t, double *out)
{
#pragma unroll
    for (int i = 0; i < MAXD; ++i)
        if (i < s.dim)
            out[i] = s.kind == GBO_SPACE_REAL_VECTOR ? dadd(from[i], dmul(dsub(to[i], from[i]), t))
                                                     : interp_angle64(from[i], to[i], t);
}

// StateSpace::validSegmentCount (StateSpace.cpp:851-854) given the FP64 distance.
__device__ __forceinline__ int segment_count_from_distance(const SpaceParams &s, double d)
{
    return (int)(s.factor * (unsigned)ceil(ddiv(d, s.lvs)));
}

// ---------------------------------------------------------------- launch accounting / errors
struct DeviceFlags
{
    unsigned int timeout;  // a bounded wait ran out
    unsigned int error;    // any other device-detected error
};

}  // namespace gbo
