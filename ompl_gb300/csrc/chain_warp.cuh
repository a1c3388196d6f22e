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
#include "common.cuh"

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

// Exact split of a double into hi + lo floats with integer operations only (no conversion
// instruction): hi keeps the top 24 significand bits, lo the next 24 (the last 5 of the 53 are
// truncated, relative error 2^-48). |x| < 2^-74 keeps hi only; |x| < 2^-100 becomes 0.
__device__ __forceinline__ ff split_double(double x)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const unsigned sign = (unsigned)(b >> 63) << 31;
    const int e = (int)((b >> 52) & 0x7ff) - 1023;
    if (e < -100)
        return {0.f, 0.f};
    const unsigned long long m = b & 0xFFFFFFFFFFFFFull;
    const float hi = __int_as_float((int)(sign | ((unsigned)(e + 127) << 23) | (unsigned)(m >> 29)));
    const unsigned rem = (unsigned)(m & 0x1FFFFFFFull);  // 29 low bits, weight 2^(e-52)
    float lo = 0.f;
    if (rem != 0u && e >= -74)
    {
        const int lz = __clz(rem);                        // >= 3
        const int p = 31 - lz;                            // position of the leading bit
        const unsigned mant = p >= 23 ? rem >> (p - 23) : rem << (23 - p);
        lo = __int_as_float((int)(sign | ((unsigned)(p + e - 52 + 127) << 23) | (mant & 0x7FFFFFu)));
    }
    return {hi, lo};
}

// Round to the nearest integer for |x| < 2^22 in the FP32 adder (no rounding instruction).
__device__ __forceinline__ float rint_add(float x)
{
    return (x + 12582912.0f) - 12582912.0f;
}

// Non-negative integer value of a float that holds an integer below 2^22.
__device__ __forceinline__ int int_of(float x)
{
    return __float_as_int(x + 12582912.0f) - 0x4B400000;
}

// Float of a non-negative integer below 2^23.
__device__ __forceinline__ float float_of(int i)
{
    return __int_as_float(0x4B000000 | i) - 8388608.0f;
}

// cos and sin of a float-float angle |t| < 64*pi/2 in FP32 arithmetic only.
// Reduction: k = nearest integer to t*2/pi, y = t - k*pi/2 with pi/2 = P1 + P2 + P3 (P1 8 and P2 18
// significant bits, so k*P1 and k*P2 are exact for |k| < 64; residual of the split ~6e-18).
// On |y| <= pi/4, Taylor polynomials of sin (to y^9) and cos (to y^10), truncation <= 2e-9,
// evaluated by Horner with FMA (rounding <= 2 FP32 ulp); the low part of y enters to first order.
// |result - exact| <= 1.3e-7 per component.
__device__ __forceinline__ void sincos_ff(ff t, float &c, float &s)
{
    constexpr float P1 = 1.5703125f;
    constexpr float P2 = 259753.0f / 536870912.0f;
    constexpr float P3 = -8.705516e-10f;
    const float m = fmaf(t.hi, 0.63661975f, 12582912.0f);
    const float k = m - 12582912.0f;
    const int q = __float_as_int(m) & 3;
    const float y1 = fmaf(-k, P1, t.hi);  // exact
    const ff sy = two_sum(y1, -k * P2);   // k*P2 exact
    const ff y = fast_two_sum(sy.hi, sy.lo + fmaf(-k, P3, t.lo));
    const float x = y.hi, x2 = x * x;
    float sp = fmaf(x2, 2.7557319e-06f, -1.984127e-04f);
    sp = fmaf(sp, x2, 8.333334e-03f);
    sp = fmaf(sp, x2, -0.16666667f);
    const float sn = fmaf(sp * x2, x, x);
    float cp = fmaf(x2, -2.755732e-07f, 2.4801588e-05f);
    cp = fmaf(cp, x2, -1.3888889e-03f);
    cp = fmaf(cp, x2, 4.1666668e-02f);
    cp = fmaf(cp, x2, -0.5f);
    const float cs = fmaf(cp, x2, 1.0f);
    const float s1 = fmaf(cs, y.lo, sn), c1 = fmaf(-sn, y.lo, cs);
    float so = (q & 1) ? c1 : s1;
    float co = (q & 1) ? s1 : c1;
    if (q & 2)
        so = -so;
    if ((q + 1) & 2)
        co = -co;
    s = so;
    c = co;
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

}  // namespace gbo
