// sin and cos of a double, correctly rounded: evaluated as a double-double whose relative error is
// about 2^-100 and rounded once, so the result is the double nearest the exact value except when that
// value lies within 2^-100 of a rounding midpoint (not met on any tested argument).
//
// Method (no table, no library call; valid for |x| < 2^20):
//   Cody and Waite's additive reduction x = k pi/2 + y, k = nearest integer to x 2/pi, with pi/2 split
//   into C1 + C2 + C3 + C4 (C1, C2 rounded to 33 significant bits, so k C1 and k C2 are exact for
//   |k| < 2^20; C3, C4 to 53 bits). x - k C1 is exact (Sterbenz), y is carried as a double-double.
//   On |y| <= pi/4 (plus rounding): sin y = y sum_{n>=0} (-1)^n y^2n / (2n+1)! and
//   cos y = sum_{n>=0} (-1)^n y^2n / (2n)!, by Horner's rule in z = y^2: the terms n >= 7 (below
//   2^-44 of the sum) in plain FP64, the rest in double-double arithmetic (crlog.cuh); truncation
//   after n = 14 (sin) and n = 15 (cos) is below 2^-110. The quadrant k mod 4 selects +-sin y or
//   +-cos y.
// Constants: pi/2 and the series coefficients (-1)^n/(2n+1)!, (-1)^n/(2n)! from their definitions in
// 400-bit arithmetic, each rounded to a double-double (leading double nearest the value, trailing
// double nearest the remainder); the trailing parts of coefficients n >= 7 are not needed.
//
// The FP64 forms of the kinematic chain and the DH arm use it so that their link directions are the
// correctly rounded values that the C library returns in all but a small fraction of arguments (the
// FP64 decisions that a one-ulp difference could change are counted, see the hazard counters).
#pragma once
#include "crlog.cuh"

namespace gbo
{

static __device__ __noinline__ void sincos_cr(double x, double *sn, double *cs)
{
    constexpr double C1 = 0x1.921fb54400000p+0, C2 = 0x1.0b4611a600000p-34, C3 = 0x1.3198a2e037073p-69,
                     C4 = 0x1.129024e088a68p-123, kTwoOverPi = 0x1.45f306dc9c883p-1;
    constexpr double SH[15] = {0x1.0000000000000p+0,  -0x1.5555555555555p-3,  0x1.1111111111111p-7,
                               -0x1.a01a01a01a01ap-13, 0x1.71de3a556c734p-19,  -0x1.ae64567f544e4p-26,
                               0x1.6124613a86d09p-33,  -0x1.ae7f3e733b81fp-41, 0x1.952c77030ad4ap-49,
                               -0x1.2f49b46814157p-57, 0x1.71b8ef6dcf572p-66,  -0x1.761b41316381ap-75,
                               0x1.3f3ccdd165fa9p-84,  -0x1.d1ab1c2dccea3p-94, 0x1.259f98b4358adp-103};
    constexpr double SL[7] = {0.0,
                              -0x1.5555555555555p-57,
                              0x1.1111111111111p-63,
                              -0x1.a01a01a01a01ap-73,
                              -0x1.c154f8ddc6c00p-73,
                              0x1.c062e06d1f209p-80,
                              0x1.f28e0cc748ebep-87};
    constexpr double CH[16] = {0x1.0000000000000p+0,   -0x1.0000000000000p-1,  0x1.5555555555555p-5,
                               -0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-16,  -0x1.27e4fb7789f5cp-22,
                               0x1.1eed8eff8d898p-29,  -0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-45,
                               -0x1.6827863b97d97p-53, 0x1.e542ba4020225p-62,  -0x1.0ce396db7f853p-70,
                               0x1.f2cf01972f578p-80,  -0x1.88e85fc6a4e5ap-89, 0x1.0a18a2635085dp-98,
                               -0x1.3932c5047d60ep-108};
    constexpr double CL[7] = {0.0,
                              0.0,
                              0x1.5555555555555p-59,
                              0x1.f49f49f49f49fp-65,
                              0x1.a01a01a01a01ap-76,
                              -0x1.cbbc05b4fa99ap-76,
                              -0x1.2aec959e14c06p-83};
    const double k = rint(__dmul_rn(x, kTwoOverPi));
    const double r = __fma_rn(-k, C1, x);  // k C1 exact and x - k C1 exact: one rounding-free operation
    DD y = dd_two_sum(r, -__dmul_rn(k, C2));
    const double p3 = __dmul_rn(k, C3);
    y = dd_add(y, {-p3, -__fma_rn(k, C3, -p3)});
    y = dd_add(y, {-__dmul_rn(k, C4), 0.0});
    const DD z = dd_mul(y, y);
    double qs = SH[14], qc = CH[15];
#pragma unroll
    for (int n = 13; n >= 7; --n)
        qs = __fma_rn(qs, z.hi, SH[n]);
#pragma unroll
    for (int n = 14; n >= 7; --n)
        qc = __fma_rn(qc, z.hi, CH[n]);
    DD s{qs, 0.0}, c{qc, 0.0};
#pragma unroll
    for (int n = 6; n >= 0; --n)
    {
        s = dd_add(dd_mul(s, z), {SH[n], SL[n]});
        c = dd_add(dd_mul(c, z), {CH[n], CL[n]});
    }
    s = dd_mul(s, y);
    const double sv = __dadd_rn(s.hi, s.lo), cv = __dadd_rn(c.hi, c.lo);
    const int q = (int)((long long)k & 3);
    *sn = q == 0 ? sv : (q == 1 ? cv : (q == 2 ? -sv : -cv));
    *cs = q == 0 ? cv : (q == 1 ? -sv : (q == 2 ? -cv : sv));
}

}  // namespace gbo
