// sin and cos of a double, correctly rounded: the double nearest the exact value (except when that value
// lies within 2^-98 of a rounding midpoint, not met on any tested argument). A fast path (below) decides
// almost every argument; the double-double series described here decides the rest.
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

// Slow path: sin and cos of x as double-doubles from the full series (see above).
static __device__ __noinline__ void sincos_dd(double x, DD &sy, DD &cy)
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
#pragma unroll 1
    for (int n = 6; n >= 0; --n)
    {
        s = dd_add(dd_mul(s, z), {SH[n], SL[n]});
        c = dd_add(dd_mul(c, z), {CH[n], CL[n]});
    }
    sy = dd_mul(s, y);
    cy = c;
}

// Rounding test of Ziv's strategy: v = h + l (|l| <= ulp(h)/2) approximates the exact value within eb;
// true when every value within eb of v rounds to h (so h is the correctly rounded result).
__device__ __forceinline__ bool rounds_to(double h, double l, double eb)
{
    const unsigned long long b = (unsigned long long)__double_as_longlong(h) & 0x7fffffffffffffffull;
    const int e = (int)(b >> 52);
    if (e < 60 || e > 2040)
        return false;  // tiny, huge or special: the slow path decides
    const double ulp = __longlong_as_double((long long)(e - 52) << 52);
    const double above = 0.5 * ulp, below = (b & 0x000fffffffffffffull) ? 0.5 * ulp : 0.25 * ulp;
    const double r = h < 0.0 ? -l : l;  // residual toward larger magnitude
    return r + eb < above && r - eb > -below;
}

// sin and cos of x, correctly rounded. Fast path: the same reduction, then
//   sin y = y - y^3/6 + y^5 S(z),  cos y = 1 - z/2 + z^2/24 + z^3 C(z),  z = y^2,
// with the two leading corrections in double-double arithmetic and S, C (their series from the
// y^5 / z^3 terms on, truncated after y^21 / z^10, relative truncation < 1e-23) in plain FP64; the sum
// carries an error bound (2^-49 of the plain-FP64 tail, which covers its roundings and the truncation,
// plus 2^-98 of the result), and Ziv's rounding test accepts the nearest double when the bound cannot
// change it. Otherwise, and for |y| < 2^-26 or |x| >= 2^20, the double-double series decides.
static __device__ __noinline__ void sincos_cr(double x, double *sn, double *cs)
{
    constexpr double C1 = 0x1.921fb54400000p+0, C2 = 0x1.0b4611a600000p-34, C3 = 0x1.3198a2e037073p-69,
                     C4 = 0x1.129024e088a68p-123, kTwoOverPi = 0x1.45f306dc9c883p-1;
    constexpr double c6h = 0x1.5555555555555p-3, c6l = 0x1.5555555555555p-57;    // 1/6
    constexpr double c24h = 0x1.5555555555555p-5, c24l = 0x1.5555555555555p-59;  // 1/24
    constexpr double S[9] = {0x1.1111111111111p-7,  -0x1.a01a01a01a01ap-13, 0x1.71de3a556c734p-19,
                             -0x1.ae64567f544e4p-26, 0x1.6124613a86d09p-33,  -0x1.ae7f3e733b81fp-41,
                             0x1.952c77030ad4ap-49,  -0x1.2f49b46814157p-57, 0x1.71b8ef6dcf572p-66};
    constexpr double C[8] = {-0x1.6c16c16c16c17p-10, 0x1.a01a01a01a01ap-16, -0x1.27e4fb7789f5cp-22,
                             0x1.1eed8eff8d898p-29,  -0x1.93974a8c07c9dp-37, 0x1.ae7f3e733b81fp-45,
                             -0x1.6827863b97d97p-53, 0x1.e542ba4020225p-62};
    const double k = rint(__dmul_rn(x, kTwoOverPi));
    const int q = (int)((long long)k & 3);
    bool ok = fabs(x) < 0x1p20;
    double sv = 0.0, cv = 0.0;
    if (ok)
    {
        const double r = __fma_rn(-k, C1, x);
        DD y = dd_two_sum(r, -__dmul_rn(k, C2));
        const double p3 = __dmul_rn(k, C3);
        y = dd_add(y, {-p3, -__fma_rn(k, C3, -p3)});
        y = dd_add(y, {-__dmul_rn(k, C4), 0.0});
        const double yh = y.hi, yl = y.lo;
        ok = fabs(yh) >= 0x1p-26;
        // z = y^2 (double-double)
        const double zh = __dmul_rn(yh, yh);
        const double zl = __fma_rn(2.0 * yh, yl, __fma_rn(yh, yh, -zh));
        // sin: y - y^3/6 + y^5 S(z)
        const double ph = __dmul_rn(yh, zh);
        const double pl = __fma_rn(yh, zl, __fma_rn(yl, zh, __fma_rn(yh, zh, -ph)));  // y^3
        const double th = __dmul_rn(ph, c6h);
        const double tl = __fma_rn(ph, c6l, __fma_rn(pl, c6h, __fma_rn(ph, c6h, -th)));  // y^3 / 6
        double sp = S[8];
#pragma unroll
        for (int n = 7; n >= 0; --n)
            sp = __fma_rn(sp, zh, S[n]);
        const double w = __dmul_rn(__dmul_rn(ph, zh), sp);  // y^5 S(z)
        const DD a = dd_two_sum(yh, -th);
        const DD s = dd_fast_two_sum(a.hi, __dadd_rn(a.lo, __dadd_rn(__dsub_rn(yl, tl), w)));
        // cos: 1 - z/2 + z^2/24 + z^3 C(z)
        const double qh = __dmul_rn(zh, zh);
        const double ql = __fma_rn(2.0 * zh, zl, __fma_rn(zh, zh, -qh));  // z^2
        const double uh = __dmul_rn(qh, c24h);
        const double ul = __fma_rn(qh, c24l, __fma_rn(ql, c24h, __fma_rn(qh, c24h, -uh)));  // z^2 / 24
        double cp = C[7];
#pragma unroll
        for (int n = 6; n >= 0; --n)
            cp = __fma_rn(cp, zh, C[n]);
        const double w2 = __dmul_rn(__dmul_rn(qh, zh), cp);  // z^3 C(z)
        const DD b1 = dd_two_sum(1.0, -0.5 * zh);
        const DD b2 = dd_two_sum(b1.hi, uh);
        const DD c =
            dd_fast_two_sum(b2.hi, __dadd_rn(__dadd_rn(b2.lo, b1.lo), __dadd_rn(__dsub_rn(ul, 0.5 * zl), w2)));
        ok = ok && rounds_to(s.hi, s.lo, fabs(w) * 0x1p-49 + fabs(s.hi) * 0x1p-98) &&
             rounds_to(c.hi, c.lo, fabs(w2) * 0x1p-49 + fabs(c.hi) * 0x1p-98);
        sv = s.hi;
        cv = c.hi;
    }
    if (!ok)
    {
        DD s, c;
        sincos_dd(x, s, c);
        sv = __dadd_rn(s.hi, s.lo);
        cv = __dadd_rn(c.hi, c.lo);
    }
    *sn = q == 0 ? sv : (q == 1 ? cv : (q == 2 ? -sv : -cv));
    *cs = q == 0 ? cv : (q == 1 ? -sv : (q == 2 ? -cv : sv));
}

}  // namespace gbo
