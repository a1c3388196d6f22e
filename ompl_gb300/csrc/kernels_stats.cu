// Measurement kernels of the FP32-guarded forms (precision statistics) and the correctly rounded
// FP64 sin/cos entry point.
//
// precision_stats: for each state, the verdict of the FP32 arithmetic taken at face value (the
// reference's comparisons applied to the FP32 values, no guard band: what an FP32-only checker would
// answer), the guarded classification (definite or ambiguous: what the bulk path re-checks in FP64),
// and the reference's FP64 verdict. A flip is a state whose face-value FP32 verdict differs from the
// FP64 one; the flip rate is flips / states. The largest |FP32 - FP64| of the compared quantities is
// recorded as well: the denominators and numerators of the segment tests (kinematic chain), the
// squared-distance margins d^2 - (rs + ro)^2 of the sphere pairs (DH arm). The FP32 values are formed
// by the same device functions as the bulk kernels (chain_segments32 + the products of
// seg_intersect32; the FK of dh_valid32), so the statistics describe the arithmetic that runs.
#include "chain_state.cuh"
#include "kernels.cuh"

namespace gbo
{

struct PrecisionTally
{
    unsigned long long states, flips, ambiguous;
    unsigned int max_err_bits;  // float bits of the largest |FP32 - FP64| (non-negative floats order as ints)
};

__device__ __forceinline__ void tally_err(unsigned &mx, float e)
{
    const unsigned b = __float_as_uint(fabsf(e));
    mx = b > mx ? b : mx;
}

// The reference's segment test (demos/KinematicChain.h:251-276) on FP32 values taken at face value.
__device__ __forceinline__ bool seg_face32(float den, float sn, float tn)
{
    if (fabsf(den) < (float)kDblEps)
        return false;
    const bool P = den > 0.f;
    if ((sn < (float)kFltEps) == P || (tn < (float)kFltEps) == P)
        return false;
    if (((sn - den) > -(float)kFltEps) == P || ((tn - den) > (float)kFltEps) == P)
        return false;
    return true;
}

// One warp per state; tests in the default order, all evaluated (no early exit).
__global__ void __launch_bounds__(256) chain_precision_kernel(SpaceParams sp, WorldArgs wa, StatesView v, int64_t n,
                                                              PrecisionTally *out)
{
    const ChainSegF32 *w32 = (const ChainSegF32 *)wa.data32;
    const double *w64 = (const double *)wa.data64;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int dim = sp.dim, nw = wa.n;
    int n_self;
    const int n_tests = chain_test_count(dim, nw, n_self);
    unsigned long long st = 0, flips = 0, amb = 0;
    unsigned mx = 0;
    for (int64_t i = warp; i < n; i += nwarps)
    {
        float vx, vy, px, py;
        chain_segments32(lane < dim ? split_double(v(i, lane)) : ff{0.f, 0.f}, lane, dim, (float)sp.link, vx, vy, px,
                         py);
        double x0, y0, x1, y1;
        chain_segments64_warp(lane < dim ? v(i, lane) : 0.0, lane, dim, sp.link, x0, y0, x1, y1);
        bool face = false, hit64 = false, definite = false, ambiguous = false;
        for (int base = 0; base < n_tests; base += 32)
        {
            const int idx = base + lane;
            const unsigned e = idx < n_tests ? chain_test_entry(idx, dim, nw) : 0u;
            const int a = chain_test_a(e), b = chain_test_b(e) & 31;
            const bool link = (e & 0x80000000u) != 0u;
            const float ax = __shfl_sync(0xffffffffu, vx, a), ay = __shfl_sync(0xffffffffu, vy, a);
            const float apx = __shfl_sync(0xffffffffu, px, a), apy = __shfl_sync(0xffffffffu, py, a);
            const float bvx = __shfl_sync(0xffffffffu, vx, b), bvy = __shfl_sync(0xffffffffu, vy, b);
            const float bpx = __shfl_sync(0xffffffffu, px, b), bpy = __shfl_sync(0xffffffffu, py, b);
            const double ax0 = __shfl_sync(0xffffffffu, x0, a), ay0 = __shfl_sync(0xffffffffu, y0, a);
            const double ax1 = __shfl_sync(0xffffffffu, x1, a), ay1 = __shfl_sync(0xffffffffu, y1, a);
            const double lbx0 = __shfl_sync(0xffffffffu, x0, b), lby0 = __shfl_sync(0xffffffffu, y0, b);
            const double lbx1 = __shfl_sync(0xffffffffu, x1, b), lby1 = __shfl_sync(0xffffffffu, y1, b);
            if (idx < n_tests)
            {
                float s32x, s32y, s02x, s02y, lo, hi, eden;
                double bx0, by0, bx1, by1;
                if (link)
                {
                    s32x = bvx;
                    s32y = bvy;
                    s02x = apx - bpx;
                    s02y = apy - bpy;
                    lo = wa.guard.self_lo;
                    hi = wa.guard.self_hi;
                    eden = wa.guard.self_den;
                    bx0 = lbx0;
                    by0 = lby0;
                    bx1 = lbx1;
                    by1 = lby1;
                }
                else
                {
                    const ChainSegF32 ws = w32[chain_test_b(e)];
                    s32x = ws.sx;
                    s32y = ws.sy;
                    s02x = apx - ws.x0;
                    s02y = apy - ws.y0;
                    lo = ws.lo;
                    hi = ws.hi;
                    eden = ws.e_den;
                    const double *o = w64 + 4 * (size_t)chain_test_b(e);
                    bx0 = o[0];
                    by0 = o[1];
                    bx1 = o[2];
                    by1 = o[3];
                }
                const float den = fmaf(ax, s32y, -s32x * ay);
                const float sn = fmaf(ax, s02y, -ay * s02x);
                const float tn = fmaf(s32x, s02y, -s32y * s02x);
                face |= seg_face32(den, sn, tn);
                const int r = seg_intersect32(ax, ay, s32x, s32y, s02x, s02y, lo, hi, eden);
                definite |= r == kInvalid;
                ambiguous |= r == kAmbiguous;
                // the reference's quantities in FP64 (KinematicChain.h:255-266 operation order)
                const double s10_x = dsub(ax1, ax0), s10_y = dsub(ay1, ay0);
                const double s32_x = dsub(bx1, bx0), s32_y = dsub(by1, by0);
                const double d64 = dsub(dmul(s10_x, s32_y), dmul(s32_x, s10_y));
                const double s02_x = dsub(ax0, bx0), s02_y = dsub(ay0, by0);
                const double sn64 = dsub(dmul(s10_x, s02_y), dmul(s10_y, s02_x));
                const double tn64 = dsub(dmul(s32_x, s02_y), dmul(s32_y, s02_x));
                tally_err(mx, (float)((double)den - d64));
                tally_err(mx, (float)((double)sn - sn64));
                tally_err(mx, (float)((double)tn - tn64));
                hit64 |= seg_intersect64(ax0, ay0, ax1, ay1, bx0, by0, bx1, by1);
            }
        }
        face = __any_sync(0xffffffffu, face);
        hit64 = __any_sync(0xffffffffu, hit64);
        definite = __any_sync(0xffffffffu, definite);
        ambiguous = __any_sync(0xffffffffu, ambiguous);
        ++st;
        flips += face != hit64 ? 1 : 0;
        amb += (ambiguous && !definite) ? 1 : 0;
    }
    for (int o = 16; o > 0; o >>= 1)
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0 && st)
    {
        atomicAdd(&out->states, st);
        atomicAdd(&out->flips, flips);
        atomicAdd(&out->ambiguous, amb);
        atomicMax(&out->max_err_bits, mx);
    }
}

// One thread per state: the FP32 forward kinematics of dh_valid32 and the FP64 one of dh_valid64 in
// lockstep; every sphere pair listed in the FP64 centre's grid cell (a superset of the pairs within
// reach of either centre) is compared in both precisions.
__global__ void __launch_bounds__(128) dh_precision_kernel(SpaceParams sp, WorldArgs wa, StatesView v, int64_t n,
                                                           PrecisionTally *out)
{
    const DHArm &arm = wa.arm;
    const double *w64 = (const double *)wa.data64;
    const int G = wa.grid_n;
    const float rs = (float)arm.rs, E = wa.dh_e;
    const float inv_spl = 1.0f / (float)arm.spl;
    unsigned long long st = 0, flips = 0, amb = 0;
    unsigned mx = 0;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        float R[3][3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}}, p[3] = {0.f, 0.f, 0.f};
        double R6[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}}, p6[3] = {0, 0, 0};
        bool face = false, hit64 = false, definite = false, ambiguous = false;
        for (int j = 0; j < arm.joints; ++j)
        {
            const double q64 = v(i, j);
            const ff qs = split_double(q64);
            const float q = qs.hi + qs.lo;
            if (!(fabsf(q) <= wa.dh_qmax))
                ambiguous = true;
            float cq, sq;
            sincosf(q, &sq, &cq);
            const float ca = arm.ca[j], sa = arm.sa[j];
            const float A[3][3] = {{cq, -sq * ca, sq * sa}, {sq, cq * ca, -cq * sa}, {0.f, sa, ca}};
            const float pA[3] = {arm.af[j] * cq, arm.af[j] * sq, arm.dfl[j]};
            double cq6, sq6;
            sincos_cr(q64, &sq6, &cq6);
            const double ca6 = (double)arm.ca[j], sa6 = (double)arm.sa[j];
            const double A6[3][3] = {
                {cq6, dmul(-sq6, ca6), dmul(sq6, sa6)}, {sq6, dmul(cq6, ca6), dmul(-cq6, sa6)}, {0.0, sa6, ca6}};
            const double pA6[3] = {dmul(arm.a[j], cq6), dmul(arm.a[j], sq6), arm.d[j]};
            float Rn[3][3], pn[3];
            double Rn6[3][3], pn6[3];
            for (int r = 0; r < 3; ++r)
            {
                for (int k = 0; k < 3; ++k)
                {
                    Rn[r][k] = fmaf(R[r][2], A[2][k], fmaf(R[r][1], A[1][k], R[r][0] * A[0][k]));
                    Rn6[r][k] =
                        dadd(dadd(dmul(R6[r][0], A6[0][k]), dmul(R6[r][1], A6[1][k])), dmul(R6[r][2], A6[2][k]));
                }
                pn[r] = fmaf(R[r][2], pA[2], fmaf(R[r][1], pA[1], fmaf(R[r][0], pA[0], p[r])));
                pn6[r] = dadd(dadd(dadd(dmul(R6[r][0], pA6[0]), dmul(R6[r][1], pA6[1])), dmul(R6[r][2], pA6[2])), p6[r]);
            }
            for (int k = 0; k < arm.spl; ++k)
            {
                const float f = ((float)k + 0.5f) * inv_spl;
                const double f6 = ddiv(dadd((double)k, 0.5), (double)arm.spl);
                float c[3];
                double c6[3];
                int cell[3];
                bool inside = true;
                for (int r = 0; r < 3; ++r)
                {
                    c[r] = fmaf(f, pn[r] - p[r], p[r]);
                    c6[r] = dadd(p6[r], dmul(f6, dsub(pn6[r], p6[r])));
                    const double g = floor((c6[r] - wa.glo64[r]) * wa.ginv64[r]);
                    inside &= (g >= 0.0 && g < (double)G);
                    cell[r] = (int)g;
                }
                if (!inside)
                    continue;
                const int cid = (cell[0] * G + cell[1]) * G + cell[2];
                for (int it = wa.cell_start[cid]; it < wa.cell_start[cid + 1]; ++it)
                {
                    float t;
                    if (wa.boxes)
                    {
                        const float4 o = wa.cell_items4[2 * it], h = wa.cell_items4[2 * it + 1];
                        const float dx = fmaxf(fabsf(c[0] - o.x) - o.w, 0.f), dy = fmaxf(fabsf(c[1] - o.y) - h.x, 0.f);
                        const float dz = fmaxf(fabsf(c[2] - o.z) - h.y, 0.f);
                        t = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) - rs * rs;
                    }
                    else
                    {
                        const float4 o = wa.cell_items4[it];
                        const float dx = c[0] - o.x, dy = c[1] - o.y, dz = c[2] - o.z;
                        const float rr = rs + o.w;
                        t = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) - rr * rr;
                    }
                    face |= t < 0.f;
                    definite |= t < -E;
                    ambiguous |= (t >= -E && t <= E);
                    const double *o6 = w64 + (wa.boxes ? 6 : 4) * wa.cell_items[it];
                    double ex, ey, ez, rr6;
                    if (wa.boxes)
                    {
                        ex = fmax(dsub(fabs(dsub(c6[0], o6[0])), o6[3]), 0.0);
                        ey = fmax(dsub(fabs(dsub(c6[1], o6[1])), o6[4]), 0.0);
                        ez = fmax(dsub(fabs(dsub(c6[2], o6[2])), o6[5]), 0.0);
                        rr6 = arm.rs;
                    }
                    else
                    {
                        ex = dsub(c6[0], o6[0]);
                        ey = dsub(c6[1], o6[1]);
                        ez = dsub(c6[2], o6[2]);
                        rr6 = dadd(arm.rs, o6[3]);
                    }
                    const double t6 = dadd(dadd(dmul(ex, ex), dmul(ey, ey)), dmul(ez, ez)), r2 = dmul(rr6, rr6);
                    hit64 |= t6 < r2;
                    tally_err(mx, (float)((double)t - (t6 - r2)));
                }
            }
            for (int r = 0; r < 3; ++r)
            {
                p[r] = pn[r];
                p6[r] = pn6[r];
                for (int k = 0; k < 3; ++k)
                {
                    R[r][k] = Rn[r][k];
                    R6[r][k] = Rn6[r][k];
                }
            }
        }
        ++st;
        flips += face != hit64 ? 1 : 0;
        amb += (ambiguous && !definite) ? 1 : 0;
    }
    if (st)
    {
        atomicAdd(&out->states, st);
        atomicAdd(&out->flips, flips);
        atomicAdd(&out->ambiguous, amb);
        atomicMax(&out->max_err_bits, mx);
    }
}

bool launch_precision_stats(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v, int64_t n,
                            void *tally)
{
    PrecisionTally *t = (PrecisionTally *)tally;
    if (wa.kind == GBO_CHECK_CHAIN_SEGMENTS && sp.dim <= 31)
    {
        const int grid = (int)std::min<int64_t>((n * 32 + 255) / 256, (int64_t)lc.sm_count * 8);
        chain_precision_kernel<<<grid, 256, 0, lc.stream>>>(sp, wa, v, n, t);
    }
    else if (wa.kind == GBO_CHECK_DH_SPHERES && wa.arm.joints <= 8)
    {
        const int grid = (int)std::min<int64_t>((n + 127) / 128, (int64_t)lc.sm_count * 16);
        dh_precision_kernel<<<grid, 128, 0, lc.stream>>>(sp, wa, v, n, t);
    }
    else
        return false;
    note_launch();
    return true;
}

__global__ void sincos_cr_kernel(const double *x, int64_t n, double *s, double *c)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
        sincos_cr(x[i], s + i, c + i);
}

void launch_sincos_cr(const LaunchCfg &lc, const double *x, int64_t n, double *s, double *c)
{
    if (n == 0)
        return;
    sincos_cr_kernel<<<(int)((n + 255) / 256), 256, 0, lc.stream>>>(x, n, s, c);
    note_launch();
}

}  // namespace gbo
