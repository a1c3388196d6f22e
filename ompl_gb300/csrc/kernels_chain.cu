// Kinematic-chain kernels built on the warp-cooperative FP32 evaluator (chain_warp.cuh).
//
//   chain_validity_warp_kernel  StateValidityChecker::isValid, one warp per state
//   chain_motion_warp_kernel    DiscreteMotionValidator::checkMotion, persistent, one warp per edge
//                               taken from the device work queue; states j = 1..nd-1 then s2 in order
//                               (DiscreteMotionValidator.cpp:48-91), stopping at the first invalid one.
// Interpolated joints are formed in float-float from exact splits of s1 and s2:
//   q_i(t) = s1_i + D_i t, D_i the shortest-arc difference of KinematicChain.h:150-176 (the wrap by
//   2*pi that interpolate applies changes no sine or cosine), t = j / nd in float-float; the link
//   angles theta_k(t) = sum_{i<=k} q_i(t) = A_k + t S_k come from per-edge prefix sums A_k of s1 and
//   S_k of D, so a state needs no scan of its joints.
// Anything the FP32 error bounds leave undecided is settled with the FP64 reference-order code: an
// ambiguous segment test (chain_round64), an undecided segment count (chain_nd64_warp), and the states of
// an edge whose joint difference lies within 1e-9 of pi, where the interpolation's own branch is not
// settled in FP32 (motion_joint64). All FP64 work sits in small out-of-line functions: an inlined or
// large call inside the edge loop costs the loop registers, and local-memory spills, on every edge.
#include "chain_state.cuh"
#include "kernels.cuh"
#include "tma.cuh"

namespace gbo
{

// Dynamic shared memory of the warp kernels: the world's ChainSegF32 records (bytes32 = 32 * nw),
// then (dim + 1) link records per warp, then one test table per warp (one u32 per test).
struct ChainSmem
{
    ChainSegF32 *w32;
    const unsigned *tab;  // this warp's table
    int nw;               // world segments
    int lb;               // index of this warp's first link record in w32
    ChainTables t;
};

__device__ bool chain_setup(const SpaceParams &sp, const WorldArgs &wa, unsigned char *smem, uint64_t *bar,
                            RunCounters *ctr, ChainSmem &cs)
{
    if (!stage_bulk(smem, wa.data32, wa.bytes32, bar, &ctr->timeout, &ctr->error))
        return false;
    ChainSegF32 *w = (ChainSegF32 *)smem;
    const int per_warp = sp.dim + 1, n_link_recs = (int)(blockDim.x >> 5) * per_warp;
    init_chain_links(w + wa.n, n_link_recs, wa.guard);
    unsigned *tabs = (unsigned *)(w + wa.n + n_link_recs);
    build_chain_tables(sp.dim, wa.n, wa.test_order, tabs, (int)(blockDim.x >> 5), cs.t);
    if (threadIdx.x == 0)
    {
        chain_hz_pos = wa.hz_pos;
        chain_hz = &ctr->hazards;
    }
    __syncthreads();
    cs.w32 = w;
    cs.tab = tabs + (threadIdx.x >> 5) * cs.t.n_tests;
    cs.nw = wa.n;
    cs.lb = wa.n + (int)(threadIdx.x >> 5) * per_warp;
    return true;
}

__device__ __forceinline__ ff lane_joint(const StatesView &v, int64_t i, int lane, int dim)
{
    return lane < dim ? split_double(v(i, lane)) : ff{0.f, 0.f};
}

// Cold FP64 paths (reference operation order), kept out of line so that the FP32 kernels keep a small
// register footprint.

// StateSpace::validSegmentCount of one edge in FP64 (StateSpace.cpp:851-854), warp-collective: the
// chain metric of distance64 (demos/KinematicChain.h:105-121) with the cumulative angles and the
// sums in the reference's order (lane by lane through shuffles) and the sines and cosines one joint
// per lane.
__device__ __noinline__ int chain_nd64_warp(const SpaceParams &sp, const StatesView &v1, const StatesView &v2,
                                            int64_t e, int lane)
{
    const int n = sp.dim;
    const double qa = lane < n ? v1(e, lane) : 0.0, qb = lane < n ? v2(e, lane) : 0.0;
    double t1 = 0., t2 = 0., m1 = 0., m2 = 0.;
    for (int i = 0; i < n; ++i)
    {
        t1 = dadd(t1, __shfl_sync(0xffffffffu, qa, i));
        t2 = dadd(t2, __shfl_sync(0xffffffffu, qb, i));
        if (i == lane)
        {
            m1 = t1;
            m2 = t2;
        }
    }
    double s1 = 0., c1 = 1., s2 = 0., c2 = 1.;
    if (lane < n)
    {
        sincos(m1, &s1, &c1);
        sincos(m2, &s2, &c2);
    }
    double dx = 0., dy = 0., dist = 0.;
    for (int i = 0; i < n; ++i)
    {
        dx = dadd(dx, dsub(__shfl_sync(0xffffffffu, c1, i), __shfl_sync(0xffffffffu, c2, i)));
        dy = dadd(dy, dsub(__shfl_sync(0xffffffffu, s1, i), __shfl_sync(0xffffffffu, s2, i)));
        dist = dadd(dist, dsqrt(dadd(dmul(dx, dx), dmul(dy, dy))));
    }
    return segment_count_from_distance(sp, dmul(dist, sp.link));
}

// Joint `ln` of checked state j of edge e in FP64, as DiscreteMotionValidator.cpp:63 forms it (j == top
// is s2 itself). Out of line: inlined, the compiler hoists the loop-invariant FP64 division j / nd out
// of the rarely taken re-check branch and executes it for every checked state.
__device__ __noinline__ double motion_joint64(const StatesView &v1, const StatesView &v2, int64_t e, int ln, int j,
                                              int nd, int top)
{
    if (j == top)
        return v2(e, ln);
    return interp_angle64(v1(e, ln), v2(e, ln), ddiv((double)j, (double)nd));
}

__global__ void __launch_bounds__(256, 4) chain_validity_warp_kernel(const __grid_constant__ SpaceParams sp,
                                                                  const __grid_constant__ WorldArgs wa,
                                                                  const __grid_constant__ StatesView v, int64_t n,
                                                                  uint8_t *out, RunCounters *ctr)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    ChainSmem cs;
    if (!chain_setup(sp, wa, smem, &bar, ctr, cs))
        return;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float L = (float)sp.link;
    const double L64 = sp.link;
    const int dim = sp.dim;
    const double *w64 = (const double *)wa.data64;
    unsigned rechecks = 0, evaluated = 0;
    for (int64_t i = warp; i < n; i += nwarps)
    {
        ++evaluated;
        float vx, vy, px, py;
        chain_segments32(lane_joint(v, i, lane, dim), lane, dim, L, vx, vy, px, py);
        auto q64 = [&](int ln) { return ln < dim ? v(i, ln) : 0.0; };
        const int r = chain_state_warp32(lane, dim, L64, vx, vy, px, py, cs.w32, cs.nw, cs.lb, w64, cs.tab, cs.t, q64,
                                         rechecks);
        if (lane == 0)
            out[i] = r == kValid ? 1 : 0;
    }
    if (lane == 0)
    {
        if (evaluated)
            atomicAdd(&ctr->evaluated, (unsigned long long)evaluated);
        if (rechecks)
            atomicAdd(&ctr->rechecked, (unsigned long long)rechecks);
    }
}

__global__ void __launch_bounds__(256, 4) chain_motion_warp_kernel(const __grid_constant__ SpaceParams sp,
                                                                const __grid_constant__ WorldArgs wa,
                                                                const __grid_constant__ StatesView v1,
                                                                const __grid_constant__ StatesView v2, int64_t n,
                                                                uint8_t *ok, int32_t *first_j, int32_t *nd_out,
                                                                RunCounters *ctr)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    ChainSmem cs;
    if (!chain_setup(sp, wa, smem, &bar, ctr, cs))
        return;
    const int lane = threadIdx.x & 31;
    const int dim = sp.dim;
    const float L = (float)sp.link;
    const double L64 = sp.link;
    const double *w64 = (const double *)wa.data64;
    constexpr float kPiF = 3.14159265358979323846f;
    unsigned evaluated = 0, rechecks = 0;
    for (;;)
    {
        unsigned long long ei = 0;
        if (lane == 0)
            ei = atomicAdd(&ctr->queue, 1ull);
        const int64_t e = (int64_t)__shfl_sync(0xffffffffu, ei, 0);
        if (e >= n)
            break;
        const double a64 = lane < dim ? v1(e, lane) : 0.0, b64 = lane < dim ? v2(e, lane) : 0.0;
        const ff a = split_double(a64), b = split_double(b64);
        // shortest-arc difference per joint; an edge whose |difference| is within 1e-9 of pi, or with a
        // joint that is not finite, is decided with the FP64 interpolation (the reference's branch on
        // fabs(diff) <= pi is not settled here)
        ff diff = two_sum(b.hi, -a.hi);
        diff = fast_two_sum(diff.hi, diff.lo + (b.lo - a.lo));
        // |diff| - pi in float-float: adh - float(pi) is exact, float(pi) - pi = 8.742278e-08 (the
        // constant's own error is ~3e-15); the whole is good to ~1e-13, far inside the 1e-9 window
        const float adh = fabsf(diff.hi);
        const float over_pi = ((adh - kPiF) + (diff.hi < 0.f ? -diff.lo : diff.lo)) + 8.742278e-08f;
        const bool finite =
            ((__double2hiint(a64) & 0x7ff00000) != 0x7ff00000) && ((__double2hiint(b64) & 0x7ff00000) != 0x7ff00000);
        const bool near_pi = lane < dim && !(fabsf(over_pi) >= 1e-9f && finite);
        // an edge with a joint difference within 1e-9 of pi builds its states with the FP64 reference
        // interpolation (motion_joint64): the branch on fabs(diff) <= pi is not settled in FP32
        const bool exact = __any_sync(0xffffffffu, near_pi);
        ff D = diff;
        if (lane < dim && over_pi > 0.f)  // the reference wraps when fabs(diff) > pi
        {
            // D = diff - sign(diff) * 2*pi in float-float
            const float sgn = diff.hi > 0.f ? -1.f : 1.f;
            const ff t1 = two_sum(diff.hi, sgn * 6.28125f);
            const ff t2 = two_sum(t1.hi, sgn * (519505.0f / 268435456.0f));
            D = fast_two_sum(t2.hi, (t1.lo + t2.lo) + (diff.lo + sgn * 2.4308403e-10f));
        }
        // absolute link angles of s1 and s2 and the prefix sums of the joint differences: state t has
        // theta_k(t) = ta_k + t * DS_k (the sum over joints of a_i + D_i t)
        // s2's angles ta + DS differ from its own prefix sums by whole turns (the wraps of D), which
        // leave every sine and cosine unchanged
        const ff ta = warp_scan_ff(a, lane), DS = warp_scan_ff(D, lane);
        const ff tb = ff_add(ta, DS);
        int nd = chain_segment_count_warp(ta, tb, lane, dim, L, wa.inv_lvs32, wa.e_dist, sp.factor);
        const bool nd64 = nd < 0;
        if (nd64)  // segment count not decided by the FP32 distance bound: the reference's FP64 count
            nd = chain_nd64_warp(sp, v1, v2, e, lane);
        if (exact || nd64)
            ++rechecks;
        const int top = nd > 1 ? nd : 1;
        // 1/nd in float-float
        const float ndf = float_of(nd > 0 ? nd : 1);
        const float inv_hi = __frcp_rn(ndf);
        const float inv_lo = fmaf(-inv_hi, ndf, 1.0f) * inv_hi;
        float jf = 0.f;
        int first = -1;
        for (int j = 1; j <= top; ++j)
        {
            jf += 1.0f;
            ff th;  // absolute link angle of lane < dim (j == top and exact are the same in every lane)
            if (j == top)
                th = tb;
            else if (exact)
                th = warp_scan_ff(lane < dim ? split_double(motion_joint64(v1, v2, e, lane, j, nd, top)) : ff{0.f, 0.f},
                                  lane);
            else
            {
                const float t_hi = jf * inv_hi;
                const float t_lo = fmaf(jf, inv_hi, -t_hi) + jf * inv_lo;
                const float p_hi = DS.hi * t_hi;
                const float p_lo = fmaf(DS.hi, t_hi, -p_hi) + fmaf(DS.hi, t_lo, DS.lo * t_hi);
                th = ff_add(ta, {p_hi, p_lo});
            }
            float vx, vy, px, py;
            chain_segments32_theta(th, lane, dim, L, vx, vy, px, py);
            auto q64 = [&](int ln) { return ln < dim ? motion_joint64(v1, v2, e, ln, j, nd, top) : 0.0; };
            const int r = chain_state_warp32(lane, dim, L64, vx, vy, px, py, cs.w32, cs.nw, cs.lb, w64, cs.tab, cs.t, q64,
                                             rechecks);
            ++evaluated;
            if (r == kInvalid)
            {
                first = j == top ? nd : j;
                break;
            }
        }
        if (lane == 0)
        {
            ok[e] = first < 0 ? 1 : 0;
            if (first_j)
                first_j[e] = first;
            if (nd_out)
                nd_out[e] = nd;
        }
    }
    if (lane == 0)
    {
        if (evaluated)
            atomicAdd(&ctr->evaluated, (unsigned long long)evaluated);
        if (rechecks)
            atomicAdd(&ctr->rechecked, (unsigned long long)rechecks);
    }
}

// Hit bitmaps of n states (SoA FP64, ld = n) for the host's test ordering: one warp per state.
__global__ void __launch_bounds__(256) chain_hits_kernel(SpaceParams sp, WorldArgs wa, const double *states, int n,
                                                         unsigned *bits, int words)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    RunCounters *none = nullptr;
    (void)none;
    __shared__ unsigned timeout, error;
    if (threadIdx.x == 0)
        timeout = error = 0;
    __syncthreads();
    if (!stage_bulk(smem, wa.data32, wa.bytes32, &bar, &timeout, &error))
        return;
    const ChainSegF32 *w = (const ChainSegF32 *)smem;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    int n_self;
    const int n_tests = chain_test_count(sp.dim, wa.n, n_self);
    StatesView v{states, 1, (int64_t)n};
    for (int i = warp; i < n; i += nwarps)
    {
        float vx, vy, px, py;
        chain_segments32(lane_joint(v, i, lane, sp.dim), lane, sp.dim, (float)sp.link, vx, vy, px, py);
        chain_state_hits32(lane, vx, vy, px, py, w, sp.dim, wa.n, n_tests, wa.guard, bits + (size_t)i * words);
    }
}

void launch_chain_hits(cudaStream_t s, const SpaceParams &sp, const WorldArgs &wa, const double *states, int n,
                       unsigned *bits, int words)
{
    if (wa.bytes32 > 48 * 1024)
    {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        cudaFuncSetAttribute((const void *)chain_hits_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             optin - 1024);
    }
    chain_hits_kernel<<<64, 256, wa.bytes32, s>>>(sp, wa, states, n, bits, words);
    note_launch();
}

static unsigned chain_smem(const SpaceParams &sp, const WorldArgs &wa, int block)
{
    const int m = sp.dim + 1;
    const int n_tests = (m - 1) * (m - 2) / 2 + m * wa.n;
    return wa.bytes32 + (unsigned)((block / 32) * m * sizeof(ChainSegF32)) +
           (unsigned)((4 * (block / 32) * n_tests + 15) & ~15);
}

// The dynamic shared memory limit of a persistent kernel is raised to the opt-in maximum - 1 KB.
static bool chain_smem_fits(unsigned bytes)
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return (int64_t)bytes + 1024 <= (int64_t)optin;
}

// Block size of the warp kernels: 256 threads, or fewer warps per CTA when the per-warp test tables of
// a large world would not fit in shared memory (down to one warp, which needs what a single shared
// table did). Returns 0 when even that does not fit.
static int chain_block(const SpaceParams &sp, const WorldArgs &wa, unsigned &sm)
{
    for (int block = 256; block >= 32; block /= 2)
    {
        sm = chain_smem(sp, wa, block);
        if (chain_smem_fits(sm))
            return block;
    }
    return 0;
}

bool launch_chain_validity_warp(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v,
                                int64_t n, uint8_t *out, RunCounters *ctr)
{
    unsigned sm = 0;
    const int block = sp.dim > 31 || !wa.stage32 ? 0 : chain_block(sp, wa, sm);
    if (!block)
        return false;
    const int grid =
        persistent_grid((const void *)chain_validity_warp_kernel, block, sm, lc, (n * 32 + block - 1) / block);
    chain_validity_warp_kernel<<<grid, block, sm, lc.stream>>>(sp, wa, v, n, out, ctr);
    note_launch();
    return true;
}

bool launch_chain_motion_warp(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v1,
                              StatesView v2, int64_t n, uint8_t *ok, int32_t *fj, int32_t *nd, RunCounters *ctr)
{
    unsigned sm = 0;
    // link angles of interpolated states reach |theta| <= 2 dim pi, inside sincos_ff's range for dim <= 15
    const int block = sp.dim > 15 || !wa.stage32 ? 0 : chain_block(sp, wa, sm);
    if (!block)
        return false;
    const int grid =
        persistent_grid((const void *)chain_motion_warp_kernel, block, sm, lc, (n * 32 + block - 1) / block);
    chain_motion_warp_kernel<<<grid, block, sm, lc.stream>>>(sp, wa, v1, v2, n, ok, fj, nd, ctr);
    note_launch();
    return true;
}

}  // namespace gbo
