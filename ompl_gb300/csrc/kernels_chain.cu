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
// ambiguous segment test (chain_resolve64), an undecided segment count (chain_nd64), and the states of
// an edge whose joint difference lies within 1e-9 of pi, where the interpolation's own branch is not
// settled in FP32 (motion_joint64). All FP64 work sits in small out-of-line functions: an inlined or
// large call inside the edge loop costs the loop registers, and local-memory spills, on every edge.
#include "chain_round.cuh"
#include "kernels.cuh"
#include "tma.cuh"

namespace gbo
{

// Dynamic shared memory of the warp kernels (16-byte aligned parts): the world's segment pairs plus a
// null pair (48 bytes each), then per warp the link records (32 bytes per segment) and link-pair
// records (48 bytes each, m - 1 of them incl. the null record), then the self table (one u32 per lane
// of each self round) and the unit order (u16).
struct ChainLayout
{
    unsigned wpair, lb, lp, self_tab, units, total;
};

__host__ __device__ inline ChainLayout chain_layout(int m, int n_pairs, int warps, int n_self_units, int n_units)
{
    ChainLayout L;
    L.wpair = 0;
    L.lb = L.wpair + 48u * (unsigned)(n_pairs + 1);
    L.lp = L.lb + 32u * (unsigned)(warps * m);
    L.self_tab = L.lp + 48u * (unsigned)(warps * (m - 1));
    L.units = L.self_tab + 128u * (unsigned)n_self_units;
    L.total = (L.units + 2u * (unsigned)n_units + 15u) & ~15u;
    return L;
}

// Entry `i` of the self table of a chain with m segments: the pair-tests (a, r) with partners
// b = a + 2, a + 4, ... (r = b - 2), a-major; entries past the end point at the null record m - 2.
__device__ __forceinline__ unsigned chain_self_entry(int i, int m)
{
    int k = i;
    for (int a = 0; a + 2 < m; ++a)
    {
        const int cnt = (m - a - 1) / 2;  // partners a + 2 .. m - 1 in pairs
        if (k < cnt)
            return (unsigned)a | ((unsigned)(a + 2 * k) << 8);  // r = b - 2 = a + 2k
        k -= cnt;
    }
    return (unsigned)(m - 2) << 8;  // null record, link 0
}

__device__ bool chain_setup(const SpaceParams &sp, const WorldArgs &wa, uint64_t *bar, RunCounters *ctr,
                            ChainWarp &cw)
{
    unsigned char *smem = chain_smem;
    const int m = sp.dim + 1, warps = (int)(blockDim.x >> 5), warp = (int)(threadIdx.x >> 5);
    const ChainLayout L = chain_layout(m, wa.n_pairs, warps, wa.n_self_units, wa.n_units);
    if (threadIdx.x == 0)
    {
        chain_hz_pos = wa.hz_pos;
        chain_hz = &ctr->hazards;
    }
    if (!stage_bulk(smem + L.wpair, wa.wpair, 48u * (unsigned)(wa.n_pairs + 1), bar, &ctr->timeout, &ctr->error))
        return false;
    // link-pair records: bounds (written once) and the null record
    const ChainGuard &g = wa.guard;
    for (int k = threadIdx.x; k < warps * (m - 1); k += blockDim.x)
    {
        const int r = k % (m - 1);
        ulonglong2 *rec = (ulonglong2 *)(smem + L.lp) + 3 * k;
        const bool null_rec = r == m - 2, tip = r == m - 3;
        if (null_rec)
        {
            rec[0] = make_ulonglong2(f2_pack(kNullCoord, kNullCoord), f2_pack(kNullCoord, kNullCoord));
            rec[1] = make_ulonglong2(0ull, 0ull);
        }
        rec[2] = make_ulonglong2(f2_pack(null_rec ? kNullE : g.self_e, (null_rec || tip) ? kNullE : g.self_e),
                                 f2_pack(null_rec ? -1.f : g.self_den, (null_rec || tip) ? -1.f : g.self_den));
    }
    unsigned *tab = (unsigned *)(smem + L.self_tab);
    for (int k = threadIdx.x; k < 32 * wa.n_self_units; k += blockDim.x)
        tab[k] = chain_self_entry(k, m);
    unsigned short *units = (unsigned short *)(smem + L.units);
    for (int k = threadIdx.x; k < wa.n_units; k += blockDim.x)
        units[k] = wa.units[k];
    __syncthreads();
    cw.lb = L.lb + 32u * (unsigned)(warp * m);
    cw.lp = L.lp + 48u * (unsigned)(warp * (m - 1));
    cw.self_tab = L.self_tab;
    cw.units = L.units;
    cw.m = m;
    cw.R = (m + 1) / 2;
    return true;
}

__device__ __forceinline__ ff lane_joint(const StatesView &v, int64_t i, int lane, int dim)
{
    return lane < dim ? split_double(v(i, lane)) : ff{0.f, 0.f};
}

// Cold FP64 paths (reference operation order), one thread, kept out of line so that the FP32
// kernels keep a small register footprint.
__device__ __noinline__ void load_pair64(const StatesView &v1, const StatesView &v2, int64_t e, int dim, double *a,
                                         double *b)
{
    for (int d = 0; d < GBO_MAXD; ++d)
    {
        a[d] = d < dim ? v1(e, d) : 0.0;
        b[d] = d < dim ? v2(e, d) : 0.0;
    }
}

// StateSpace::validSegmentCount of one edge in FP64 (StateSpace.cpp:851-854).
__device__ __noinline__ int chain_nd64(const SpaceParams &sp, const StatesView &v1, const StatesView &v2, int64_t e)
{
    double a[GBO_MAXD], b[GBO_MAXD];
    load_pair64(v1, v2, e, sp.dim, a, b);
    return segment_count_from_distance(sp, distance64<GBO_MAXD>(sp, a, b));
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

// The lane's world pair of chunk 0 (registers), reloaded by chain_state_test for other chunks.
__device__ __forceinline__ SegPair first_pair(const WorldArgs &wa, int lane)
{
    const int p = lane & 15;
    return load_seg_pair(chain_rec(0) + 3 * (p < wa.n_pairs ? p : wa.n_pairs));
}

// Marker of a deferred edge or state in the ok / validity output between the two passes.
constexpr uint8_t kDeferred = 2;

// StateValidityChecker::isValid, one warp per state. Pass 1 (RESOLVE false) answers every state whose
// rounds are decided in FP32 and marks the others kDeferred; pass 2 (RESOLVE true) scans the output
// for the marks and answers those states with the FP64 re-check of their ambiguous tests.
template <bool RESOLVE>
__global__ void __launch_bounds__(256, 4) chain_validity_warp_kernel(const __grid_constant__ SpaceParams sp,
                                                                  const __grid_constant__ WorldArgs wa,
                                                                  const __grid_constant__ StatesView v, int64_t n,
                                                                  uint8_t *out, RunCounters *ctr)
{
    __shared__ uint64_t bar;
    ChainWarp cw;
    if (!chain_setup(sp, wa, &bar, ctr, cw))
        return;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const float L = (float)sp.link;
    const double L64 = sp.link;
    const int dim = sp.dim;
    SegPair mine = first_pair(wa, lane);
    int chunk = 0;
    unsigned rechecks = 0, evaluated = 0;
    auto one = [&](int64_t i) {
        float vx, vy, px, py;
        chain_segments32(lane_joint(v, i, lane, dim), lane, dim, L, vx, vy, px, py);
        write_link_records(cw, lane, vx, vy, px, py);
        auto q64 = [&](int ln) { return ln < dim ? v(i, ln) : 0.0; };
        return chain_state_test<RESOLVE>(cw, wa, lane, dim, L64, mine, chunk, q64, rechecks);
    };
    if constexpr (!RESOLVE)
    {
        for (int64_t i = warp; i < n; i += nwarps)
        {
            ++evaluated;
            const int r = one(i);
            if (lane == 0)
                out[i] = r == kValid ? 1 : (r == kInvalid ? 0 : kDeferred);
        }
    }
    else
    {
        for (int64_t base = warp * 32; base < n; base += nwarps * 32)
        {
            const int64_t i = base + lane;
            unsigned todo = __ballot_sync(0xffffffffu, i < n && out[i] == kDeferred);
            while (todo)
            {
                const int src = __ffs(todo) - 1;
                todo &= todo - 1;
                const int r = one(base + src);
                if (lane == 0)
                    out[base + src] = r == kValid ? 1 : 0;
            }
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

// DiscreteMotionValidator::checkMotion, one warp per edge. Pass 1 (RESOLVE false, persistent, edges from
// the device work queue) answers every edge whose segment count and states are decided in FP32 and
// marks the others kDeferred in ok (an undecided segment count, a joint difference within 1e-9 of pi or
// not finite, or a state with an ambiguous round and no definite collision); pass 2 (RESOLVE true)
// scans ok for the marks and checks those edges from their first state with the FP64 pieces.
template <bool RESOLVE>
__global__ void __launch_bounds__(256, 4) chain_motion_warp_kernel(const __grid_constant__ SpaceParams sp,
                                                                const __grid_constant__ WorldArgs wa,
                                                                const __grid_constant__ StatesView v1,
                                                                const __grid_constant__ StatesView v2, int64_t n,
                                                                uint8_t *ok, int32_t *first_j, int32_t *nd_out,
                                                                RunCounters *ctr)
{
    __shared__ uint64_t bar;
    ChainWarp cw;
    if (!chain_setup(sp, wa, &bar, ctr, cw))
        return;
    const int lane = threadIdx.x & 31;
    const int dim = sp.dim;
    const float L = (float)sp.link;
    const double L64 = sp.link;
    constexpr float kPiF = 3.14159265358979323846f;
    SegPair mine = first_pair(wa, lane);
    int chunk = 0;
    unsigned evaluated = 0, rechecks = 0;
    // one edge: returns false when pass 1 defers it (ok[e] = kDeferred)
    auto edge = [&](int64_t e) {
        const double a64 = lane < dim ? v1(e, lane) : 0.0, b64 = lane < dim ? v2(e, lane) : 0.0;
        const ff a = split_double(a64), b = split_double(b64);
        // shortest-arc difference per joint; an edge whose |difference| is within 1e-9 of pi (or with a
        // joint that is not finite) is decided with the FP64 interpolation (the reference's branch on
        // fabs(diff) <= pi is not settled here)
        ff diff = two_sum(b.hi, -a.hi);
        diff = fast_two_sum(diff.hi, diff.lo + (b.lo - a.lo));
        // |diff| - pi in float-float: adh - float(pi) is exact, float(pi) - pi = 8.742278e-08 (the
        // constant's own error is ~3e-15); the whole is good to ~1e-13, far inside the 1e-9 window
        const float adh = fabsf(diff.hi);
        const float over_pi = ((adh - kPiF) + (diff.hi < 0.f ? -diff.lo : diff.lo)) + 8.742278e-08f;
        const bool near_pi = lane < dim && !(fabsf(over_pi) >= 1e-9f && fabs(a64) <= 1e30 && fabs(b64) <= 1e30);
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
        // absolute link angles of s1 and the prefix sums of the joint differences: state t has
        // theta_k(t) = ta_k + t * DS_k; s2's angles ta_k + DS_k differ from its own prefix sums by
        // whole turns (the wraps of D), which leave every sine and cosine unchanged
        const ff ta = warp_scan_ff16(a, lane, dim), DS = warp_scan_ff16(D, lane, dim);
        int nd = chain_segment_count_warp(ta, ff_add(ta, DS), lane, dim, L, wa.inv_lvs32, wa.e_dist, sp.factor);
        const bool nd64 = nd < 0;
        if constexpr (!RESOLVE)
        {
            if (exact || nd64)
                return false;
        }
        else
        {
            if (nd64)
            {
                // segment count not decided by the FP32 distance bound: the reference's FP64 count
                if (lane == 0)
                    nd = chain_nd64(sp, v1, v2, e);
                nd = __shfl_sync(0xffffffffu, nd, 0);
            }
            if (exact || nd64)
                ++rechecks;
        }
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
            ff th;  // absolute link angle of lane < dim
            if (RESOLVE && exact)
                th = warp_scan_ff16(lane < dim ? split_double(motion_joint64(v1, v2, e, lane, j, nd, top))
                                               : ff{0.f, 0.f},
                                    lane, dim);
            else if (j == top)
                th = ff_add(ta, DS);
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
            write_link_records(cw, lane, vx, vy, px, py);
            auto q64 = [&](int ln) { return ln < dim ? motion_joint64(v1, v2, e, ln, j, nd, top) : 0.0; };
            const int r = chain_state_test<RESOLVE>(cw, wa, lane, dim, L64, mine, chunk, q64, rechecks);
            ++evaluated;
            if (!RESOLVE && r == kAmbiguous)
                return false;
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
        return true;
    };
    if constexpr (!RESOLVE)
    {
        for (;;)
        {
            unsigned long long ei = 0;
            if (lane == 0)
                ei = atomicAdd(&ctr->queue, 1ull);
            const int64_t e = (int64_t)__shfl_sync(0xffffffffu, ei, 0);
            if (e >= n)
                break;
            if (!edge(e) && lane == 0)
                ok[e] = kDeferred;
        }
    }
    else
    {
        const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
        const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
        for (int64_t base = warp * 32; base < n; base += nwarps * 32)
        {
            const int64_t i = base + lane;
            unsigned todo = __ballot_sync(0xffffffffu, i < n && ok[i] == kDeferred);
            while (todo)
            {
                const int src = __ffs(todo) - 1;
                todo &= todo - 1;
                edge(base + src);
            }
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

// The dynamic shared memory limit of a persistent kernel is raised to the opt-in maximum - 1 KB.
static bool chain_smem_fits(unsigned bytes)
{
    int dev = 0, optin = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    return (int64_t)bytes + 1024 <= (int64_t)optin;
}

// Block size of the warp kernels: 256 threads, or fewer warps per CTA when a large world's pairs and
// the per-warp records would not fit in shared memory. Returns 0 when even one warp does not fit.
static int chain_block(const SpaceParams &sp, const WorldArgs &wa, unsigned &sm)
{
    if (!wa.wpair || wa.n_units <= 0)
        return 0;
    for (int block = 256; block >= 32; block /= 2)
    {
        sm = chain_layout(sp.dim + 1, wa.n_pairs, block / 32, wa.n_self_units, wa.n_units).total;
        if (chain_smem_fits(sm))
            return block;
    }
    return 0;
}

// The resolving pass runs on a smaller grid (it scans the marks and handles the few deferred items).
static int chain_resolve_grid(const void *kernel, int block, unsigned sm, const LaunchCfg &lc, int64_t n)
{
    const int64_t want = std::max<int64_t>(1, std::min<int64_t>((n + 1023) / 1024, 2 * (int64_t)lc.sm_count));
    return persistent_grid(kernel, block, sm, lc, want);
}

bool launch_chain_validity_warp(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v,
                                int64_t n, uint8_t *out, RunCounters *ctr)
{
    unsigned sm = 0;
    const int block = sp.dim > 31 ? 0 : chain_block(sp, wa, sm);
    if (!block)
        return false;
    const int grid =
        persistent_grid((const void *)chain_validity_warp_kernel<false>, block, sm, lc, (n * 32 + block - 1) / block);
    chain_validity_warp_kernel<false><<<grid, block, sm, lc.stream>>>(sp, wa, v, n, out, ctr);
    note_launch();
    const int g2 = chain_resolve_grid((const void *)chain_validity_warp_kernel<true>, block, sm, lc, n);
    chain_validity_warp_kernel<true><<<g2, block, sm, lc.stream>>>(sp, wa, v, n, out, ctr);
    note_launch();
    return true;
}

bool launch_chain_motion_warp(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v1,
                              StatesView v2, int64_t n, uint8_t *ok, int32_t *fj, int32_t *nd, RunCounters *ctr)
{
    unsigned sm = 0;
    // link angles of interpolated states reach |theta| <= 2 dim pi, inside sincos_ff's range for dim <= 15
    const int block = sp.dim > 15 ? 0 : chain_block(sp, wa, sm);
    if (!block)
        return false;
    const int grid =
        persistent_grid((const void *)chain_motion_warp_kernel<false>, block, sm, lc, (n * 32 + block - 1) / block);
    chain_motion_warp_kernel<false><<<grid, block, sm, lc.stream>>>(sp, wa, v1, v2, n, ok, fj, nd, ctr);
    note_launch();
    const int g2 = chain_resolve_grid((const void *)chain_motion_warp_kernel<true>, block, sm, lc, n);
    chain_motion_warp_kernel<true><<<g2, block, sm, lc.stream>>>(sp, wa, v1, v2, n, ok, fj, nd, ctr);
    note_launch();
    return true;
}

}  // namespace gbo
