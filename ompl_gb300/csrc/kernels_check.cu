// Validity and discrete-motion kernels.
//
//   validity_kernel      StateValidityChecker::isValid over a batch (thread per state)
//   motion_plain_kernel  DiscreteMotionValidator::checkMotion, one warp per edge: lanes take 32
//                        consecutive checked states, __ballot_sync picks the first invalid one and the
//                        warp stops at the first chunk that holds one (FP64, the drop-in form)
//   motion_tile_kernel   persistent: a warp takes 32 edges from the device work queue, computes their
//                        segment counts lane-parallel, then re-spreads its 32 lanes over the edges still
//                        alive (one lane per edge while all live, more lanes per edge as edges finish)
//   motion_warp_kernel   persistent: one edge per warp from the work queue, 32 steps per ballot
//
// The checked states and the reported first invalid index follow DiscreteMotionValidator.cpp:48-91:
// states j/nd for j = 1..nd-1 in order, then s2 itself (index nd); nd = validSegmentCount(s1, s2).
#include <algorithm>

#include "kernels.cuh"
#include "tma.cuh"

namespace gbo
{

// Checked state j of an edge in a RealVectorStateSpace (interpolate, RealVectorStateSpace.cpp:257-265)
// as FP32 values, computed in float-float with no FP64 instruction: within ~1e-13 of the reference's
// FP64 state before the final rounding, i.e. within u|q| + 1e-13 of it, which the FP32 guard bounds
// cover. j == top is s2 itself.
template <int MAXD>
__device__ __forceinline__ void state_at_rv32(const double *a, const double *b, int dim, int j, int nd, int top,
                                              float *q)
{
    if (j == top)
    {
#pragma unroll
        for (int d = 0; d < MAXD; ++d)
            if (d < dim)
            {
                const ff v = split_double(b[d]);
                q[d] = v.hi + v.lo;
            }
        return;
    }
    const float ndf = float_of(nd);
    const float inv_hi = __frcp_rn(ndf);
    const float inv_lo = fmaf(-inv_hi, ndf, 1.0f) * inv_hi;
    const float jf = float_of(j);
    const float t_hi = jf * inv_hi;
    const float t_lo = fmaf(jf, inv_hi, -t_hi) + jf * inv_lo;
#pragma unroll
    for (int d = 0; d < MAXD; ++d)
        if (d < dim)
        {
            const ff A = split_double(a[d]), Bv = split_double(b[d]);
            ff D = two_sum(Bv.hi, -A.hi);
            D = fast_two_sum(D.hi, D.lo + (Bv.lo - A.lo));
            const float p_hi = D.hi * t_hi;
            const float p_lo = fmaf(D.hi, t_hi, -p_hi) + fmaf(D.hi, t_lo, D.lo * t_hi);
            const ff r = ff_add(A, ff{p_hi, p_lo});
            q[d] = r.hi + r.lo;
        }
}

template <int MAXD>
__device__ __forceinline__ void state_at(const SpaceParams &sp, const double *a, const double *b, int j, int nd,
                                         int top, double *q)
{
    if (j == top)
    {
#pragma unroll
        for (int d = 0; d < MAXD; ++d)
            q[d] = b[d];
    }
    else
        interpolate64<MAXD>(sp, a, b, ddiv((double)j, (double)nd), q);
}

template <int CK, int MAXD>
struct Eval
{
    const double *w64 = nullptr;
    const ChainSegF32 *w32 = nullptr;
    const DHArm *arm = nullptr;
    const float4 *sph32 = nullptr;
    int nw = 0;
    ChainGuard g{};
    const WorldArgs *wa = nullptr;
    unsigned long long *hz = nullptr;  // hazard counter of the launch (RunCounters::hazards)

    __device__ bool valid64(const SpaceParams &s, const double *q) const
    {
        if constexpr (CK == GBO_CHECK_CIRCLES)
            return circles_valid64(w64, nw, q[0], q[1]);
        else if constexpr (CK == GBO_CHECK_CHAIN_SEGMENTS)
            return chain_valid64<MAXD>(s, q, w64, nw, wa->hz_pos, hz);
        else if constexpr (CK == GBO_CHECK_DH_SPHERES)
            return dh_valid64<MAXD>(*arm, q, w64, *wa, hz);
        else
            return true;
    }
    // 0 invalid, 1 valid, 2 ambiguous
    __device__ int valid32(const SpaceParams &s, const double *q) const
    {
        if constexpr (CK == GBO_CHECK_CHAIN_SEGMENTS)
            return chain_valid32<MAXD>(s, q, w32, nw, g);
        else if constexpr (CK == GBO_CHECK_DH_SPHERES)
        {
            float qf[MAXD];
#pragma unroll
            for (int d = 0; d < MAXD; ++d)
                qf[d] = d < s.dim ? split_double(q[d]).hi + split_double(q[d]).lo : 0.f;
            return dh_valid32<MAXD>(*arm, qf, sph32, *wa);
        }
        else
            return valid64(s, q) ? kValid : kInvalid;
    }
    // Verdict on checked state j of the edge (a, b) (j == top is b). The DH arm in a RealVectorStateSpace
    // evaluates the FP32 form on float-float interpolated angles and may return kAmbiguous: the caller
    // resolves those lanes warp-cooperatively (dh_resolve_warp). The other forms return kValid or
    // kInvalid, re-checked per lane.
    template <int PREC>
    __device__ int eval_at(const SpaceParams &s, const double *a, const double *b, int j, int nd, int top,
                           unsigned &rechecks) const
    {
        if constexpr (PREC == GBO_PRECISION_FP32_GUARDED && CK == GBO_CHECK_DH_SPHERES)
        {
            if (s.kind == GBO_SPACE_REAL_VECTOR)
            {
                float qf[MAXD];
                state_at_rv32<MAXD>(a, b, s.dim, j, nd, top, qf);
                return dh_valid32<MAXD>(*arm, qf, sph32, *wa);
            }
        }
        double q[MAXD];
        state_at<MAXD>(s, a, b, j, nd, top, q);
        return valid<PREC>(s, q, rechecks) ? kValid : kInvalid;
    }
    template <int PREC>
    __device__ bool valid(const SpaceParams &s, const double *q, unsigned &rechecks) const
    {
        if constexpr (PREC == GBO_PRECISION_FP64)
            return valid64(s, q);
        else
        {
            int r = valid32(s, q);
            if (r == kAmbiguous)
            {
                ++rechecks;
                return valid64(s, q);
            }
            return r == kValid;
        }
    }
};

// Stage the world into dynamic shared memory and build the evaluator over it.
template <int CK, int MAXD, int PREC>
__device__ bool setup_world(const WorldArgs &wa, unsigned char *smem, uint64_t *bar, RunCounters *ctr,
                            Eval<CK, MAXD> &ev)
{
    ev.nw = wa.n;
    ev.g = wa.guard;
    ev.wa = &wa;
    ev.arm = &wa.arm;
    ev.hz = ctr ? &ctr->hazards : nullptr;
    unsigned char *p = smem;
    if (PREC == GBO_PRECISION_FP32_GUARDED && (CK == GBO_CHECK_CHAIN_SEGMENTS || CK == GBO_CHECK_DH_SPHERES))
    {
        if (wa.stage32)
        {
            if (!stage_bulk(p, wa.data32, wa.bytes32, bar, &ctr->timeout, &ctr->error))
                return false;
            ev.w32 = (const ChainSegF32 *)p;
            ev.sph32 = (const float4 *)p;
        }
        else
        {
            // too large for shared memory: read from global memory (L2 / L1)
            ev.w32 = (const ChainSegF32 *)wa.data32;
            ev.sph32 = (const float4 *)wa.data32;
        }
        ev.w64 = (const double *)wa.data64;  // FP64 re-checks read the world from global memory (L2)
    }
    else if (wa.stage64)
    {
        if (!stage_bulk(p, wa.data64, wa.bytes64, bar, &ctr->timeout, &ctr->error))
            return false;
        ev.w64 = (const double *)p;
    }
    else
        ev.w64 = (const double *)wa.data64;
    return true;
}

template <int MAXD>
__device__ __forceinline__ void load_state(const StatesView &v, int64_t i, int dim, double *q)
{
#pragma unroll
    for (int d = 0; d < MAXD; ++d)
        q[d] = d < dim ? v(i, d) : 0.0;
}

__device__ __forceinline__ void flush_counts(RunCounters *ctr, unsigned evaluated, unsigned rechecks)
{
    // warp-aggregated counters
    unsigned e = evaluated, r = rechecks;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        e += __shfl_xor_sync(0xffffffffu, e, o);
        r += __shfl_xor_sync(0xffffffffu, r, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        if (e)
            atomicAdd(&ctr->evaluated, (unsigned long long)e);
        if (r)
            atomicAdd(&ctr->rechecked, (unsigned long long)r);
    }
}

template <int CK, int MAXD, int PREC>
__global__ void __launch_bounds__(256) validity_kernel(SpaceParams sp, WorldArgs wa, StatesView v, int64_t n,
                                                       uint8_t *out, RunCounters *ctr)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    Eval<CK, MAXD> ev;
    if (!setup_world<CK, MAXD, PREC>(wa, smem, &bar, ctr, ev))
        return;
    unsigned evaluated = 0, rechecks = 0;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    for (int64_t base = (int64_t)blockIdx.x * blockDim.x; base < n; base += stride)
    {
        int64_t i = base + threadIdx.x;
        if (i < n)
        {
            double q[MAXD];
            load_state<MAXD>(v, i, sp.dim, q);
            out[i] = ev.template valid<PREC>(sp, q, rechecks) ? 1 : 0;
            ++evaluated;
        }
    }
    flush_counts(ctr, evaluated, rechecks);
}

// Segment count nd of an edge. FP64: the reference expression. FP32_GUARDED (kinematic chain): the
// workspace metric in FP32 with bound e_dist; when ceil(distance / lvs) is not decided by the
// interval [d - e, d + e] the FP64 expression decides.
template <int MAXD, int PREC>
__device__ int segment_count(const SpaceParams &sp, const WorldArgs &wa, const double *a, const double *b,
                             unsigned &rechecks)
{
    if constexpr (PREC == GBO_PRECISION_FP32_GUARDED)
    {
        if (sp.kind == GBO_SPACE_KINEMATIC_CHAIN)
        {
            double t1 = 0., t2 = 0.;
            float dx = 0.f, dy = 0.f, dist = 0.f;
#pragma unroll
            for (int i = 0; i < MAXD; ++i)
                if (i < sp.dim)
                {
                    t1 = dadd(t1, a[i]);
                    t2 = dadd(t2, b[i]);
                    float c1, s1, c2, s2;
                    dir32(t1, c1, s1);
                    dir32(t2, c2, s2);
                    dx += c1 - c2;
                    dy += s1 - s2;
                    dist += sqrtf(fmaf(dx, dx, dy * dy));
                }
            dist *= (float)sp.link;
            const float e = wa.e_dist;
            const float lo = (dist - e) * wa.inv_lvs32 * (1.0f - 4.0f * 5.96e-8f);
            const float hi = (dist + e) * wa.inv_lvs32 * (1.0f + 4.0f * 5.96e-8f);
            const float cl = ceilf(lo), ch = ceilf(hi);
            if (cl == ch && lo > 0.f)
                return (int)(sp.factor * (unsigned)cl);
            ++rechecks;
        }
    }
    return segment_count_from_distance(sp, distance64<MAXD>(sp, a, b));
}

// Resolve the lanes whose verdict r is kAmbiguous with the warp-cooperative FP64 test, one state at a
// time (warp-uniform call): the lane writes its FP64 state to the warp's buffer wq (state_of), then the
// whole warp evaluates it.
template <int CK, int MAXD, class StateFn>
__device__ __forceinline__ int resolve_warp(const Eval<CK, MAXD> &ev, int r, int lane, double *wq, double (*wpos)[3],
                                            StateFn state_of, unsigned &rechecks)
{
    unsigned A = __ballot_sync(0xffffffffu, r == kAmbiguous);
    while (A)
    {
        const int src = __ffs(A) - 1;
        A &= A - 1;
        if (lane == src)
            state_of(wq);
        __syncwarp();
        const bool hit = dh_valid64_warp(*ev.arm, wq, ev.w64, *ev.wa, wpos, lane, ev.hz);
        if (lane == src)
        {
            r = hit ? kInvalid : kValid;
            ++rechecks;
        }
        __syncwarp();
    }
    return r;
}

template <int CK, int MAXD>
__global__ void __launch_bounds__(256) motion_plain_kernel(SpaceParams sp, WorldArgs wa, StatesView v1,
                                                           StatesView v2, int64_t n, uint8_t *ok, int32_t *first_j,
                                                           int32_t *nd_out, RunCounters *ctr)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    Eval<CK, MAXD> ev;
    if (!setup_world<CK, MAXD, GBO_PRECISION_FP64>(wa, smem, &bar, ctr, ev))
        return;
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    unsigned evaluated = 0, rechecks = 0;
    for (int64_t e = warp; e < n; e += nwarps)
    {
        double a[MAXD], b[MAXD];
        load_state<MAXD>(v1, e, sp.dim, a);
        load_state<MAXD>(v2, e, sp.dim, b);
        const int nd = segment_count_from_distance(sp, distance64<MAXD>(sp, a, b));
        const int top = nd > 1 ? nd : 1;
        int first = -1;
        for (int base = 1; base <= top; base += 32)
        {
            const int j = base + lane;
            bool bad = false;
            if (j <= top)
            {
                double q[MAXD];
                state_at<MAXD>(sp, a, b, j, nd, top, q);
                bad = !ev.valid64(sp, q);
                ++evaluated;
            }
            const unsigned m = __ballot_sync(0xffffffffu, bad);
            if (m)
            {
                const int jj = base + __ffs(m) - 1;
                first = jj == top ? nd : jj;
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
    flush_counts(ctr, evaluated, rechecks);
}

template <int CK, int MAXD, int PREC>
__global__ void __launch_bounds__(256, CK == GBO_CHECK_DH_SPHERES ? 4 : 1) motion_tile_kernel(SpaceParams sp, WorldArgs wa, StatesView v1, StatesView v2,
                                                          int64_t n, uint8_t *ok, int32_t *first_j, int32_t *nd_out,
                                                          RunCounters *ctr)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    Eval<CK, MAXD> ev;
    if (!setup_world<CK, MAXD, PREC>(wa, smem, &bar, ctr, ev))
        return;
    const int lane = threadIdx.x & 31;
    unsigned evaluated = 0, rechecks = 0;
    for (;;)
    {
        unsigned long long tile = 0;
        if (lane == 0)
            tile = atomicAdd(&ctr->queue, 1ull);
        tile = __shfl_sync(0xffffffffu, tile, 0);
        const int64_t e0 = (int64_t)tile * 32;
        if (e0 >= n)
            break;
        const int64_t e = e0 + lane;
        const bool have = e < n;
        int nd = 0, top = 1, next = 1, first = -1;
        if (have)
        {
            double a[MAXD], b[MAXD];
            load_state<MAXD>(v1, e, sp.dim, a);
            load_state<MAXD>(v2, e, sp.dim, b);
            nd = segment_count<MAXD, PREC>(sp, wa, a, b, rechecks);
            top = nd > 1 ? nd : 1;
        }
        bool live = have;
        unsigned M = __ballot_sync(0xffffffffu, live);
        while (M)
        {
            const int cnt = __popc(M);
            const int r = lane % cnt, rep = lane / cnt;
            const int owner = __fns(M, 0, r + 1);
            const int o_next = __shfl_sync(0xffffffffu, next, owner);
            const int o_top = __shfl_sync(0xffffffffu, top, owner);
            const int o_nd = __shfl_sync(0xffffffffu, nd, owner);
            const int j = o_next + rep;
            int verdict = kValid;
            if (j <= o_top)
            {
                double a[MAXD], b[MAXD];
                load_state<MAXD>(v1, e0 + owner, sp.dim, a);
                load_state<MAXD>(v2, e0 + owner, sp.dim, b);
                verdict = ev.template eval_at<PREC>(sp, a, b, j, o_nd, o_top, rechecks);
                ++evaluated;
            }
            if constexpr (CK == GBO_CHECK_DH_SPHERES && PREC == GBO_PRECISION_FP32_GUARDED)
            {
                __shared__ double dh_q[8][GBO_MAXD];
                __shared__ double dh_pos[8][9][3];
                const int w = threadIdx.x >> 5;
                verdict = resolve_warp(ev, verdict, lane, dh_q[w], dh_pos[w],
                                       [&](double *q) {
                                           double a[MAXD], b[MAXD];
                                           load_state<MAXD>(v1, e0 + owner, sp.dim, a);
                                           load_state<MAXD>(v2, e0 + owner, sp.dim, b);
                                           state_at<MAXD>(sp, a, b, j, o_nd, o_top, q);
                                       },
                                       rechecks);
            }
            const bool bad = verdict == kInvalid;
            const unsigned B = __ballot_sync(0xffffffffu, bad);
            if (live)
            {
                const int myr = __popc(M & ((1u << lane) - 1u));
                unsigned G = 0;
                for (int l = myr; l < 32; l += cnt)
                    G |= 1u << l;
                const unsigned Bm = B & G;
                if (Bm)
                {
                    const int l = __ffs(Bm) - 1;
                    const int jj = next + (l - myr) / cnt;
                    first = jj == top ? nd : jj;
                    live = false;
                }
                else
                {
                    const int assigned = __popc(G);
                    next += assigned;
                    if (next > top)
                        live = false;
                }
            }
            M = __ballot_sync(0xffffffffu, live);
        }
        if (have)
        {
            ok[e] = first < 0 ? 1 : 0;
            if (first_j)
                first_j[e] = first;
            if (nd_out)
                nd_out[e] = nd;
        }
    }
    flush_counts(ctr, evaluated, rechecks);
}

template <int CK, int MAXD, int PREC>
__global__ void __launch_bounds__(256, CK == GBO_CHECK_DH_SPHERES ? 4 : 1) motion_warp_kernel(SpaceParams sp, WorldArgs wa, StatesView v1, StatesView v2,
                                                          int64_t n, uint8_t *ok, int32_t *first_j, int32_t *nd_out,
                                                          RunCounters *ctr)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    Eval<CK, MAXD> ev;
    if (!setup_world<CK, MAXD, PREC>(wa, smem, &bar, ctr, ev))
        return;
    const int lane = threadIdx.x & 31;
    unsigned evaluated = 0, rechecks = 0;
    for (;;)
    {
        unsigned long long ei = 0;
        if (lane == 0)
            ei = atomicAdd(&ctr->queue, 1ull);
        const int64_t e = (int64_t)__shfl_sync(0xffffffffu, ei, 0);
        if (e >= n)
            break;
        unsigned rc = 0;
        int nd;
        {
            double a[MAXD], b[MAXD];
            load_state<MAXD>(v1, e, sp.dim, a);
            load_state<MAXD>(v2, e, sp.dim, b);
            nd = segment_count<MAXD, PREC>(sp, wa, a, b, rc);
        }
        if (lane == 0)
            rechecks += rc;
        const int top = nd > 1 ? nd : 1;
        int first = -1;
        for (int base = 1; base <= top; base += 32)
        {
            const int j = base + lane;
            int verdict = kValid;
            if (j <= top)
            {
                // the endpoints are re-read per state (same edge in every lane: broadcast L1 hits), so
                // that they do not hold 2 x MAXD doubles of registers across the state loop
                double a[MAXD], b[MAXD];
                load_state<MAXD>(v1, e, sp.dim, a);
                load_state<MAXD>(v2, e, sp.dim, b);
                verdict = ev.template eval_at<PREC>(sp, a, b, j, nd, top, rechecks);
                ++evaluated;
            }
            if constexpr (CK == GBO_CHECK_DH_SPHERES && PREC == GBO_PRECISION_FP32_GUARDED)
            {
                __shared__ double dh_q[8][GBO_MAXD];
                __shared__ double dh_pos[8][9][3];
                const int w = threadIdx.x >> 5;
                verdict = resolve_warp(ev, verdict, lane, dh_q[w], dh_pos[w],
                                       [&](double *q) {
                                           double a[MAXD], b[MAXD];
                                           load_state<MAXD>(v1, e, sp.dim, a);
                                           load_state<MAXD>(v2, e, sp.dim, b);
                                           state_at<MAXD>(sp, a, b, j, nd, top, q);
                                       },
                                       rechecks);
            }
            const bool bad = verdict == kInvalid;
            const unsigned m = __ballot_sync(0xffffffffu, bad);
            if (m)
            {
                const int jj = base + __ffs(m) - 1;
                first = jj == top ? nd : jj;
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
    flush_counts(ctr, evaluated, rechecks);
}

// lastValid of DiscreteMotionValidator.cpp:66-68,79-81 from (first_j, nd).
template <int MAXD>
__global__ void last_valid_kernel(SpaceParams sp, StatesView v1, StatesView v2, const int32_t *first_j,
                                  const int32_t *nd, int64_t n, double *last_t, MutStatesView out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    const int fj = first_j[i];
    const double nan = __longlong_as_double(0x7ff8000000000000ll);
    if (fj < 0)
    {
        if (last_t)
            last_t[i] = nan;
        if (out.p)
            for (int d = 0; d < sp.dim; ++d)
                out(i, d) = nan;
        return;
    }
    const double t = ddiv((double)(fj - 1), (double)nd[i]);
    if (last_t)
        last_t[i] = t;
    if (out.p)
    {
        double a[MAXD], b[MAXD], q[MAXD];
        load_state<MAXD>(v1, i, sp.dim, a);
        load_state<MAXD>(v2, i, sp.dim, b);
        interpolate64<MAXD>(sp, a, b, t, q);
        for (int d = 0; d < sp.dim; ++d)
            out(i, d) = q[d];
    }
}

template <int MAXD>
__global__ void distance_kernel(SpaceParams sp, StatesView va, StatesView vb, int64_t n, double *out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double a[MAXD], b[MAXD];
    load_state<MAXD>(va, i, sp.dim, a);
    load_state<MAXD>(vb, i, sp.dim, b);
    out[i] = distance64<MAXD>(sp, a, b);
}

template <int MAXD>
__global__ void interpolate_kernel(SpaceParams sp, StatesView va, StatesView vb, const double *t, int64_t n,
                                   MutStatesView out)
{
    const int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
        return;
    double a[MAXD], b[MAXD], q[MAXD];
    load_state<MAXD>(va, i, sp.dim, a);
    load_state<MAXD>(vb, i, sp.dim, b);
    interpolate64<MAXD>(sp, a, b, t[i], q);
    for (int d = 0; d < sp.dim; ++d)
        out(i, d) = q[d];
}

// SpaceInformation::getMotionStates(s1, s2, states, count, endpoints, alloc = true)
// (SpaceInformation.cpp:215-286) for a batch of edges: edge e yields m rows e*m .. e*m + m - 1:
// [s1,] interpolate(s1, s2, j / (count + 1)) for j = 1..count[, s2]. Thread per output row.
template <int MAXD>
__global__ void motion_states_kernel(SpaceParams sp, StatesView v1, StatesView v2, int64_t n, unsigned count,
                                     int endpoints, MutStatesView out)
{
    const int64_t m = endpoints ? (int64_t)count + 2 : (int64_t)count;
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n * m; r += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t e = r / m, k = r - e * m;
        double a[MAXD], b[MAXD], q[MAXD];
        load_state<MAXD>(v1, e, sp.dim, a);
        load_state<MAXD>(v2, e, sp.dim, b);
        if (endpoints && k == 0)
            for (int d = 0; d < sp.dim; ++d)
                out(r, d) = a[d];
        else if (endpoints && k == m - 1)
            for (int d = 0; d < sp.dim; ++d)
                out(r, d) = b[d];
        else
        {
            const unsigned j = (unsigned)(endpoints ? k : k + 1);
            interpolate64<MAXD>(sp, a, b, ddiv((double)j, (double)(count + 1u)), q);
            for (int d = 0; d < sp.dim; ++d)
                out(r, d) = q[d];
        }
    }
}

// Row gather: out row i = src row idx[i] (UniformValidStateSampler results).
template <int MAXD>
__global__ void gather_rows_kernel(StatesView src, const int64_t *idx, int64_t n, int dim, MutStatesView out)
{
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        const int64_t j = idx[i];
        for (int d = 0; d < dim; ++d)
            out(i, d) = src(j, d);
    }
}

// SpaceInformation::checkMotion(states, count, firstInvalid) (SpaceInformation.cpp:288-299): first
// invalid index of an ordered chain, by a grid-stride scan with an atomicMin.
template <int CK, int MAXD>
__global__ void __launch_bounds__(256) states_chain_kernel(SpaceParams sp, WorldArgs wa, StatesView v, int64_t n,
                                                           unsigned long long *first, RunCounters *ctr)
{
    extern __shared__ __align__(128) unsigned char smem[];
    __shared__ uint64_t bar;
    Eval<CK, MAXD> ev;
    if (!setup_world<CK, MAXD, GBO_PRECISION_FP64>(wa, smem, &bar, ctr, ev))
        return;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    {
        if ((unsigned long long)i >= *(volatile unsigned long long *)first)
            break;
        double q[MAXD];
        load_state<MAXD>(v, i, sp.dim, q);
        if (!ev.valid64(sp, q))
            atomicMin(first, (unsigned long long)i);
    }
}

// ---------------------------------------------------------------- host-side launchers

template <int CK, int MAXD, int PREC>
static void launch_validity_t(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v, int64_t n,
                              uint8_t *out, RunCounters *ctr)
{
    auto k = validity_kernel<CK, MAXD, PREC>;
    const unsigned sm = world_smem_bytes(wa, PREC);
    const int grid = persistent_grid((const void *)k, 256, sm, lc, (n + 255) / 256);
    k<<<grid, 256, sm, lc.stream>>>(sp, wa, v, n, out, ctr);
    note_launch();
}

template <int CK, int MAXD, int PREC>
static void launch_motion_t(const LaunchCfg &lc, int schedule, const SpaceParams &sp, const WorldArgs &wa,
                            StatesView v1, StatesView v2, int64_t n, uint8_t *ok, int32_t *fj, int32_t *nd,
                            RunCounters *ctr)
{
    if (schedule == GBO_SCHEDULE_PLAIN)
    {
        auto k = motion_plain_kernel<CK, MAXD>;
        const unsigned sm = world_smem_bytes(wa, GBO_PRECISION_FP64);
        const int grid = persistent_grid((const void *)k, 256, sm, lc, (n * 32 + 255) / 256);
        k<<<grid, 256, sm, lc.stream>>>(sp, wa, v1, v2, n, ok, fj, nd, ctr);
    }
    else if (schedule == GBO_SCHEDULE_WARP)
    {
        auto k = motion_warp_kernel<CK, MAXD, PREC>;
        const unsigned sm = world_smem_bytes(wa, PREC);
        const int grid = persistent_grid((const void *)k, 256, sm, lc, (n * 32 + 255) / 256);
        k<<<grid, 256, sm, lc.stream>>>(sp, wa, v1, v2, n, ok, fj, nd, ctr);
    }
    else
    {
        auto k = motion_tile_kernel<CK, MAXD, PREC>;
        const unsigned sm = world_smem_bytes(wa, PREC);
        const int grid = persistent_grid((const void *)k, 256, sm, lc, (n + 255) / 256);
        k<<<grid, 256, sm, lc.stream>>>(sp, wa, v1, v2, n, ok, fj, nd, ctr);
    }
    note_launch();
}

template <int CK, int MAXD>
static void launch_chain_t(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v, int64_t n,
                           unsigned long long *first, RunCounters *ctr)
{
    auto k = states_chain_kernel<CK, MAXD>;
    const unsigned sm = world_smem_bytes(wa, GBO_PRECISION_FP64);
    const int grid = persistent_grid((const void *)k, 256, sm, lc, (n + 255) / 256);
    k<<<grid, 256, sm, lc.stream>>>(sp, wa, v, n, first, ctr);
    note_launch();
}

// Dispatch on (checker kind, dimension bucket, precision).
#define GBO_DISPATCH(CKV, DIM, PRECV, CALL)                                                                          \
    do                                                                                                               \
    {                                                                                                                \
        if ((CKV) == GBO_CHECK_CIRCLES)                                                                              \
        {                                                                                                            \
            constexpr int CK = GBO_CHECK_CIRCLES, MAXD = 2, PREC = GBO_PRECISION_FP64;                               \
            CALL;                                                                                                    \
        }                                                                                                            \
        else if ((CKV) == GBO_CHECK_CHAIN_SEGMENTS)                                                                  \
        {                                                                                                            \
            constexpr int CK = GBO_CHECK_CHAIN_SEGMENTS;                                                             \
            if ((DIM) == 10)                                                                                         \
            {                                                                                                        \
                constexpr int MAXD = 10;                                                                             \
                if ((PRECV) == GBO_PRECISION_FP64)                                                                   \
                {                                                                                                    \
                    constexpr int PREC = GBO_PRECISION_FP64;                                                         \
                    CALL;                                                                                            \
                }                                                                                                    \
                else                                                                                                 \
                {                                                                                                    \
                    constexpr int PREC = GBO_PRECISION_FP32_GUARDED;                                                 \
                    CALL;                                                                                            \
                }                                                                                                    \
            }                                                                                                        \
            else                                                                                                     \
            {                                                                                                        \
                constexpr int MAXD = 16;                                                                             \
                if ((PRECV) == GBO_PRECISION_FP64)                                                                   \
                {                                                                                                    \
                    constexpr int PREC = GBO_PRECISION_FP64;                                                         \
                    CALL;                                                                                            \
                }                                                                                                    \
                else                                                                                                 \
                {                                                                                                    \
                    constexpr int PREC = GBO_PRECISION_FP32_GUARDED;                                                 \
                    CALL;                                                                                            \
                }                                                                                                    \
            }                                                                                                        \
        }                                                                                                            \
        else if ((CKV) == GBO_CHECK_DH_SPHERES)                                                                      \
        {                                                                                                            \
            constexpr int CK = GBO_CHECK_DH_SPHERES, MAXD = 8;                                                       \
            if ((PRECV) == GBO_PRECISION_FP64)                                                                       \
            {                                                                                                        \
                constexpr int PREC = GBO_PRECISION_FP64;                                                             \
                CALL;                                                                                                \
            }                                                                                                        \
            else                                                                                                     \
            {                                                                                                        \
                constexpr int PREC = GBO_PRECISION_FP32_GUARDED;                                                     \
                CALL;                                                                                                \
            }                                                                                                        \
        }                                                                                                            \
        else                                                                                                         \
        {                                                                                                            \
            constexpr int CK = GBO_CHECK_ALL_VALID, MAXD = 16, PREC = GBO_PRECISION_FP64;                            \
            CALL;                                                                                                    \
        }                                                                                                            \
    } while (0)

void launch_validity(const LaunchCfg &lc, int precision, const SpaceParams &sp, const WorldArgs &wa, StatesView v,
                     int64_t n, uint8_t *out, RunCounters *ctr)
{
    if (wa.kind == GBO_CHECK_CHAIN_SEGMENTS && precision == GBO_PRECISION_FP32_GUARDED &&
        launch_chain_validity_warp(lc, sp, wa, v, n, out, ctr))
        return;
    GBO_DISPATCH(wa.kind, sp.dim, precision, (launch_validity_t<CK, MAXD, PREC>(lc, sp, wa, v, n, out, ctr)));
}

void launch_motion(const LaunchCfg &lc, int precision, int schedule, const SpaceParams &sp, const WorldArgs &wa,
                   StatesView v1, StatesView v2, int64_t n, uint8_t *ok, int32_t *fj, int32_t *nd, RunCounters *ctr)
{
    if (wa.kind == GBO_CHECK_CHAIN_SEGMENTS && precision == GBO_PRECISION_FP32_GUARDED &&
        schedule == GBO_SCHEDULE_WARP && launch_chain_motion_warp(lc, sp, wa, v1, v2, n, ok, fj, nd, ctr))
        return;
    GBO_DISPATCH(wa.kind, sp.dim, precision,
                 (launch_motion_t<CK, MAXD, PREC>(lc, schedule, sp, wa, v1, v2, n, ok, fj, nd, ctr)));
}

void launch_states_chain(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v, int64_t n,
                         unsigned long long *first, RunCounters *ctr)
{
    GBO_DISPATCH(wa.kind, sp.dim, GBO_PRECISION_FP64, (launch_chain_t<CK, MAXD>(lc, sp, wa, v, n, first, ctr)));
}

void launch_last_valid(const LaunchCfg &lc, const SpaceParams &sp, StatesView v1, StatesView v2, const int32_t *fj,
                       const int32_t *nd, int64_t n, double *last_t, MutStatesView out)
{
    const int grid = (int)((n + 255) / 256);
    if (grid == 0)
        return;
    last_valid_kernel<GBO_MAXD><<<grid, 256, 0, lc.stream>>>(sp, v1, v2, fj, nd, n, last_t, out);
    note_launch();
}

void launch_distance(const LaunchCfg &lc, const SpaceParams &sp, StatesView a, StatesView b, int64_t n, double *out)
{
    const int grid = (int)((n + 255) / 256);
    if (grid == 0)
        return;
    distance_kernel<GBO_MAXD><<<grid, 256, 0, lc.stream>>>(sp, a, b, n, out);
    note_launch();
}

void launch_motion_states(const LaunchCfg &lc, const SpaceParams &sp, StatesView v1, StatesView v2, int64_t n,
                          unsigned count, int endpoints, MutStatesView out)
{
    const int64_t rows = n * (endpoints ? (int64_t)count + 2 : (int64_t)count);
    const int64_t grid = std::min<int64_t>((rows + 255) / 256, (int64_t)lc.sm_count * 16);
    if (grid == 0)
        return;
    motion_states_kernel<GBO_MAXD><<<(int)grid, 256, 0, lc.stream>>>(sp, v1, v2, n, count, endpoints, out);
    note_launch();
}

void launch_gather_rows(const LaunchCfg &lc, StatesView src, const int64_t *idx, int64_t n, int dim,
                        MutStatesView out)
{
    const int64_t grid = std::min<int64_t>((n + 255) / 256, (int64_t)lc.sm_count * 16);
    if (grid == 0)
        return;
    gather_rows_kernel<GBO_MAXD><<<(int)grid, 256, 0, lc.stream>>>(src, idx, n, dim, out);
    note_launch();
}

// Self-test of the bounded waits: a barrier nothing arrives at, waited on for limit_ns; out[0] = 1 when
// the wait ran out, out[1] = the nanoseconds it took.
__global__ void wait_probe_kernel(unsigned long long limit_ns, unsigned long long *out)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0)
        mbar_init(&bar, 1);
    __syncthreads();
    const unsigned long long t0 = global_ns();
    const bool ok = mbar_wait_bounded(&bar, 0, limit_ns);
    if (threadIdx.x == 0)
    {
        out[0] = ok ? 0ull : 1ull;
        out[1] = global_ns() - t0;
    }
}

void launch_wait_probe(unsigned long long limit_ns, unsigned long long *out)
{
    wait_probe_kernel<<<1, 32>>>(limit_ns, out);
    note_launch();
}

void launch_interpolate(const LaunchCfg &lc, const SpaceParams &sp, StatesView a, StatesView b, const double *t,
                        int64_t n, MutStatesView out)
{
    const int grid = (int)((n + 255) / 256);
    if (grid == 0)
        return;
    interpolate_kernel<GBO_MAXD><<<grid, 256, 0, lc.stream>>>(sp, a, b, t, n, out);
    note_launch();
}

}  // namespace gbo
