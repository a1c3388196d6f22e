// Kernel-side argument structures and the launcher interface between the C ABI (capi.cu) and the
// kernel translation units.
#pragma once
#include "common.cuh"
#include "checkers.cuh"

namespace gbo
{

struct RunCounters
{
    unsigned long long queue;      // work-queue head of persistent kernels (reset before each launch)
    unsigned long long evaluated;  // states evaluated
    unsigned long long rechecked;  // states (or segment counts / kNN queries) re-evaluated in FP64
    unsigned long long fallbacks;  // kNN queries answered by the exact FP64 scan
    unsigned long long hazards;    // FP64 decisions a one-ulp change of a sine or cosine could reverse
    unsigned long long bytes;      // kNN cell search: feature and box bytes read
    unsigned int max_err_bits;     // kNN: largest |FP32 - FP64| distance of a re-checked candidate (float bits)
    unsigned int timeout;          // a bounded wait ran out
    unsigned int error;
};

struct DHArm
{
    int joints;
    int spl;          // spheres per link
    double rs;        // robot sphere radius
    double a[8], d[8];
    float ca[8], sa[8];  // cos/sin of alpha (exactly 0 or +-1)
    float af[8], dfl[8];
};

struct WorldArgs
{
    int kind;
    int n;
    const void *data64;   // FP64 rows (circles x,y,r*r | segments x0,y0,x1,y1 | spheres x,y,z,r)
    unsigned bytes64;     // padded to 16 bytes
    int stage64;          // stage data64 into shared memory
    const void *data32;   // FP32 rows (ChainSegF32 | float4 spheres)
    unsigned bytes32;
    int stage32;
    ChainGuard guard;
    float e_dist;         // bound on |fp32 - fp64| of the chain workspace distance
    float inv_lvs32;      // 1 / longest valid segment, FP32
    DHArm arm;
    // uniform grid over the world spheres (cells hold spheres whose box grown by rs + margin overlaps)
    const int *cell_start;
    const int *cell_items;
    const float4 *cell_items4;  // the listed spheres themselves (FP32), parallel to cell_items
    int grid_n;
    float glo[3], ginv[3];
    double glo64[3], ginv64[3];
    float dh_e;           // bound on |d^2 - (rs+ro)^2| error of the FP32 sphere (box) test near contact
    int boxes;            // DH arm world of axis-aligned boxes: rows (cx, cy, cz, hx, hy, hz), FP32 cell
                          // items two float4 each, (cx, cy, cz, hx) and (hy, hz, 0, 0)
    float dh_qmax;  // largest |joint angle| the FP32 guard covers (larger: FP64)
    // one-ulp hazard bounds of the FP64 forms (checkers.cuh): how far a chain joint position / a DH sphere
    // centre (Euclidean) can move when every sine and cosine of the forward kinematics moves by one ulp
    double hz_pos;
    double hz_dh;
    const unsigned *test_order;  // kinematic chain: segment-test order (likely intersections first)
};

struct LaunchCfg
{
    cudaStream_t stream;
    int sm_count;
};

int persistent_grid(const void *kernel, int block, unsigned smem, const LaunchCfg &lc, int64_t max_blocks);
unsigned world_smem_bytes(const WorldArgs &wa, int precision);
void note_launch();

void launch_validity(const LaunchCfg &lc, int precision, const SpaceParams &sp, const WorldArgs &wa, StatesView v,
                     int64_t n, uint8_t *out, RunCounters *ctr);
void launch_motion(const LaunchCfg &lc, int precision, int schedule, const SpaceParams &sp, const WorldArgs &wa,
                   StatesView v1, StatesView v2, int64_t n, uint8_t *ok, int32_t *fj, int32_t *nd, RunCounters *ctr);
void launch_states_chain(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v, int64_t n,
                         unsigned long long *first, RunCounters *ctr);
void launch_last_valid(const LaunchCfg &lc, const SpaceParams &sp, StatesView v1, StatesView v2, const int32_t *fj,
                       const int32_t *nd, int64_t n, double *last_t, MutStatesView out);
void launch_chain_hits(cudaStream_t s, const SpaceParams &sp, const WorldArgs &wa, const double *states, int n,
                       unsigned *bits, int words);
bool launch_chain_validity_warp(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v,
                                int64_t n, uint8_t *out, RunCounters *ctr);
bool launch_chain_motion_warp(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v1,
                              StatesView v2, int64_t n, uint8_t *ok, int32_t *fj, int32_t *nd, RunCounters *ctr);
void launch_distance(const LaunchCfg &lc, const SpaceParams &sp, StatesView a, StatesView b, int64_t n, double *out);
void launch_interpolate(const LaunchCfg &lc, const SpaceParams &sp, StatesView a, StatesView b, const double *t,
                        int64_t n, MutStatesView out);
void launch_wait_probe(unsigned long long limit_ns, unsigned long long *out);
void launch_motion_states(const LaunchCfg &lc, const SpaceParams &sp, StatesView v1, StatesView v2, int64_t n,
                          unsigned count, int endpoints, MutStatesView out);
void launch_gather_rows(const LaunchCfg &lc, StatesView src, const int64_t *idx, int64_t n, int dim,
                        MutStatesView out);
bool launch_precision_stats(const LaunchCfg &lc, const SpaceParams &sp, const WorldArgs &wa, StatesView v, int64_t n,
                            void *tally);
void launch_sincos_cr(const LaunchCfg &lc, const double *x, int64_t n, double *s, double *c);

// ---------------------------------------------------------------- DH sphere arm
// FP64 form: the arm definition (this operation order for the sphere centres is the definition the
// test oracle restates), candidates from the uniform grid (a superset of every colliding sphere),
// exact test.
// Hazard test of one FP64 sphere pair (see checkers.cuh): t = |d|^2 with d moved by at most P.
__device__ __forceinline__ void dh_hazard64(double dx, double dy, double dz, double t, double rr2, double P,
                                            unsigned long long *hz)
{
    if (hz && fabs(t - rr2) <= 1e-9)
    {
        const double e = 2.0 * (2.0 * (fabs(dx) + fabs(dy) + fabs(dz)) * P + 3.0 * P * P + 0x1p-51 * (t + rr2));
        if (fabs(t - rr2) <= e)
            atomicAdd(hz, 1ull);
    }
}

// FP64 narrow phase of one robot sphere (centre c, radius rs) and one listed world obstacle `o`, with
// the hazard count: a world sphere (x, y, z, r) is hit iff (dx dx + dy dy) + dz dz < (rs + r)^2; an
// axis-aligned box (cx, cy, cz, hx, hy, hz) iff (gx gx + gy gy) + gz gz < rs rs with
// g = max(|c - centre| - half extent, 0) per axis (the squared distance of c from the box).
__device__ __forceinline__ bool dh_pair64(const double *c, const double *o, double rs, bool boxes, double P,
                                          unsigned long long *hz)
{
    double dx, dy, dz, rr;
    if (boxes)
    {
        dx = dsub(fabs(dsub(c[0], o[0])), o[3]);
        dy = dsub(fabs(dsub(c[1], o[1])), o[4]);
        dz = dsub(fabs(dsub(c[2], o[2])), o[5]);
        dx = dx > 0.0 ? dx : 0.0;
        dy = dy > 0.0 ? dy : 0.0;
        dz = dz > 0.0 ? dz : 0.0;
        rr = rs;
    }
    else
    {
        dx = dsub(c[0], o[0]);
        dy = dsub(c[1], o[1]);
        dz = dsub(c[2], o[2]);
        rr = dadd(rs, o[3]);
    }
    const double t = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)), rr2 = dmul(rr, rr);
    dh_hazard64(dx, dy, dz, t, rr2, P, hz);
    return t < rr2;
}

template <int MAXD>
__device__ bool dh_valid64(const DHArm &arm, const double *q, const double *w, const WorldArgs &wa,
                           unsigned long long *hz = nullptr)
{
    const int stride = wa.boxes ? 6 : 4;
    double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double p[3] = {0, 0, 0};
    const int G = wa.grid_n;
#pragma unroll 1
    for (int i = 0; i < arm.joints; ++i)
    {
        double cq, sq;
        sincos_cr(q[i], &sq, &cq);
        const double ca = (double)arm.ca[i], sa = (double)arm.sa[i];
        const double A[3][3] = {{cq, dmul(-sq, ca), dmul(sq, sa)}, {sq, dmul(cq, ca), dmul(-cq, sa)}, {0.0, sa, ca}};
        const double pA[3] = {dmul(arm.a[i], cq), dmul(arm.a[i], sq), arm.d[i]};
        double Rn[3][3], pn[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
#pragma unroll
            for (int k = 0; k < 3; ++k)
                Rn[r][k] = dadd(dadd(dmul(R[r][0], A[0][k]), dmul(R[r][1], A[1][k])), dmul(R[r][2], A[2][k]));
            pn[r] = dadd(dadd(dadd(dmul(R[r][0], pA[0]), dmul(R[r][1], pA[1])), dmul(R[r][2], pA[2])), p[r]);
        }
#pragma unroll 1
        for (int k = 0; k < arm.spl; ++k)
        {
            const double f = ddiv(dadd((double)k, 0.5), (double)arm.spl);
            double c[3];
#pragma unroll
            for (int r = 0; r < 3; ++r)
                c[r] = dadd(p[r], dmul(f, dsub(pn[r], p[r])));
            int cell[3];
            bool inside = true;
#pragma unroll
            for (int r = 0; r < 3; ++r)
            {
                double g = floor((c[r] - wa.glo64[r]) * wa.ginv64[r]);
                inside &= (g >= 0.0 && g < (double)G);
                cell[r] = (int)g;
            }
            if (!inside)
                continue;
            const int cid = (cell[0] * G + cell[1]) * G + cell[2];
            const int b = wa.cell_start[cid], e = wa.cell_start[cid + 1];
            for (int it = b; it < e; ++it)
                if (dh_pair64(c, w + stride * wa.cell_items[it], arm.rs, wa.boxes, wa.hz_dh, hz))
                    return false;
        }
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
            p[r] = pn[r];
#pragma unroll
            for (int k = 0; k < 3; ++k)
                R[r][k] = Rn[r][k];
        }
    }
    return true;
}

// FP64 form of one state, warp-cooperative (warp-uniform call; q and pos in shared memory, q holding the
// state): every lane runs the forward kinematics above (identical values, so one warp instruction per
// step), lane 0 records the joint positions in pos[0..joints], and the spheres are spread over the
// lanes, each centre and each pair test in the operation order of dh_valid64. Same boolean as
// dh_valid64 on the same state. Out of line: the callers' FP32 loops keep their registers.
static __device__ __noinline__ bool dh_valid64_warp(const DHArm &arm, const double *q, const double *w,
                                                    const WorldArgs &wa, double (*pos)[3], int lane,
                                                    unsigned long long *hz)
{
    double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    double p[3] = {0, 0, 0};
    const int G = wa.grid_n;
    if (lane == 0)
        pos[0][0] = pos[0][1] = pos[0][2] = 0.0;
    // the joints' sines and cosines, one joint per lane (the FK below is the same in every lane)
    double cq_l = 1.0, sq_l = 0.0;
    if (lane < arm.joints)
        sincos(q[lane], &sq_l, &cq_l);
#pragma unroll 1
    for (int i = 0; i < arm.joints; ++i)
    {
        const double cq = __shfl_sync(0xffffffffu, cq_l, i), sq = __shfl_sync(0xffffffffu, sq_l, i);
        const double ca = (double)arm.ca[i], sa = (double)arm.sa[i];
        const double A[3][3] = {{cq, dmul(-sq, ca), dmul(sq, sa)}, {sq, dmul(cq, ca), dmul(-cq, sa)}, {0.0, sa, ca}};
        const double pA[3] = {dmul(arm.a[i], cq), dmul(arm.a[i], sq), arm.d[i]};
        double Rn[3][3], pn[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
#pragma unroll
            for (int k = 0; k < 3; ++k)
                Rn[r][k] = dadd(dadd(dmul(R[r][0], A[0][k]), dmul(R[r][1], A[1][k])), dmul(R[r][2], A[2][k]));
            pn[r] = dadd(dadd(dadd(dmul(R[r][0], pA[0]), dmul(R[r][1], pA[1])), dmul(R[r][2], pA[2])), p[r]);
        }
        if (lane == 0)
            for (int r = 0; r < 3; ++r)
                pos[i + 1][r] = pn[r];
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
            p[r] = pn[r];
#pragma unroll
            for (int k = 0; k < 3; ++k)
                R[r][k] = Rn[r][k];
        }
    }
    __syncwarp();
    bool hit = false;
    for (int s = lane; s < arm.joints * arm.spl && !hit; s += 32)
    {
        const int i = s / arm.spl, k = s - i * arm.spl;
        const double f = ddiv(dadd((double)k, 0.5), (double)arm.spl);
        double c[3];
        int cell[3];
        bool inside = true;
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
            c[r] = dadd(pos[i][r], dmul(f, dsub(pos[i + 1][r], pos[i][r])));
            const double g = floor((c[r] - wa.glo64[r]) * wa.ginv64[r]);
            inside &= (g >= 0.0 && g < (double)G);
            cell[r] = (int)g;
        }
        if (!inside)
            continue;
        const int cid = (cell[0] * G + cell[1]) * G + cell[2];
        const int b = wa.cell_start[cid], e = wa.cell_start[cid + 1];
        const int stride = wa.boxes ? 6 : 4;
        for (int it = b; it < e && !hit; ++it)
            hit = dh_pair64(c, w + stride * wa.cell_items[it], arm.rs, wa.boxes, wa.hz_dh, hz);
    }
    return __any_sync(0xffffffffu, hit);
}

// FP32 form: FK, centres and the narrow phase in FP32; a pair whose d^2 - (rs+ro)^2 (boxes: the squared
// distance to the box - rs^2) lies within +-dh_e is ambiguous (dh_e bounds the FP32 error of that
// difference near contact). q: the joint
// angles as FP32 values within u|q| (+1e-12) of the reference's FP64 angles.
template <int MAXD>
__device__ int dh_valid32(const DHArm &arm, const float *q, const float4 *sph, const WorldArgs &wa)
{
    float R[3][3] = {{1.f, 0.f, 0.f}, {0.f, 1.f, 0.f}, {0.f, 0.f, 1.f}};
    float p[3] = {0.f, 0.f, 0.f};
    const int G = wa.grid_n;
    const float rs = (float)arm.rs, E = wa.dh_e;
    const float inv_spl = 1.0f / (float)arm.spl;
    bool amb = false;
#pragma unroll 1
    for (int i = 0; i < arm.joints; ++i)
    {
        if (!(fabsf(q[i]) <= wa.dh_qmax))
            return kAmbiguous;  // outside the angle range the error bound was derived for
        float cq, sq;
        sincosf(q[i], &sq, &cq);
        const float ca = arm.ca[i], sa = arm.sa[i];
        const float A[3][3] = {{cq, -sq * ca, sq * sa}, {sq, cq * ca, -cq * sa}, {0.f, sa, ca}};
        const float pA[3] = {arm.af[i] * cq, arm.af[i] * sq, arm.dfl[i]};
        float Rn[3][3], pn[3];
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
#pragma unroll
            for (int k = 0; k < 3; ++k)
                Rn[r][k] = fmaf(R[r][2], A[2][k], fmaf(R[r][1], A[1][k], R[r][0] * A[0][k]));
            pn[r] = fmaf(R[r][2], pA[2], fmaf(R[r][1], pA[1], fmaf(R[r][0], pA[0], p[r])));
        }
#pragma unroll 1
        for (int k = 0; k < arm.spl; ++k)
        {
            const float f = ((float)k + 0.5f) * inv_spl;
            float c[3];
            int cell[3];
            bool inside = true;
#pragma unroll
            for (int r = 0; r < 3; ++r)
            {
                c[r] = fmaf(f, pn[r] - p[r], p[r]);
                float g = floorf((c[r] - wa.glo[r]) * wa.ginv[r]);
                inside &= (g >= 0.f && g < (float)G);
                cell[r] = (int)g;
            }
            if (!inside)
                continue;
            const int cid = (cell[0] * G + cell[1]) * G + cell[2];
            const int b = __ldg(wa.cell_start + cid), e = __ldg(wa.cell_start + cid + 1);
            if (wa.boxes)
                for (int it = b; it < e; ++it)
                {
                    const float4 o = __ldg(wa.cell_items4 + 2 * it), h = __ldg(wa.cell_items4 + 2 * it + 1);
                    const float dx = fmaxf(fabsf(c[0] - o.x) - o.w, 0.f), dy = fmaxf(fabsf(c[1] - o.y) - h.x, 0.f);
                    const float dz = fmaxf(fabsf(c[2] - o.z) - h.y, 0.f);
                    const float t = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) - rs * rs;
                    if (t < -E)
                        return kInvalid;
                    amb |= (t <= E);
                }
            else
                for (int it = b; it < e; ++it)
                {
                    const float4 o = __ldg(wa.cell_items4 + it);
                    const float dx = c[0] - o.x, dy = c[1] - o.y, dz = c[2] - o.z;
                    const float rr = rs + o.w;
                    const float t = fmaf(dz, dz, fmaf(dy, dy, dx * dx)) - rr * rr;
                    if (t < -E)
                        return kInvalid;
                    amb |= (t <= E);
                }
        }
#pragma unroll
        for (int r = 0; r < 3; ++r)
        {
            p[r] = pn[r];
#pragma unroll
            for (int k = 0; k < 3; ++k)
                R[r][k] = Rn[r][k];
        }
    }
    return amb ? kAmbiguous : kValid;
}

}  // namespace gbo
