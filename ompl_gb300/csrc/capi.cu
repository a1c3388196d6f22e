// C ABI of libgbompl (include/gbompl.h): object lifetimes, argument checking, guard-band bounds,
// the uniform grid over world spheres, staging for host-memory calls, and kernel launches.
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <random>

#include <nvtx3/nvToolsExt.h>

#include "chain_state.cuh"
#include "kernels_nn.cuh"
#include "tma.cuh"

using namespace gbo;

namespace
{
thread_local std::string g_err;
std::atomic<unsigned long long> g_launches{0};

gbo_status fail(gbo_status s, const std::string &msg)
{
    g_err = msg;
    return s;
}

#define CUDA_TRY(expr)                                                                                               \
    do                                                                                                               \
    {                                                                                                                \
        cudaError_t _e = (expr);                                                                                     \
        if (_e != cudaSuccess)                                                                                       \
            return fail(_e == cudaErrorMemoryAllocation ? GBO_ERR_OUT_OF_MEMORY : GBO_ERR_CUDA,                      \
                        std::string(#expr) + ": " + cudaGetErrorString(_e));                                         \
    } while (0)

#define CHECK_LAUNCH()                                                                                               \
    do                                                                                                               \
    {                                                                                                                \
        cudaError_t _e = cudaGetLastError();                                                                         \
        if (_e != cudaSuccess)                                                                                       \
            return fail(GBO_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(_e));                      \
    } while (0)

int g_sm_count = 0;
int g_device_ok = -1;  // -1 unknown, 0 no, 1 yes

gbo_status ensure_device()
{
    if (g_device_ok == 1)
        return GBO_OK;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    {
        cudaGetLastError();
        g_device_ok = 0;
        return fail(GBO_ERR_NO_DEVICE, "no CUDA device");
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p;
    if (cudaGetDeviceProperties(&p, dev) != cudaSuccess)
        return fail(GBO_ERR_NO_DEVICE, "cudaGetDeviceProperties failed");
    if (!(p.major == 10 && p.minor == 3))
        return fail(GBO_ERR_NO_DEVICE, "libgbompl is built for sm_103a only; device is sm_" +
                                           std::to_string(p.major) + std::to_string(p.minor));
    g_sm_count = p.multiProcessorCount;
    g_device_ok = 1;
    return GBO_OK;
}

LaunchCfg lcfg(gbo_stream s)
{
    LaunchCfg lc;
    lc.stream = (cudaStream_t)s;
    lc.sm_count = g_sm_count;
    return lc;
}

constexpr double kU32 = 5.9604644775390625e-08;  // 2^-24, FP32 unit roundoff
// Bound on |cos/sin FP32 - exact| of one link direction (sincos_ff, chain_warp.cuh): Horner rounding
// <= 2 ulp (1.2e-7), Taylor truncation <= 2e-9, reduction and low-part terms < 1e-12.
constexpr double kEpsDir = 1.3e-7;
constexpr double kPiH = 3.141592653589793238462643383279502884;

bool valid_layout(int layout, int64_t n, int64_t ld, int dim)
{
    if (layout == GBO_LAYOUT_SOA)
        return ld >= n;
    if (layout == GBO_LAYOUT_AOS)
        return ld >= dim;
    return false;
}

// Ring of device counter slots so that calls in flight on different streams do not share one.
struct CounterRing
{
    RunCounters *dev = nullptr;
    std::atomic<unsigned> next{0};
    unsigned last = 0;
    static constexpr unsigned kSlots = 64;
    gbo_status init()
    {
        CUDA_TRY(cudaMalloc(&dev, sizeof(RunCounters) * kSlots));
        CUDA_TRY(cudaMemset(dev, 0, sizeof(RunCounters) * kSlots));
        return GBO_OK;
    }
    RunCounters *take(cudaStream_t s)
    {
        unsigned i = next.fetch_add(1) % kSlots;
        last = i;
        cudaMemsetAsync(dev + i, 0, sizeof(RunCounters), s);
        return dev + i;
    }
    ~CounterRing()
    {
        if (dev)
            cudaFree(dev);
    }
};

struct Pinned
{
    void *p = nullptr;
    size_t bytes = 0;
    gbo_status reserve(size_t b)
    {
        if (b <= bytes)
            return GBO_OK;
        if (p)
            cudaFreeHost(p);
        p = nullptr;
        bytes = 0;
        CUDA_TRY(cudaMallocHost(&p, b));
        bytes = b;
        return GBO_OK;
    }
    ~Pinned()
    {
        if (p)
            cudaFreeHost(p);
    }
};

// Per-object device scratch that grows geometrically with the stream-ordered allocator. Outgrown
// buffers are kept until the object is destroyed: freeing them during a call would synchronise the
// whole device (cudaFree) and stall every other stream.
struct DevBuf
{
    void *p = nullptr;
    size_t bytes = 0;
    std::vector<void *> outgrown;
    gbo_status reserve(size_t b, cudaStream_t stream = nullptr)
    {
        if (b <= bytes)
            return GBO_OK;
        const size_t want = std::max(b, 2 * bytes);
        void *np = nullptr;
        CUDA_TRY(cudaMallocAsync(&np, want, stream));
        if (p)
            outgrown.push_back(p);
        p = np;
        bytes = want;
        return GBO_OK;
    }
    ~DevBuf()
    {
        if (p || !outgrown.empty())
            cudaDeviceSynchronize();
        if (p)
            cudaFree(p);
        for (void *q : outgrown)
            cudaFree(q);
    }
};

size_t pad16(size_t b)
{
    return (b + 15) & ~size_t(15);
}
}  // namespace

struct gbo_space
{
    SpaceParams sp{};
    double extent = 0.0;
};

struct gbo_checker
{
    SpaceParams sp{};
    int kind = 0;
    int precision = GBO_PRECISION_FP64;
    WorldArgs wa{};
    void *d64 = nullptr, *d32 = nullptr;
    int *cell_start = nullptr, *cell_items = nullptr;
    float *cell_items4 = nullptr;
    unsigned *test_order = nullptr;
    CounterRing ctr;
    int tuned_schedule = -1;
    std::mutex mu, tune_mu;
    cudaStream_t host_stream = nullptr;
    Pinned pin_in, pin_out;
    DevBuf dev_in, dev_out;
    ~gbo_checker()
    {
        if (d64)
            cudaFree(d64);
        if (d32)
            cudaFree(d32);
        if (cell_start)
            cudaFree(cell_start);
        if (cell_items)
            cudaFree(cell_items);
        if (cell_items4)
            cudaFree(cell_items4);
        if (test_order)
            cudaFree(test_order);
        if (host_stream)
            cudaStreamDestroy(host_stream);
    }
};

struct gbo_sampler
{
    SpaceParams sp{};
    SamplerState *st = nullptr;
    std::mutex mu;
    cudaStream_t host_stream = nullptr;
    Pinned pin;
    DevBuf dev, words;  // words: the word-stream scratch of the device calls
    DevBuf gwork;       // GaussChunk, per-CTA counts and pairs of sampleGaussian
    bool has_saved = false;  // mirrors SamplerState::has_saved (a cached Gaussian value is pending)
    ~gbo_sampler()
    {
        if (host_stream)
            cudaStreamDestroy(host_stream);
        if (st)
            cudaFree(st);
    }
};

// Cell index of a gbo_nn over a RealVector / wrapped space (kernels_nn.cu): built by the first large
// batch after a change of the element set (add / remove / clear clear `valid`).
struct NNBoxCells
{
    bool valid = false;
    int L = 0, C = 0;
    DevBuf cell, count, start, fill, skey, pts8, box;
    DevBuf qcell, qcount, qstart, qfill, qorder;
};

// Cell index of a kinematic-chain gbo_nn (kernels_nn.cu), built like NNBoxCells.
struct NNChainCells
{
    bool valid = false;
    DevBuf key, count, start, fill, skey, sfeat, box, cstart, cbox;
};

struct gbo_nn
{
    SpaceParams sp{};
    int precision = GBO_PRECISION_FP32_GUARDED;
    int64_t cap = 0, size = 0, alive_count = 0;
    int F = 0;
    double *pts64 = nullptr;
    float *feat32 = nullptr;
    unsigned char *alive = nullptr;
    float eps32 = 0.f;
    NNBoxCells cells;
    NNChainCells ccells;
    DevBuf qfeat, fb_list, part, qorder;
    DevBuf ranks;  // keys of the present elements in order (approximate nearest after removals)
    CounterRing ctr;
    unsigned long long queries = 0;
    std::mutex mu;
    cudaStream_t host_stream = nullptr;
    Pinned pin;
    DevBuf dev;
    ~gbo_nn()
    {
        if (host_stream)
            cudaStreamDestroy(host_stream);
        if (pts64)
            cudaFree(pts64);
        if (feat32)
            cudaFree(feat32);
        if (alive)
            cudaFree(alive);
    }
};

namespace
{
// NVTX range over a C-ABI call (visible to ncu / Nsight; no cost without an attached tool)
struct Trace
{
    explicit Trace(const char *name) { nvtxRangePushA(name); }
    ~Trace() { nvtxRangePop(); }
};
}  // namespace

namespace gbo
{
void note_launch()
{
    g_launches.fetch_add(1, std::memory_order_relaxed);
}

int persistent_grid(const void *kernel, int block, unsigned smem, const LaunchCfg &lc, int64_t max_blocks)
{
    static std::mutex mu;
    static std::map<std::pair<const void *, std::pair<unsigned, int>>, int> occ;
    static std::map<const void *, bool> raised;
    int per_sm = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (smem > 48 * 1024 && !raised[kernel])
        {
            // raise the kernel's dynamic shared-memory limit once, to the device's opt-in maximum, so
            // that launches with any world size up to it remain valid
            int dev = 0, optin = 0;
            cudaGetDevice(&dev);
            cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
            cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin - 1024);
            raised[kernel] = true;
        }
        auto key = std::make_pair(kernel, std::make_pair(smem, block));
        auto it = occ.find(key);
        if (it == occ.end())
        {
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, smem);
            if (per_sm < 1)
                per_sm = 1;
            occ[key] = per_sm;
        }
        else
            per_sm = it->second;
    }
    int64_t g = (int64_t)per_sm * lc.sm_count;
    if (max_blocks < g)
        g = max_blocks;
    return (int)(g < 1 ? 1 : g);
}

unsigned world_smem_bytes(const WorldArgs &wa, int precision)
{
    if (precision == GBO_PRECISION_FP32_GUARDED &&
        (wa.kind == GBO_CHECK_CHAIN_SEGMENTS || wa.kind == GBO_CHECK_DH_SPHERES))
        return wa.stage32 ? wa.bytes32 : 0;
    return wa.stage64 ? wa.bytes64 : 0;
}
}  // namespace gbo

namespace
{
// Guard-band bounds of the FP32 kinematic-chain test (see checkers.cuh). All bounds are
// worst-case: eps_dir covers float conversion of the reduced angle (u*pi) plus the sincosf error
// (2 ulp); link vectors VX = c*L have error L*(eps_dir + 2u); a position after k links has error
// k*(L*(eps_dir + u) + u*R) with R the reach; a cross product a x b of vectors with component
// magnitudes <= A, B and component errors da, db has error 2*(da*B + db*A + da*db) + 3u*A*B.
// Each bound is inflated by a safety factor of 2.
void chain_bounds(const SpaceParams &sp, const double *w, int n, ChainGuard &g, std::vector<ChainSegF32> &segs,
                  float &e_dist)
{
    const double u = kU32, L = sp.link, nl = sp.dim;
    const double eps_dir = kEpsDir;
    const double R = nl * L + 0.001;
    const double dV = L * (eps_dir + 2 * u) + 1e-15;
    const double dP = (nl + 1) * (L * (eps_dir + u) + u * R) + 1e-15;
    auto cross = [&](double A, double B, double da, double db) {
        return 2.0 * (da * B + db * A + da * db) + 3.0 * u * A * B + 1e-15;
    };
    const double safety = 2.0;
    // one bound e for the four numerator comparisons (that of s_numer - denom or t_numer - denom,
    // which include the others), stored as the thresholds FLT_EPSILON -/+ e rounded outward
    const double flt_eps = std::ldexp(1.0, -23);
    auto down = [](double x) {
        float f = (float)x;
        return (double)f > x ? std::nextafter(f, -INFINITY) : f;
    };
    auto up = [](double x) {
        float f = (float)x;
        return (double)f < x ? std::nextafter(f, INFINITY) : f;
    };
    auto numer_bound = [&](double A, double B, double C, double eden, double es, double et) {
        const double eu = es + eden + u * 2 * (A * C + A * B), ev = et + eden + u * 2 * (B * C + A * B);
        return safety * std::max(std::max(es, et), std::max(eu, ev));
    };
    g.eps_dir = (float)eps_dir;
    {
        const double A = L, B = L, C = 2 * R, dC = 2 * dP + 2 * u * R;
        const double eden = cross(A, B, dV, dV), es = cross(A, C, dV, dC), et = cross(B, C, dV, dC);
        const double e = numer_bound(A, B, C, eden, es, et);
        g.self_den = up(safety * eden + 1e-12);
        g.self_lo = down(flt_eps - e);
        g.self_hi = up(flt_eps + e);
    }
    segs.resize(n);
    for (int j = 0; j < n; ++j)
    {
        const double x0 = w[4 * j], y0 = w[4 * j + 1], x1 = w[4 * j + 2], y1 = w[4 * j + 3];
        const double sx = x1 - x0, sy = y1 - y0;
        const double B = std::max(std::fabs(sx), std::fabs(sy));
        const double W0 = std::max(std::fabs(x0), std::fabs(y0));
        const double A = L, C = R + W0;
        const double dB = u * B, dC = dP + u * W0 + u * C;
        const double eden = cross(A, B, dV, dB), es = cross(A, C, dV, dC), et = cross(B, C, dB, dC);
        ChainSegF32 s{};
        s.x0 = (float)x0;
        s.y0 = (float)y0;
        s.sx = (float)sx;
        s.sy = (float)sy;
        const double e = numer_bound(A, B, C, eden, es, et);
        s.e_den = up(safety * eden + 1e-12);
        s.lo = down(flt_eps - e);
        s.hi = up(flt_eps + e);
        segs[j] = s;
    }
    // workspace distance (segment_count, FP32 form): dx_i accumulates 2i direction errors and i
    // roundings of partial sums bounded by 2i; the norm adds |ddx| + |ddy| and a relative 2^-22.
    double e = 0.0;
    for (int i = 1; i <= sp.dim; ++i)
    {
        const double ddx = 2.0 * i * eps_dir + u * 2.0 * i * i;
        e += 2.0 * ddx + std::ldexp(1.0, -21) * 2.0 * i;
    }
    e = L * (e + u * sp.dim * 2.0 * sp.dim) + u * L * 2.0 * sp.dim * sp.dim;
    e_dist = (float)(safety * e);
}

// Chain kNN features X_i = sum_{m<=i} cos(theta_m) accumulate i direction errors and i roundings.
float chain_knn_eps(const SpaceParams &sp)
{
    const double u = kU32, L = sp.link;
    const double eps_dir = kEpsDir;
    double e = 0.0;
    for (int i = 1; i <= sp.dim; ++i)
    {
        const double dX = i * eps_dir + u * i * i;            // one feature
        const double ddx = 2.0 * dX + u * 2.0 * i;            // difference of features
        e += 2.0 * ddx + std::ldexp(1.0, -21) * 2.0 * i + u * 2.0 * i * sp.dim;
    }
    return (float)(2.0 * L * e * 1.01 + 1e-12);
}

// Box / wrapped spaces: features are coordinates rounded to FP32 (error u*|x|), squared distance
// accumulated with FMA (relative error <= (dim + 2) u); bound on |sqrt(s32) - d64|.
float box_knn_eps(const SpaceParams &sp)
{
    double m2 = 0.0, span2 = 0.0;
    for (int d = 0; d < sp.dim; ++d)
    {
        const double lo = sp.kind == GBO_SPACE_REAL_VECTOR ? sp.low[d] : -kPiH;
        const double hi = sp.kind == GBO_SPACE_REAL_VECTOR ? sp.high[d] : kPiH;
        const double m = std::max(std::fabs(lo), std::fabs(hi));
        m2 += m * m;
        span2 += (hi - lo) * (hi - lo);
    }
    const double coord = 2.0 * kU32 * std::sqrt(m2) + (sp.kind == GBO_SPACE_REAL_VECTOR ? 0.0 : 4.0 * kU32 * 7.0);
    const double rel = (sp.dim + 4) * kU32 * std::sqrt(span2);
    return (float)(2.0 * (coord + rel) + 1e-12);
}
}  // namespace

// Segment-test order of a kinematic-chain checker. The validity result does not depend on the order in
// which the segment tests run; the warp-cooperative kernels stop at the first round of 32 tests that
// holds a definite intersection, so tests that are likely to intersect go first. The order is a greedy
// cover of the definite intersections found (FP32, guarded) in 8192 states drawn uniformly from the
// joint bounds: repeatedly take the test that intersects in most states not yet covered.
static gbo_status order_chain_tests(gbo_checker *c)
{
    const SpaceParams &sp = c->sp;
    const int n = sp.dim, m = n + 1, nw = c->wa.n;
    const int n_tests = (m - 1) * (m - 2) / 2 + m * nw;
    const int words = (n_tests + 31) / 32;
    const int S = 8192;
    std::mt19937_64 rng(0x9e3779b97f4a7c15ull);
    std::uniform_real_distribution<double> U(-kPiH, kPiH);
    std::vector<double> st((size_t)n * S);
    for (auto &x : st)
        x = U(rng);
    double *dst = nullptr;
    unsigned *dbits = nullptr;
    CUDA_TRY(cudaMalloc(&dst, st.size() * sizeof(double)));
    if (cudaMalloc(&dbits, (size_t)S * words * sizeof(unsigned)) != cudaSuccess)
    {
        cudaFree(dst);
        return fail(GBO_ERR_OUT_OF_MEMORY, "test-order scratch allocation failed");
    }
    cudaMemcpy(dst, st.data(), st.size() * sizeof(double), cudaMemcpyHostToDevice);
    WorldArgs wa = c->wa;
    wa.test_order = nullptr;
    launch_chain_hits(nullptr, sp, wa, dst, S, dbits, words);
    std::vector<unsigned> bits((size_t)S * words);
    cudaError_t e = cudaMemcpy(bits.data(), dbits, bits.size() * sizeof(unsigned), cudaMemcpyDeviceToHost);
    cudaFree(dst);
    cudaFree(dbits);
    if (e != cudaSuccess)
        return fail(GBO_ERR_CUDA, std::string("test ordering: ") + cudaGetErrorString(e));
    // transpose to per-test state bitsets
    const int sw = S / 64;
    std::vector<uint64_t> tb((size_t)n_tests * sw, 0);
    for (int s = 0; s < S; ++s)
        for (int t = 0; t < n_tests; ++t)
            if (bits[(size_t)s * words + t / 32] >> (t % 32) & 1u)
                tb[(size_t)t * sw + s / 64] |= 1ull << (s % 64);
    std::vector<uint64_t> covered(sw, 0);
    std::vector<char> used(n_tests, 0);
    std::vector<unsigned> order;
    order.reserve(n_tests);
    for (int step = 0; step < n_tests; ++step)
    {
        int best = -1;
        long best_gain = -1;
        for (int t = 0; t < n_tests; ++t)
        {
            if (used[t])
                continue;
            long g = 0;
            for (int w = 0; w < sw; ++w)
                g += __builtin_popcountll(tb[(size_t)t * sw + w] & ~covered[w]);
            if (g > best_gain)
            {
                best_gain = g;
                best = t;
            }
        }
        if (best_gain <= 0)
            break;
        used[best] = 1;
        order.push_back(chain_test_entry(best, n, nw));
        for (int w = 0; w < sw; ++w)
            covered[w] |= tb[(size_t)best * sw + w];
    }
    for (int t = 0; t < n_tests; ++t)
        if (!used[t])
            order.push_back(chain_test_entry(t, n, nw));
    CUDA_TRY(cudaMalloc(&c->test_order, order.size() * sizeof(unsigned)));
    CUDA_TRY(cudaMemcpy(c->test_order, order.data(), order.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
    c->wa.test_order = c->test_order;
    return GBO_OK;
}

extern "C" {

const char *gbo_status_string(gbo_status s)
{
    switch (s)
    {
        case GBO_OK:
            return "ok";
        case GBO_ERR_INVALID_ARGUMENT:
            return "invalid argument";
        case GBO_ERR_CUDA:
            return "CUDA error";
        case GBO_ERR_NO_DEVICE:
            return "no usable device";
        case GBO_ERR_OUT_OF_MEMORY:
            return "out of memory";
        case GBO_ERR_TIMEOUT:
            return "device wait timed out";
        case GBO_ERR_UNSUPPORTED:
            return "unsupported";
        default:
            return "unknown status";
    }
}

const char *gbo_last_error(void)
{
    return g_err.c_str();
}

uint64_t gbo_launch_count(void)
{
    return g_launches.load();
}

gbo_status gbo_selftest_bounded_wait(int64_t limit_ns, double *elapsed_ms)
{
    if (limit_ns <= 0 || limit_ns > 2000000000ll)
        return fail(GBO_ERR_INVALID_ARGUMENT, "wait limit must be in (0, 2 s]");
    if (auto st = ensure_device())
        return st;
    unsigned long long *d = nullptr;
    CUDA_TRY(cudaMalloc(&d, 2 * sizeof(unsigned long long)));
    launch_wait_probe((unsigned long long)limit_ns, d);
    unsigned long long h[2] = {0, 0};
    const cudaError_t e = cudaMemcpy(h, d, sizeof(h), cudaMemcpyDeviceToHost);
    cudaFree(d);
    if (e != cudaSuccess)
        return fail(GBO_ERR_CUDA, std::string("bounded-wait self-test: ") + cudaGetErrorString(e));
    if (elapsed_ms)
        *elapsed_ms = (double)h[1] * 1e-6;
    return h[0] ? fail(GBO_ERR_TIMEOUT, "the probe's wait ran out, as intended") : GBO_OK;
}

gbo_status gbo_device_check(int *sm_count, int *cc_major, int *cc_minor)
{
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0)
    {
        cudaGetLastError();
        return fail(GBO_ERR_NO_DEVICE, "no CUDA device");
    }
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceProp p;
    CUDA_TRY(cudaGetDeviceProperties(&p, dev));
    if (sm_count)
        *sm_count = p.multiProcessorCount;
    if (cc_major)
        *cc_major = p.major;
    if (cc_minor)
        *cc_minor = p.minor;
    return ensure_device();
}

// ---------------------------------------------------------------- spaces
gbo_status gbo_space_create(int kind, int dim, const double *low, const double *high, double param, double lvs,
                            double lvs_fraction, unsigned factor, gbo_space **out)
{
    if (!out)
        return fail(GBO_ERR_INVALID_ARGUMENT, "out is NULL");
    if (kind < GBO_SPACE_REAL_VECTOR || kind > GBO_SPACE_WRAP_L2)
        return fail(GBO_ERR_INVALID_ARGUMENT, "unknown space kind");
    if (dim < 1 || dim > GBO_MAXD)
        return fail(dim > GBO_MAXD ? GBO_ERR_UNSUPPORTED : GBO_ERR_INVALID_ARGUMENT, "dimension must be 1..16");
    if (kind == GBO_SPACE_SO2 && dim != 1)
        return fail(GBO_ERR_INVALID_ARGUMENT, "SO2 has dimension 1");
    if (kind == GBO_SPACE_REAL_VECTOR && (!low || !high))
        return fail(GBO_ERR_INVALID_ARGUMENT, "RealVector bounds required");
    if (factor < 1)
        return fail(GBO_ERR_INVALID_ARGUMENT,
                    "The multiplicative factor for the valid segment count between two states must be strictly positive");
    auto *s = new gbo_space();
    s->sp.kind = kind;
    s->sp.dim = dim;
    s->sp.factor = factor;
    s->sp.link = param;
    for (int d = 0; d < dim; ++d)
    {
        if (kind == GBO_SPACE_REAL_VECTOR)
        {
            if (!(low[d] <= high[d]))
            {
                delete s;
                return fail(GBO_ERR_INVALID_ARGUMENT, "lower bound above upper bound");
            }
            s->sp.low[d] = low[d];
            s->sp.high[d] = high[d];
        }
        else
        {
            s->sp.low[d] = -kPiH;
            s->sp.high[d] = kPiH;
        }
    }
    // StateSpace::setup (StateSpace.cpp:237-249) with the kind's getMaximumExtent
    double e = 0.0;
    if (kind == GBO_SPACE_SO2)
        e = kPiH;
    else
    {
        for (int d = 0; d < dim; ++d)
        {
            const double r = kind == GBO_SPACE_WRAP_L2 ? kPiH : s->sp.high[d] - s->sp.low[d];
            e += r * r;
        }
        e = std::sqrt(e);
    }
    s->extent = e;
    if (lvs <= 0.0)
    {
        const double eps = 2.220446049250313e-16;
        if (lvs_fraction < eps || lvs_fraction > 1.0 - eps)
        {
            delete s;
            return fail(GBO_ERR_INVALID_ARGUMENT, "The fraction of the extent must be larger than 0 and less than 1");
        }
        lvs = e * lvs_fraction;
    }
    if (!(lvs >= 2.220446049250313e-16))
    {
        delete s;
        return fail(GBO_ERR_INVALID_ARGUMENT, "The longest valid segment must be positive.");
    }
    s->sp.lvs = lvs;
    *out = s;
    return GBO_OK;
}

gbo_status gbo_space_destroy(gbo_space *s)
{
    delete s;
    return GBO_OK;
}

gbo_status gbo_space_info(const gbo_space *s, double *max_extent, double *lvs)
{
    if (!s)
        return fail(GBO_ERR_INVALID_ARGUMENT, "space is NULL");
    if (max_extent)
        *max_extent = s->extent;
    if (lvs)
        *lvs = s->sp.lvs;
    return GBO_OK;
}

gbo_status gbo_space_distance(const gbo_space *s, const double *a, const double *b, int64_t n, int64_t ld, int layout,
                              double *out, gbo_stream stream)
{
    if (!s || (n > 0 && (!a || !b || !out)) || n < 0 || !valid_layout(layout, n, ld, s->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad distance arguments");
    if (auto st = ensure_device())
        return st;
    launch_distance(lcfg(stream), s->sp, make_view(a, ld, layout), make_view(b, ld, layout), n, out);
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_space_interpolate(const gbo_space *s, const double *a, const double *b, const double *t, int64_t n,
                                 int64_t ld, int layout, double *out, gbo_stream stream)
{
    if (!s || (n > 0 && (!a || !b || !t || !out)) || n < 0 || !valid_layout(layout, n, ld, s->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad interpolate arguments");
    if (auto st = ensure_device())
        return st;
    StatesView ov = make_view(out, ld, layout);
    launch_interpolate(lcfg(stream), s->sp, make_view(a, ld, layout), make_view(b, ld, layout), t, n,
                       MutStatesView{out, ov.si, ov.sd});
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_get_motion_states(const gbo_space *s, const double *s1, const double *s2, int64_t n, int64_t ld,
                                 int layout, unsigned count, int endpoints, double *out, int64_t out_ld,
                                 gbo_stream stream)
{
    const int64_t m = endpoints ? (int64_t)count + 2 : (int64_t)count;
    if (!s || n < 0 || (n > 0 && (!s1 || !s2 || (m > 0 && !out))) || !valid_layout(layout, n, ld, s->sp.dim) ||
        !valid_layout(layout, n * m, out_ld, s->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad getMotionStates arguments");
    if (n == 0 || m == 0)
        return GBO_OK;
    if (auto st = ensure_device())
        return st;
    StatesView ov = make_view(out, out_ld, layout);
    launch_motion_states(lcfg(stream), s->sp, make_view(s1, ld, layout), make_view(s2, ld, layout), n, count,
                         endpoints ? 1 : 0, MutStatesView{out, ov.si, ov.sd});
    CHECK_LAUNCH();
    return GBO_OK;
}

// ---------------------------------------------------------------- checkers
gbo_status gbo_checker_create(const gbo_space *space, int kind, const double *world, int64_t n_world,
                              const double *dh, int n_joints, int spheres_per_link, double sphere_radius,
                              gbo_checker **out)
{
    if (!space || !out)
        return fail(GBO_ERR_INVALID_ARGUMENT, "space/out is NULL");
    if (kind < GBO_CHECK_ALL_VALID || kind > GBO_CHECK_DH_BOXES)
        return fail(GBO_ERR_INVALID_ARGUMENT, "unknown checker kind");
    // boxes use the DH sphere-arm kernels with a box narrow phase (WorldArgs::boxes)
    const bool boxes = kind == GBO_CHECK_DH_BOXES;
    const int stride = boxes ? 6 : 4;
    if (n_world < 0 || (n_world > 0 && !world) || n_world > (1 << 24))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad world");
    const SpaceParams &sp = space->sp;
    if (kind == GBO_CHECK_CIRCLES && sp.dim != 2)
        return fail(GBO_ERR_INVALID_ARGUMENT, "the circle checker needs a 2-D space");
    if (kind == GBO_CHECK_CHAIN_SEGMENTS && sp.kind != GBO_SPACE_KINEMATIC_CHAIN)
        return fail(GBO_ERR_INVALID_ARGUMENT, "the chain checker needs a kinematic-chain space");
    if ((kind == GBO_CHECK_DH_SPHERES || boxes) &&
        (!dh || n_joints < 1 || n_joints > 8 || n_joints != sp.dim || spheres_per_link < 1 || sphere_radius < 0))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad DH arm (1..8 joints = space dimension)");
    if (auto st = ensure_device())
        return st;
    auto *c = new gbo_checker();
    c->sp = sp;
    c->kind = kind;
    WorldArgs &wa = c->wa;
    wa.kind = boxes ? GBO_CHECK_DH_SPHERES : kind;
    wa.boxes = boxes ? 1 : 0;
    wa.n = (int)n_world;
    wa.inv_lvs32 = (float)(1.0 / sp.lvs);
    auto cleanup = [&](gbo_status s) {
        delete c;
        return s;
    };
    if (c->ctr.init() != GBO_OK)
        return cleanup(GBO_ERR_OUT_OF_MEMORY);
    std::vector<double> w64;
    if (kind == GBO_CHECK_CIRCLES)
    {
        for (int64_t i = 0; i < n_world; ++i)
        {
            w64.push_back(world[3 * i]);
            w64.push_back(world[3 * i + 1]);
            w64.push_back(world[3 * i + 2] * world[3 * i + 2]);  // circles2D.h:51 r2_ = r * r
        }
    }
    else if (kind != GBO_CHECK_ALL_VALID)
        w64.assign(world, world + stride * n_world);
    size_t b64 = pad16(w64.size() * sizeof(double));
    if (b64)
    {
        if (cudaMalloc(&c->d64, b64) != cudaSuccess)
            return cleanup(fail(GBO_ERR_OUT_OF_MEMORY, "world allocation failed"));
        cudaMemset(c->d64, 0, b64);
        cudaMemcpy(c->d64, w64.data(), w64.size() * sizeof(double), cudaMemcpyHostToDevice);
    }
    wa.data64 = c->d64;
    wa.bytes64 = (unsigned)b64;
    wa.stage64 = (b64 > 0 && b64 <= 96 * 1024 && wa.kind != GBO_CHECK_DH_SPHERES) ? 1 : 0;
    if (kind == GBO_CHECK_CHAIN_SEGMENTS)
    {
        std::vector<ChainSegF32> segs;
        chain_bounds(sp, world, (int)n_world, wa.guard, segs, wa.e_dist);
        // trig hazard bound of the FP64 forms: joint k's position is a sum of k link vectors cos/sin * L;
        // the device's sines and cosines (CUDA's FP64 sincos, within 2 ulps, or the correctly rounded
        // ones) and the C library's (within 1 ulp) differ by at most 4 ulps (<= 4 * 2^-52), which moves
        // each product by at most 4 L 2^-52 plus its rounding, and each partial sum by its rounding
        // (2^-53 of the reach); safety factor 2
        {
            const double L = sp.link, reach = sp.dim * std::fabs(L) + 0.001;
            wa.hz_pos = 2.0 * (sp.dim + 1) * (std::fabs(L) * 0x1p-50 + std::fabs(L) * 0x1p-53 + reach * 0x1p-53);
        }
        size_t b32 = pad16(segs.size() * sizeof(ChainSegF32));
        if (b32)
        {
            if (cudaMalloc(&c->d32, b32) != cudaSuccess)
                return cleanup(fail(GBO_ERR_OUT_OF_MEMORY, "world allocation failed"));
            cudaMemcpy(c->d32, segs.data(), segs.size() * sizeof(ChainSegF32), cudaMemcpyHostToDevice);
        }
        wa.data32 = c->d32;
        wa.bytes32 = (unsigned)b32;
        wa.stage32 = b32 > 0 && b32 <= 96 * 1024;
        if (!wa.stage32 && b32)
            return cleanup(fail(GBO_ERR_UNSUPPORTED, "segment world too large for shared memory"));
        if (b32 && sp.dim <= 31)
            if (auto st = order_chain_tests(c))
                return cleanup(st);
    }
    if (wa.kind == GBO_CHECK_DH_SPHERES)
    {
        DHArm &arm = wa.arm;
        arm.joints = n_joints;
        arm.spl = spheres_per_link;
        arm.rs = sphere_radius;
        for (int i = 0; i < n_joints; ++i)
        {
            arm.a[i] = dh[3 * i];
            arm.d[i] = dh[3 * i + 1];
            const int code = (int)dh[3 * i + 2];
            if (code < -1 || code > 1)
                return cleanup(fail(GBO_ERR_INVALID_ARGUMENT, "alpha code must be -1, 0 or +1"));
            arm.ca[i] = code == 0 ? 1.f : 0.f;
            arm.sa[i] = code == 0 ? 0.f : (float)code;
            arm.af[i] = (float)arm.a[i];
            arm.dfl[i] = (float)arm.d[i];
        }
        // FP32 obstacles (rows as given)
        std::vector<float> s32(stride * n_world);
        double rmax = 0.0;
        for (int64_t i = 0; i < stride * n_world; ++i)
            s32[i] = (float)world[i];
        for (int64_t i = 0; i < n_world; ++i)
            rmax = std::max(rmax, boxes ? 0.0 : world[4 * i + 3]);
        size_t b32 = pad16(s32.size() * sizeof(float));
        if (b32)
        {
            if (cudaMalloc(&c->d32, b32) != cudaSuccess)
                return cleanup(fail(GBO_ERR_OUT_OF_MEMORY, "world allocation failed"));
            cudaMemcpy(c->d32, s32.data(), s32.size() * sizeof(float), cudaMemcpyHostToDevice);
        }
        wa.data32 = c->d32;
        wa.bytes32 = (unsigned)b32;
        wa.stage32 = 0;  // the FP32 narrow phase reads the spheres listed in the grid cells (cell_items4)
        // FK error bound in FP32 (spectral-norm propagation): |dR_k| <= k (2 eps_t + 16u),
        // |dp| <= sum_k (|dR_k| |pA| + |pA| (eps_t + u) + 4u (|p| + |pA|)); centres add 3u|p|.
        // angles: |q| <= qmax (the space's bounds; states beyond them are re-checked in FP64), rounded to
        // FP32 (u |q|, +1% for the float-float interpolation), sincosf within 2 ulp
        double qmax = kPiH;
        if (sp.kind == GBO_SPACE_REAL_VECTOR)
        {
            qmax = 0.0;
            for (int d = 0; d < sp.dim; ++d)
                qmax = std::max(qmax, std::max(std::fabs(sp.low[d]), std::fabs(sp.high[d])));
        }
        wa.dh_qmax = (float)qmax;
        const double u = kU32, eps_t = u * qmax * 1.01 + 2.0 * std::ldexp(1.0, -23);
        double dR = 0.0, dp = 0.0, reach = 0.0;
        for (int i = 0; i < n_joints; ++i)
        {
            const double pa = std::sqrt(arm.a[i] * arm.a[i] + arm.d[i] * arm.d[i]);
            reach += pa;
            dp += dR * pa + pa * (eps_t + u) * 2.0 + 4.0 * u * (reach + pa);
            dR += 2.0 * eps_t + 16.0 * u;
        }
        const double dc = (dp + 3.0 * u * reach) * std::sqrt(3.0);  // Euclidean centre error
        // the same propagation for the FP64 forms when every sine and cosine moves by 4 ulps (4 * 2^-52,
        // CUDA's FP64 sincos against the C library's): the trig hazard bound of a sphere centre
        // (safety factor 2)
        {
            const double u64 = 0x1p-53, et = 0x1p-50;
            double dR64 = 0.0, dp64 = 0.0, reach64 = 0.0;
            for (int i = 0; i < n_joints; ++i)
            {
                const double pa = std::sqrt(arm.a[i] * arm.a[i] + arm.d[i] * arm.d[i]);
                reach64 += pa;
                dp64 += dR64 * pa + pa * (et + u64) * 2.0 + 4.0 * u64 * (reach64 + pa);
                dR64 += 2.0 * et + 16.0 * u64;
            }
            wa.hz_dh = 2.0 * (dp64 + 3.0 * u64 * reach64) * std::sqrt(3.0);
        }
        // The grid below lists an obstacle in every cell within rs (+ r) + margin of it, so a listed
        // obstacle lies within D = rs (+ rmax) + margin + one cell diagonal of the robot sphere centre:
        // |d^2 - d_ref^2| <= 2|d| dc + dc^2 (+ rounding of d^2, rr^2). Boxes: the distance of a point
        // from a box is 1-Lipschitz per axis; each axis adds the roundings of |c - centre| - half
        // extent and of the FP32 box (<= 40u for coordinates below 4).
        const double margin = 1e-3;
        const int G = 64;
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        // world obstacle i: centre o(i, r), half extent h(i, r) (boxes) or radius (spheres), and the
        // reach added around it (rs + margin for boxes, rs + r + margin for spheres)
        auto o_of = [&](int64_t i, int r) { return world[stride * i + r]; };
        auto half = [&](int64_t i, int r) { return boxes ? world[stride * i + 3 + r] : 0.0; };
        auto grow = [&](int64_t i) { return (boxes ? 0.0 : world[4 * i + 3]) + sphere_radius + margin; };
        for (int64_t i = 0; i < n_world; ++i)
            for (int r = 0; r < 3; ++r)
            {
                const double ext = grow(i) + half(i, r);
                lo[r] = std::min(lo[r], o_of(i, r) - ext);
                hi[r] = std::max(hi[r], o_of(i, r) + ext);
            }
        if (n_world == 0)
            for (int r = 0; r < 3; ++r)
            {
                lo[r] = -1;
                hi[r] = 1;
            }
        double diag2 = 0.0;
        for (int r = 0; r < 3; ++r)
        {
            lo[r] -= margin;
            hi[r] += margin;
            diag2 += ((hi[r] - lo[r]) / G) * ((hi[r] - lo[r]) / G);
        }
        const double D = 1.01 * (sphere_radius + rmax + margin + std::sqrt(diag2));
        const double dcx = boxes ? dc + 40.0 * u * std::sqrt(3.0) : dc;
        const double E = 2.0 * D * dcx + dcx * dcx + 8.0 * u * D * D + 4.0 * u * (D * D);
        wa.dh_e = (float)(2.0 * E);
        // uniform 64^3 grid: a sphere is listed in every cell whose box lies within rs + ro + margin of its
        // centre (exact sphere-box distance), so the cell holding a robot sphere centre lists every world
        // sphere that can touch it; cells store the index (FP64 path) and the FP32 sphere itself.
        double inv[3], cell[3];
        for (int r = 0; r < 3; ++r)
        {
            inv[r] = G / (hi[r] - lo[r]);
            cell[r] = (hi[r] - lo[r]) / G;
            wa.glo64[r] = lo[r];
            wa.ginv64[r] = inv[r];
            wa.glo[r] = (float)lo[r];
            wa.ginv[r] = (float)inv[r];
        }
        const size_t ncell = (size_t)G * G * G;
        std::vector<int> start(ncell + 1, 0);
        auto visit = [&](int64_t i, auto &&emit) {
            const double ext = grow(i);
            int c0[3], c1[3];
            for (int r = 0; r < 3; ++r)
            {
                c0[r] = std::max(0, (int)std::floor((o_of(i, r) - half(i, r) - ext - lo[r]) * inv[r]) - 1);
                c1[r] = std::min(G - 1, (int)std::floor((o_of(i, r) + half(i, r) + ext - lo[r]) * inv[r]) + 1);
            }
            for (int x = c0[0]; x <= c1[0]; ++x)
                for (int y = c0[1]; y <= c1[1]; ++y)
                    for (int z = c0[2]; z <= c1[2]; ++z)
                    {
                        const int ix[3] = {x, y, z};
                        double d2 = 0.0;
                        for (int r = 0; r < 3; ++r)
                        {
                            const double b0 = lo[r] + ix[r] * cell[r], b1 = b0 + cell[r];
                            const double o0 = o_of(i, r) - half(i, r), o1 = o_of(i, r) + half(i, r);
                            const double g = o1 < b0 ? b0 - o1 : (o0 > b1 ? o0 - b1 : 0.0);
                            d2 += g * g;
                        }
                        if (d2 <= ext * ext * (1.0 + 1e-9))
                            emit(((size_t)x * G + y) * G + z);
                    }
        };
        for (int64_t i = 0; i < n_world; ++i)
            visit(i, [&](size_t k) { start[k + 1]++; });
        for (size_t k = 0; k < ncell; ++k)
            start[k + 1] += start[k];
        std::vector<int> fill(start.begin(), start.end() - 1), items(std::max(1, start[ncell]));
        const int per_item = boxes ? 8 : 4;
        std::vector<float> items4(per_item * items.size(), 0.f);
        for (int64_t i = 0; i < n_world; ++i)
            visit(i, [&](size_t k) {
                const int pos = fill[k]++;
                items[pos] = (int)i;
                for (int r = 0; r < stride; ++r)
                    items4[per_item * (size_t)pos + r] = (float)world[stride * i + r];
            });
        if (cudaMalloc(&c->cell_start, start.size() * sizeof(int)) != cudaSuccess ||
            cudaMalloc(&c->cell_items, items.size() * sizeof(int)) != cudaSuccess ||
            cudaMalloc(&c->cell_items4, items4.size() * sizeof(float)) != cudaSuccess)
            return cleanup(fail(GBO_ERR_OUT_OF_MEMORY, "grid allocation failed"));
        cudaMemcpy(c->cell_start, start.data(), start.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(c->cell_items, items.data(), items.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(c->cell_items4, items4.data(), items4.size() * sizeof(float), cudaMemcpyHostToDevice);
        wa.cell_items4 = (const float4 *)c->cell_items4;
        wa.cell_start = c->cell_start;
        wa.cell_items = c->cell_items;
        wa.grid_n = G;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        return cleanup(fail(GBO_ERR_CUDA, cudaGetErrorString(e)));
    if (cudaStreamCreateWithFlags(&c->host_stream, cudaStreamNonBlocking) != cudaSuccess)
        return cleanup(fail(GBO_ERR_CUDA, "stream creation failed"));
    *out = c;
    return GBO_OK;
}

gbo_status gbo_checker_destroy(gbo_checker *c)
{
    if (c)
        cudaDeviceSynchronize();
    delete c;
    return GBO_OK;
}

gbo_status gbo_checker_set_precision(gbo_checker *c, int precision)
{
    if (!c || (precision != GBO_PRECISION_FP64 && precision != GBO_PRECISION_FP32_GUARDED))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad precision");
    c->precision = precision;
    return GBO_OK;
}

gbo_status gbo_checker_stats(const gbo_checker *c, uint64_t *evaluated, uint64_t *rechecked)
{
    if (!c)
        return fail(GBO_ERR_INVALID_ARGUMENT, "checker is NULL");
    RunCounters h{};
    CUDA_TRY(cudaMemcpy(&h, c->ctr.dev + c->ctr.last, sizeof(h), cudaMemcpyDeviceToHost));
    if (evaluated)
        *evaluated = h.evaluated;
    if (rechecked)
        *rechecked = h.rechecked;
    if (h.timeout)
        return fail(GBO_ERR_TIMEOUT, "a device-side wait ran out in the last call");
    if (h.error)
        return fail(GBO_ERR_CUDA, "a kernel refused to stage its world into shared memory in the last call");
    return GBO_OK;
}

gbo_status gbo_checker_counters(const gbo_checker *c, uint64_t *evaluated, uint64_t *rechecked, uint64_t *hazards)
{
    if (!c)
        return fail(GBO_ERR_INVALID_ARGUMENT, "checker is NULL");
    RunCounters h{};
    CUDA_TRY(cudaMemcpy(&h, c->ctr.dev + c->ctr.last, sizeof(h), cudaMemcpyDeviceToHost));
    if (evaluated)
        *evaluated = h.evaluated;
    if (rechecked)
        *rechecked = h.rechecked;
    if (hazards)
        *hazards = h.hazards;
    return GBO_OK;
}

gbo_status gbo_is_valid(gbo_checker *c, const double *states, int64_t n, int64_t ld, int layout, uint8_t *out,
                        gbo_stream stream)
{
    Trace trace("gbo_is_valid");
    if (!c || n < 0 || (n > 0 && (!states || !out)) || !valid_layout(layout, n, ld, c->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad isValid arguments");
    if (n == 0)
        return GBO_OK;
    LaunchCfg lc = lcfg(stream);
    RunCounters *ctr = c->ctr.take(lc.stream);
    launch_validity(lc, c->precision, c->sp, c->wa, make_view(states, ld, layout), n, out, ctr);
    CHECK_LAUNCH();
    return GBO_OK;
}

static gbo_status motion_impl(gbo_checker *c, const double *s1, const double *s2, int64_t n, int64_t ld, int layout,
                              int schedule, uint8_t *ok, int32_t *first_j, int32_t *nd, cudaStream_t stream)
{
    LaunchCfg lc = lcfg(stream);
    RunCounters *ctr = c->ctr.take(lc.stream);
    launch_motion(lc, c->precision, schedule, c->sp, c->wa, make_view(s1, ld, layout), make_view(s2, ld, layout), n,
                  ok, first_j, nd, ctr);
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_check_motion(gbo_checker *c, const double *s1, const double *s2, int64_t n, int64_t ld, int layout,
                            int schedule, uint8_t *ok, int32_t *first_j, int32_t *nd, gbo_stream stream)
{
    Trace trace("gbo_check_motion");
    if (!c || n < 0 || (n > 0 && (!s1 || !s2 || !ok)) || !valid_layout(layout, n, ld, c->sp.dim) ||
        schedule < GBO_SCHEDULE_PLAIN || schedule > GBO_SCHEDULE_AUTO)
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad checkMotion arguments");
    if (n == 0)
        return GBO_OK;
    if (schedule == GBO_SCHEDULE_AUTO)
    {
        std::lock_guard<std::mutex> lk(c->tune_mu);
        if (c->tuned_schedule < 0)
        {
            // autotune: time both persistent schedules on (a prefix of) this batch
            const int64_t m = std::min<int64_t>(n, 65536);
            cudaEvent_t e0, e1;
            cudaEventCreate(&e0);
            cudaEventCreate(&e1);
            float best = 1e30f;
            int pick = GBO_SCHEDULE_TILE;
            for (int sch : {GBO_SCHEDULE_TILE, GBO_SCHEDULE_WARP})
            {
                for (int rep = 0; rep < 2; ++rep)
                {
                    cudaEventRecord(e0, (cudaStream_t)stream);
                    if (auto st = motion_impl(c, s1, s2, m, ld, layout, sch, ok, first_j, nd, (cudaStream_t)stream))
                        return st;
                    cudaEventRecord(e1, (cudaStream_t)stream);
                    cudaEventSynchronize(e1);
                    float ms = 0.f;
                    cudaEventElapsedTime(&ms, e0, e1);
                    if (rep == 1 && ms < best)
                    {
                        best = ms;
                        pick = sch;
                    }
                }
            }
            cudaEventDestroy(e0);
            cudaEventDestroy(e1);
            c->tuned_schedule = pick;
        }
        schedule = c->tuned_schedule;
    }
    return motion_impl(c, s1, s2, n, ld, layout, schedule, ok, first_j, nd, (cudaStream_t)stream);
}

gbo_status gbo_last_valid(const gbo_space *s, const double *s1, const double *s2, const int32_t *first_j,
                          const int32_t *nd, int64_t n, int64_t ld, int layout, double *last_t, double *last_state,
                          gbo_stream stream)
{
    if (!s || n < 0 || (n > 0 && (!s1 || !s2 || !first_j || !nd)) || !valid_layout(layout, n, ld, s->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad lastValid arguments");
    StatesView ov = make_view(last_state, ld, layout);
    launch_last_valid(lcfg(stream), s->sp, make_view(s1, ld, layout), make_view(s2, ld, layout), first_j, nd, n,
                      last_t, MutStatesView{last_state, ov.si, ov.sd});
    CHECK_LAUNCH();
    return GBO_OK;
}

__global__ void finish_states_chain(const unsigned long long *first, int64_t count, uint8_t *ok, int64_t *fi)
{
    const unsigned long long f = *first;
    const bool good = f >= (unsigned long long)count;
    *ok = good ? 1 : 0;
    if (fi)
        *fi = good ? -1 : (int64_t)f;
}

gbo_status gbo_check_motion_states(gbo_checker *c, const double *states, int64_t count, int64_t ld, int layout,
                                   uint8_t *ok, int64_t *first_invalid, gbo_stream stream)
{
    if (!c || count < 0 || (count > 0 && !states) || !ok || !valid_layout(layout, count, ld, c->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad checkMotion(states) arguments");
    LaunchCfg lc = lcfg(stream);
    RunCounters *ctr = c->ctr.take(lc.stream);
    unsigned long long *first = &ctr->queue;  // slot's queue word doubles as the running minimum
    CUDA_TRY(cudaMemsetAsync(first, 0xff, sizeof(unsigned long long), lc.stream));
    if (count > 0)
        launch_states_chain(lc, c->sp, c->wa, make_view(states, ld, layout), count, first, ctr);
    finish_states_chain<<<1, 1, 0, lc.stream>>>(first, count, ok, first_invalid);
    note_launch();
    CHECK_LAUNCH();
    return GBO_OK;
}

// Device address of a page-locked host array (cudaMallocHost / cudaHostRegister), or null for
// pageable or device memory. Kernels read and write such arrays in place over the coherent host
// link, so the transfer overlaps with the work inside the launch instead of preceding it.
static void *mapped_host(const void *p)
{
    cudaPointerAttributes a{};
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

gbo_status gbo_is_valid_host(gbo_checker *c, const double *states, int64_t n, uint8_t *out)
{
    Trace trace("gbo_is_valid_host");
    if (!c || n < 0 || (n > 0 && (!states || !out)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad isValid arguments");
    if (n == 0)
        return GBO_OK;
    std::lock_guard<std::mutex> lk(c->mu);
    const size_t bin = (size_t)n * c->sp.dim * sizeof(double);
    const double *din = (const double *)mapped_host(states);
    uint8_t *dout = (uint8_t *)mapped_host(out);
    if (!din)
    {
        if (auto st = c->pin_in.reserve(bin))
            return st;
        if (auto st = c->dev_in.reserve(bin, c->host_stream))
            return st;
        std::memcpy(c->pin_in.p, states, bin);
        CUDA_TRY(cudaMemcpyAsync(c->dev_in.p, c->pin_in.p, bin, cudaMemcpyHostToDevice, c->host_stream));
        din = (const double *)c->dev_in.p;
    }
    if (!dout)
    {
        if (auto st = c->dev_out.reserve((size_t)n, c->host_stream))
            return st;
    }
    if (auto st = gbo_is_valid(c, din, n, c->sp.dim, GBO_LAYOUT_AOS, dout ? dout : (uint8_t *)c->dev_out.p,
                               c->host_stream))
        return st;
    if (!dout)
        CUDA_TRY(cudaMemcpyAsync(out, c->dev_out.p, (size_t)n, cudaMemcpyDeviceToHost, c->host_stream));
    CUDA_TRY(cudaStreamSynchronize(c->host_stream));
    return GBO_OK;
}

gbo_status gbo_check_motion_host(gbo_checker *c, const double *s1, const double *s2, int64_t n, uint8_t *ok,
                                 double *last_t, double *last_state)
{
    Trace trace("gbo_check_motion_host");
    if (!c || n < 0 || (n > 0 && (!s1 || !s2 || !ok)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad checkMotion arguments");
    if (n == 0)
        return GBO_OK;
    std::lock_guard<std::mutex> lk(c->mu);
    const int dim = c->sp.dim;
    const size_t bst = (size_t)n * dim * sizeof(double);
    // page-locked arrays are used in place (mapped_host); the others go through device buffers
    const double *m1 = (const double *)mapped_host(s1), *m2 = (const double *)mapped_host(s2);
    const bool in_place = m1 && m2;
    uint8_t *mok = (uint8_t *)mapped_host(ok);
    double *mlt = (double *)mapped_host(last_t), *mls = (double *)mapped_host(last_state);
    // device layout: [s1 | s2 (copy path)] | first_j | nd | ok | last_t | last_state
    const size_t off_fj = in_place ? 0 : 2 * bst, off_nd = off_fj + 4 * (size_t)n, off_ok = off_nd + 4 * (size_t)n;
    const size_t off_lt = pad16(off_ok + (size_t)n), off_ls = off_lt + 8 * (size_t)n, total = off_ls + bst;
    if (auto st = c->dev_in.reserve(total, c->host_stream))
        return st;
    char *d = (char *)c->dev_in.p;
    if (!in_place)
    {
        // straight from the caller's arrays to the device (no staging copy on the host)
        CUDA_TRY(cudaMemcpyAsync(d, s1, bst, cudaMemcpyHostToDevice, c->host_stream));
        CUDA_TRY(cudaMemcpyAsync(d + bst, s2, bst, cudaMemcpyHostToDevice, c->host_stream));
        m1 = (const double *)d;
        m2 = (const double *)(d + bst);
    }
    uint8_t *okd = mok ? mok : (uint8_t *)(d + off_ok);
    int32_t *fj = (int32_t *)(d + off_fj), *ndv = (int32_t *)(d + off_nd);
    const int sched = c->precision == GBO_PRECISION_FP64 ? GBO_SCHEDULE_PLAIN : GBO_SCHEDULE_AUTO;
    if (auto st = gbo_check_motion(c, m1, m2, n, dim, GBO_LAYOUT_AOS, sched, okd, fj, ndv, c->host_stream))
        return st;
    double *ltd = mlt ? mlt : (double *)(d + off_lt), *lsd = mls ? mls : (double *)(d + off_ls);
    if (last_t || last_state)
    {
        launch_last_valid(lcfg(c->host_stream), c->sp, make_view(m1, dim, GBO_LAYOUT_AOS),
                          make_view(m2, dim, GBO_LAYOUT_AOS), fj, ndv, n, ltd,
                          MutStatesView{last_state ? lsd : nullptr, dim, 1});
        CHECK_LAUNCH();
    }
    if (!mok)
        CUDA_TRY(cudaMemcpyAsync(ok, okd, (size_t)n, cudaMemcpyDeviceToHost, c->host_stream));
    if (last_t && !mlt)
        CUDA_TRY(cudaMemcpyAsync(last_t, ltd, 8 * (size_t)n, cudaMemcpyDeviceToHost, c->host_stream));
    if (last_state && !mls)
        CUDA_TRY(cudaMemcpyAsync(last_state, lsd, bst, cudaMemcpyDeviceToHost, c->host_stream));
    CUDA_TRY(cudaStreamSynchronize(c->host_stream));
    return GBO_OK;
}

// ---------------------------------------------------------------- samplers
gbo_status gbo_sampler_create(const gbo_space *space, uint32_t local_seed, gbo_sampler **out)
{
    if (!space || !out)
        return fail(GBO_ERR_INVALID_ARGUMENT, "space/out is NULL");
    if (auto st = ensure_device())
        return st;
    auto *s = new gbo_sampler();
    s->sp = space->sp;
    // mt19937 seeding (std::mersenne_twister_engine::seed): x0 = seed, x_i = f * (x_{i-1} ^ (x_{i-1} >> 30)) + i
    SamplerState h{};
    h.mt[0] = local_seed;
    for (unsigned i = 1; i < 624; ++i)
        h.mt[i] = 1812433253u * (h.mt[i - 1] ^ (h.mt[i - 1] >> 30)) + i;
    h.pos = 624;
    if (cudaMalloc(&s->st, sizeof(SamplerState)) != cudaSuccess)
    {
        delete s;
        return fail(GBO_ERR_OUT_OF_MEMORY, "sampler allocation failed");
    }
    cudaMemcpy(s->st, &h, sizeof(h), cudaMemcpyHostToDevice);
    if (cudaStreamCreateWithFlags(&s->host_stream, cudaStreamNonBlocking) != cudaSuccess)
    {
        delete s;
        return fail(GBO_ERR_CUDA, "stream creation failed");
    }
    *out = s;
    return GBO_OK;
}

gbo_status gbo_sampler_destroy(gbo_sampler *s)
{
    delete s;
    return GBO_OK;
}

// Word-stream scratch of a sampling call of n states (stream-ordered growth): 2 words per value, at
// most 16M words (larger calls run in chunks).
static gbo_status sampler_words(gbo_sampler *s, int64_t n, gbo_stream stream, int64_t &cap)
{
    cap = std::max<int64_t>(2, std::min<int64_t>(2 * n * s->sp.dim, (int64_t)1 << 24));
    return s->words.reserve((size_t)cap * sizeof(unsigned), (cudaStream_t)stream);
}

// sampleUniform / sampleUniformNear over n states. Calls of at least 2^18 stream words run on segments
// of the stream generated side by side from jump-ahead windows (segments of L = 2^m words, m >= 15, the
// smallest m that keeps them at most 160); smaller calls run the recurrence on one CTA.
static gbo_status sample_uniform_call(gbo_sampler *s, const double *near, StatesView nearv, double distance,
                                      int64_t n, MutStatesView out, gbo_stream stream)
{
    const int64_t values = n * s->sp.dim, W = 2 * values;
    if (W >= ((int64_t)1 << 18) && values < ((int64_t)1 << 31) && mt_field_ready())
    {
        int m = 15;
        while (m < 24 && W > ((int64_t)160 << m))
            ++m;
        const int64_t L = (int64_t)1 << m;
        const int nseg = (int)((W + L - 1) / L);
        const uint32_t *polys = nullptr;
        if (nseg > 1)
            if (auto st = mt_jump_table((uint64_t)L, nseg - 1, &polys))
                return fail(st, "jump-ahead polynomials could not be prepared");
        if (auto st = s->words.reserve((size_t)sample_jump_words(nseg, W) * sizeof(unsigned), (cudaStream_t)stream))
            return st;
        launch_sample_uniform_jump(lcfg(stream), s->st, s->sp, near, nearv, distance, n, out, (unsigned *)s->words.p,
                                   polys, L, nseg);
        CHECK_LAUNCH();
        return GBO_OK;
    }
    int64_t cap = 0;
    if (auto st = sampler_words(s, n, stream, cap))
        return st;
    launch_sample_uniform(lcfg(stream), s->st, s->sp, near, nearv, distance, n, out, (unsigned *)s->words.p, cap);
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_sample_uniform(gbo_sampler *s, int64_t n, double *out, int64_t ld, int layout, gbo_stream stream)
{
    Trace trace("gbo_sample_uniform");
    if (!s || n < 0 || (n > 0 && !out) || !valid_layout(layout, n, ld, s->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sampleUniform arguments");
    StatesView ov = make_view(out, ld, layout);
    return sample_uniform_call(s, nullptr, StatesView{}, 0.0, n, MutStatesView{out, ov.si, ov.sd}, stream);
}

gbo_status gbo_sample_uniform_near(gbo_sampler *s, const double *near, double distance, int64_t n, int64_t ld,
                                   int layout, double *out, gbo_stream stream)
{
    if (!s || n < 0 || (n > 0 && (!out || !near)) || !valid_layout(layout, n, ld, s->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sampleUniformNear arguments");
    StatesView ov = make_view(out, ld, layout);
    return sample_uniform_call(s, near, make_view(near, ld, layout), distance, n, MutStatesView{out, ov.si, ov.sd},
                               stream);
}

// StateSampler::sampleGaussian (StateSampler.h:96-100) for n states, state i drawn around mean row i
// (mean and out share ld and layout). Returns after the call's stream work: the number of candidate
// draws is data dependent and the host reads each chunk's progress.
gbo_status gbo_sample_gaussian(gbo_sampler *s, const double *mean, double stddev, int64_t n, int64_t ld, int layout,
                               double *out, gbo_stream stream)
{
    Trace trace("gbo_sample_gaussian");
    if (!s || n < 0 || (n > 0 && (!out || !mean)) || !valid_layout(layout, n, ld, s->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sampleGaussian arguments");
    const int64_t M = n * s->sp.dim;
    if (M == 0)
        return GBO_OK;
    // raw words for the expected candidates plus a margin and one whole block (capped; larger calls
    // run in several chunks)
    const double mu = (double)((M + 1) / 2) / 0.7853981633974483;
    const int64_t cap = std::min<int64_t>(((int64_t)1 << 25) + 628,
                                          4 * (int64_t)std::ceil(mu + 8.0 * std::sqrt(mu) + 64.0) + 628);
    cudaStream_t st = (cudaStream_t)stream;
    // large chunks draw their candidates' words on jump-ahead segments (segment length chosen as for
    // sampleUniform from the first chunk's words; later chunks are shorter and use fewer segments)
    const int64_t W0 = 4 * ((cap - 624) / 4);  // the most words a chunk draws (4 per candidate)
    const uint32_t *polys = nullptr;
    int64_t L = 0, jump_words = 0;
    if (W0 >= ((int64_t)1 << 18) && mt_field_ready())
    {
        int m = 15;
        while (m < 24 && W0 > ((int64_t)160 << m))
            ++m;
        L = (int64_t)1 << m;
        const int nseg = (int)((W0 + L - 1) / L);
        if (nseg > 1)
            if (auto e = mt_jump_table((uint64_t)L, nseg - 1, &polys))
                return fail(e, "jump-ahead polynomials could not be prepared");
        if (nseg == 1)
            polys = nullptr;
        jump_words = sample_jump_words(nseg, 0);
    }
    const int64_t cap_al = (cap + 3) & ~(int64_t)3;
    if (auto e = s->words.reserve((size_t)(cap_al + jump_words) * sizeof(unsigned), st))
        return e;
    const size_t cnt_bytes = pad16(sizeof(GaussChunk) + sizeof(long long) * (size_t)(cap / 4096 + 2));
    const size_t slots = (size_t)gauss_pair_slots(cap);
    if (auto e = s->gwork.reserve(cnt_bytes + slots * (sizeof(double2) + sizeof(unsigned short) + 2 * sizeof(unsigned)),
                                  st))
        return e;
    double2 *pair = (double2 *)((char *)s->gwork.p + cnt_bytes);
    const StatesView ov = make_view(out, ld, layout);
    const int64_t chunks = launch_sample_gaussian(
        lcfg(st), s->st, s->has_saved, s->sp, make_view(mean, ld, layout), stddev, n, MutStatesView{out, ov.si, ov.sd},
        (unsigned *)s->words.p, cap, (GaussChunk *)s->gwork.p, (long long *)((char *)s->gwork.p + sizeof(GaussChunk)),
        pair, (unsigned short *)(pair + slots), (unsigned *)((unsigned short *)(pair + slots) + slots),
        polys ? (unsigned *)s->words.p + cap_al : nullptr, polys, L);
    if (chunks < 0)
        return fail(GBO_ERR_CUDA, std::string("sampleGaussian: ") + cudaGetErrorString(cudaGetLastError()));
    CHECK_LAUNCH();
    s->has_saved = ((M - (s->has_saved ? 1 : 0)) & 1) != 0;
    return GBO_OK;
}

// UniformValidStateSampler::sample, n calls. A call draws until a valid state or `attempts` draws;
// the stream must end where OMPL's would, so no draw is made that no call consumes. Each round draws
// one state per unresolved call (every such call consumes at least one more), checks them, and walks
// the flags on the host; after 8 rounds the rest is drawn speculatively up to its upper bound
// (attempts per call) from a saved copy of the generator, which is then restored and advanced by
// exactly the draws consumed.
gbo_status gbo_sample_valid(gbo_sampler *s, gbo_checker *c, int64_t n, unsigned attempts, double *out, int64_t ld,
                            int layout, uint8_t *ok, gbo_stream stream)
{
    Trace trace("gbo_sample_valid");
    if (!s || !c || n < 0 || (n > 0 && (!out || !ok)) || !valid_layout(layout, n, ld, s->sp.dim) ||
        c->sp.dim != s->sp.dim)
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sampleValid arguments");
    if (n == 0)
        return GBO_OK;
    const int64_t A = attempts > 0 ? attempts : 1;  // do { ... } while: one draw at least
    const int dim = s->sp.dim;
    cudaStream_t st = (cudaStream_t)stream;
    const StatesView ov = make_view(out, ld, layout);
    const LaunchCfg lc = lcfg(st);
    std::vector<uint8_t> flags, okh;
    std::vector<int64_t> src;
    int64_t done = 0, open = 0;  // calls resolved; draws of the unresolved call so far
    constexpr int64_t kSpeculativeCap = 1ll << 26;
    for (int round = 0; done < n; ++round)
    {
        const int64_t r = n - done;
        const bool spec = round >= 8 && r * A - open <= kSpeculativeCap;
        const int64_t gen = spec ? r * A - open : r;
        double *buf = nullptr;
        uint8_t *fl = nullptr;
        int64_t *idx = nullptr;
        SamplerState *ckpt = nullptr;
        CUDA_TRY(cudaMallocAsync((void **)&buf, (size_t)gen * dim * sizeof(double), st));
        CUDA_TRY(cudaMallocAsync((void **)&fl, (size_t)gen, st));
        CUDA_TRY(cudaMallocAsync((void **)&idx, (size_t)r * sizeof(int64_t), st));
        if (spec)
        {
            CUDA_TRY(cudaMallocAsync((void **)&ckpt, sizeof(SamplerState), st));
            CUDA_TRY(cudaMemcpyAsync(ckpt, s->st, sizeof(SamplerState), cudaMemcpyDeviceToDevice, st));
        }
        if (auto e = gbo_sample_uniform(s, gen, buf, dim, GBO_LAYOUT_AOS, stream))
            return e;
        if (auto e = gbo_is_valid(c, buf, gen, dim, GBO_LAYOUT_AOS, fl, stream))
            return e;
        flags.resize((size_t)gen);
        CUDA_TRY(cudaMemcpyAsync(flags.data(), fl, (size_t)gen, cudaMemcpyDeviceToHost, st));
        CUDA_TRY(cudaStreamSynchronize(st));
        src.clear();
        okh.clear();
        int64_t q = 0;
        while (done + (int64_t)src.size() < n && q < gen)
        {
            ++open;
            if (flags[(size_t)q] || open == A)
            {
                src.push_back(q);
                okh.push_back(flags[(size_t)q] ? 1 : 0);
                open = 0;
            }
            ++q;
        }
        if (spec)
        {
            // back to the saved generator, advanced by exactly the q draws consumed (same values)
            CUDA_TRY(cudaMemcpyAsync(s->st, ckpt, sizeof(SamplerState), cudaMemcpyDeviceToDevice, st));
            if (auto e = gbo_sample_uniform(s, q, buf, dim, GBO_LAYOUT_AOS, stream))
                return e;
        }
        const int64_t m = (int64_t)src.size();
        if (m)
        {
            CUDA_TRY(cudaMemcpyAsync(idx, src.data(), (size_t)m * sizeof(int64_t), cudaMemcpyHostToDevice, st));
            CUDA_TRY(cudaMemcpyAsync(ok + done, okh.data(), (size_t)m, cudaMemcpyHostToDevice, st));
            launch_gather_rows(lc, StatesView{buf, dim, 1}, idx, m, dim,
                               MutStatesView{out + done * ov.si, ov.si, ov.sd});
            CHECK_LAUNCH();
        }
        cudaFreeAsync(buf, st);
        cudaFreeAsync(fl, st);
        cudaFreeAsync(idx, st);
        if (ckpt)
            cudaFreeAsync(ckpt, st);
        CUDA_TRY(cudaStreamSynchronize(st));  // src / okh are reused by the next round
        done += m;
    }
    return GBO_OK;
}

// ---------------------------------------------------------------- nearest neighbours
gbo_status gbo_nn_create(const gbo_space *space, int64_t capacity, gbo_nn **out)
{
    if (!space || !out || capacity < 1)
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad nn arguments");
    if (auto st = ensure_device())
        return st;
    auto *nn = new gbo_nn();
    nn->sp = space->sp;
    nn->cap = capacity;
    nn->F = space->sp.kind == GBO_SPACE_KINEMATIC_CHAIN ? 2 * space->sp.dim : space->sp.dim;
    nn->eps32 = space->sp.kind == GBO_SPACE_KINEMATIC_CHAIN ? chain_knn_eps(space->sp) : box_knn_eps(space->sp);
    if (cudaMalloc(&nn->pts64, sizeof(double) * space->sp.dim * capacity) != cudaSuccess ||
        cudaMalloc(&nn->feat32, sizeof(float) * nn->F * capacity) != cudaSuccess ||
        cudaMalloc(&nn->alive, capacity) != cudaSuccess || nn->ctr.init() != GBO_OK)
    {
        delete nn;
        return fail(GBO_ERR_OUT_OF_MEMORY, "nearest-neighbour index allocation failed");
    }
    cudaMemset(nn->alive, 0, capacity);
    if (cudaStreamCreateWithFlags(&nn->host_stream, cudaStreamNonBlocking) != cudaSuccess)
    {
        delete nn;
        return fail(GBO_ERR_CUDA, "stream creation failed");
    }
    *out = nn;
    return GBO_OK;
}

gbo_status gbo_nn_destroy(gbo_nn *nn)
{
    if (nn)
        cudaDeviceSynchronize();
    delete nn;
    return GBO_OK;
}

gbo_status gbo_nn_set_precision(gbo_nn *nn, int precision)
{
    if (!nn || (precision != GBO_PRECISION_FP64 && precision != GBO_PRECISION_FP32_GUARDED))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad precision");
    nn->precision = precision;
    return GBO_OK;
}

gbo_status gbo_nn_add(gbo_nn *nn, const double *states, int64_t n, int64_t ld, int layout, int64_t *first_key,
                      gbo_stream stream)
{
    if (!nn || n < 0 || (n > 0 && !states) || !valid_layout(layout, n, ld, nn->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad add arguments");
    if (nn->size + n > nn->cap)
        return fail(GBO_ERR_OUT_OF_MEMORY, "nearest-neighbour index capacity exceeded");
    if (first_key)
        *first_key = nn->size;
    LaunchCfg lc = lcfg(stream);
    StatesView v = make_view(states, ld, layout);
    launch_store_points(lc, v, n, nn->sp.dim, nn->pts64, nn->cap, nn->size, nn->alive);
    // features of the new elements, written at column offset `size` of the [F][cap] array
    launch_features(lc, nn->sp, v, n, nn->feat32 + nn->size, nn->cap);
    CHECK_LAUNCH();
    nn->size += n;
    nn->alive_count += n;
    nn->cells.valid = false;
    nn->ccells.valid = false;
    return GBO_OK;
}

gbo_status gbo_nn_remove(gbo_nn *nn, const int64_t *keys, int64_t n, gbo_stream stream)
{
    if (!nn || n < 0 || (n > 0 && !keys))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad remove arguments");
    launch_remove(lcfg(stream), keys, n, nn->size, nn->alive);
    CHECK_LAUNCH();
    nn->alive_count = -1;  // recounted on demand
    nn->cells.valid = false;
    nn->ccells.valid = false;
    return GBO_OK;
}

gbo_status gbo_nn_clear(gbo_nn *nn)
{
    if (!nn)
        return fail(GBO_ERR_INVALID_ARGUMENT, "nn is NULL");
    CUDA_TRY(cudaDeviceSynchronize());
    CUDA_TRY(cudaMemset(nn->alive, 0, nn->cap));
    nn->size = 0;
    nn->alive_count = 0;
    nn->cells.valid = false;
    nn->ccells.valid = false;
    return GBO_OK;
}

gbo_status gbo_nn_size(const gbo_nn *nn, int64_t *size)
{
    if (!nn || !size)
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad size arguments");
    auto *m = const_cast<gbo_nn *>(nn);
    if (m->alive_count < 0)
    {
        std::vector<unsigned char> h(m->size);
        CUDA_TRY(cudaDeviceSynchronize());
        if (m->size)
            CUDA_TRY(cudaMemcpy(h.data(), m->alive, m->size, cudaMemcpyDeviceToHost));
        int64_t c = 0;
        for (auto x : h)
            c += x;
        m->alive_count = c;
    }
    *size = m->alive_count;
    return GBO_OK;
}

static NNArgs nn_args(const gbo_nn *nn)
{
    NNArgs a;
    a.pts64 = nn->pts64;
    a.feat32 = nn->feat32;
    a.alive = nn->alive;
    a.cap = nn->cap;
    a.size = nn->size;
    a.eps32 = nn->eps32;
    return a;
}

// (Re)build the cell index of a RealVector / wrapped gbo_nn in stream order.
static gbo_status ensure_box_cells(gbo_nn *nn, const LaunchCfg &lc)
{
    NNBoxCells &c = nn->cells;
    if (c.valid)
        return GBO_OK;
    c.L = bcell_levels(nn->sp.dim, nn->size);
    c.C = 1;
    for (int d = 0; d < nn->sp.dim; ++d)
        c.C *= c.L;
    const int64_t n = std::max<int64_t>(nn->size, 1);
    const cudaStream_t s = lc.stream;
    for (auto r : {c.cell.reserve((size_t)n * sizeof(int), s), c.count.reserve((size_t)c.C * sizeof(int), s),
                   c.start.reserve((size_t)(c.C + 1) * sizeof(int), s), c.fill.reserve((size_t)c.C * sizeof(int), s),
                   c.skey.reserve((size_t)n * sizeof(int64_t), s), c.pts8.reserve((size_t)n * 2 * sizeof(float4), s),
                   c.box.reserve((size_t)c.C * 4 * sizeof(float4), s)})
        if (r)
            return r;
    launch_bcell_build(lc, nn_args(nn), nn->sp, c.L, c.C, (int *)c.cell.p, (int *)c.count.p, (int *)c.start.p,
                       (int *)c.fill.p, (int64_t *)c.skey.p, (float4 *)c.pts8.p, (float4 *)c.box.p);
    CHECK_LAUNCH();
    c.valid = true;
    return GBO_OK;
}

static gbo_status ensure_chain_cells(gbo_nn *nn, const LaunchCfg &lc)
{
    NNChainCells &c = nn->ccells;
    if (c.valid)
        return GBO_OK;
    const int64_t n = std::max<int64_t>(nn->size, 1);
    const cudaStream_t s = lc.stream;
    for (auto r : {c.key.reserve((size_t)n * sizeof(int), s), c.count.reserve(kQueryKeys * sizeof(int), s),
                   c.start.reserve(kQueryKeys * sizeof(int), s), c.fill.reserve(kQueryKeys * sizeof(int), s),
                   c.skey.reserve((size_t)n * sizeof(int64_t), s), c.sfeat.reserve((size_t)n * 5 * sizeof(float4), s),
                   c.box.reserve((size_t)kQueryKeys * 5 * sizeof(uint4), s),
                   c.cstart.reserve((size_t)(kQueryKeys + 1) * sizeof(int), s),
                   c.cbox.reserve((size_t)(n / 32 + kQueryKeys) * 5 * sizeof(uint4), s)})
        if (r)
            return r;
    launch_ccell_build(lc, nn_args(nn), nn->sp, (int *)c.key.p, (int *)c.count.p, (int *)c.start.p, (int *)c.fill.p,
                       (int64_t *)c.skey.p, (float4 *)c.sfeat.p, (uint4 *)c.box.p, (int *)c.cstart.p,
                       (uint4 *)c.cbox.p);
    CHECK_LAUNCH();
    c.valid = true;
    return GBO_OK;
}

gbo_status gbo_nn_nearest_k(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout, int k,
                            const int64_t *prefix, int64_t *idx, double *dist, gbo_stream stream)
{
    Trace trace("gbo_nn_nearest_k");
    if (!nn || nq < 0 || k < 1 || (nq > 0 && (!q || !idx)) || !valid_layout(layout, nq, ld, nn->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad nearestK arguments");
    if (k > 64)
        return fail(GBO_ERR_UNSUPPORTED, "nearestK supports k <= 64");
    if (nq == 0)
        return GBO_OK;
    LaunchCfg lc = lcfg(stream);
    NNArgs a = nn_args(nn);
    StatesView qv = make_view(q, ld, layout);
    RunCounters *ctr = nn->ctr.take(lc.stream);
    nn->queries += nq;
    if (nn->precision == GBO_PRECISION_FP32_GUARDED && k <= knn_fp32_max_k(nn->sp))
    {
        if (auto st = nn->qfeat.reserve(sizeof(float) * nn->F * nq, lc.stream))
            return st;
        if (auto st = nn->fb_list.reserve(sizeof(unsigned long long) * nq, lc.stream))
            return st;
        unsigned long long *fb_n = &ctr->queue;
        const int P = knn_chunks(lc, nq, nn->size);
        const int keep = knn_keep(k);
        const size_t pl = (size_t)P * nq * keep;
        if (auto st = nn->part.reserve(pl * (sizeof(float) + sizeof(int64_t)) + (size_t)nq * sizeof(unsigned) + 64,
                                       lc.stream))
            return st;
        int64_t *part_k = (int64_t *)nn->part.p;
        float *part_d = (float *)(part_k + pl);
        unsigned *thr = (unsigned *)(part_d + pl);  // per-query bound shared by the chunks of the FP32 scan
        launch_features(lc, nn->sp, qv, nq, (float *)nn->qfeat.p, nq);
        // large batches over a large RealVector / wrapped index: cell index (PRM's prefix kNN)
        if ((nn->sp.kind == GBO_SPACE_WRAP_L2 || nn->sp.kind == GBO_SPACE_REAL_VECTOR) && nn->sp.dim <= 8 &&
            nn->size >= 65536 && nn->size < (1ll << 31) && nq >= 256)
        {
            if (auto st = ensure_box_cells(nn, lc))
                return st;
            NNBoxCells &c = nn->cells;
            const int bands = prefix ? 4 : 1, keys = bands * c.C;
            for (auto r : {c.qcell.reserve((size_t)nq * sizeof(int), lc.stream),
                           c.qcount.reserve((size_t)keys * sizeof(int), lc.stream),
                           c.qstart.reserve((size_t)(keys + 1) * sizeof(int), lc.stream),
                           c.qfill.reserve((size_t)keys * sizeof(int), lc.stream),
                           c.qorder.reserve((size_t)nq * sizeof(int64_t), lc.stream)})
                if (r)
                    return r;
            launch_bcell_query_order(lc, nn->sp, c.L, c.C, (const float *)nn->qfeat.p, nq, prefix, nn->size, bands,
                                     (int *)c.qcell.p, (int *)c.qcount.p, (int *)c.qstart.p, (int *)c.qfill.p,
                                     (int64_t *)c.qorder.p);
            BoxCellArgs ci{(const int *)c.start.p, (const int64_t *)c.skey.p, (const float4 *)c.pts8.p,
                           (const float4 *)c.box.p, c.C};
            if (launch_knn_bcell(lc, a, ci, nn->sp, qv, (const float *)nn->qfeat.p, nq, (const int64_t *)c.qorder.p,
                                 (const int *)c.qcell.p, k, prefix, idx, dist, (unsigned long long *)nn->fb_list.p,
                                 fb_n, ctr, part_d, part_k))
            {
                launch_knn_exact(lc, a, nn->sp, qv, nq, k, prefix, idx, dist,
                                 (const unsigned long long *)nn->fb_list.p, fb_n, std::min<int64_t>(nq, 4096));
                CHECK_LAUNCH();
                return GBO_OK;
            }
        }
        // large batches without prefix limits run in spatial order (the lanes of a warp then prune the
        // same elements); with PRM prefix limits the given order keeps each CTA's scan range short
        const int64_t *order = nullptr;
        if (!prefix && nq >= 1024)
        {
            const size_t wb = ((size_t)3 * kQueryKeys + nq) * sizeof(int);
            if (auto st = nn->qorder.reserve(wb + (size_t)nq * sizeof(int64_t) + 16, lc.stream))
                return st;
            int *work = (int *)nn->qorder.p;
            int64_t *ord = (int64_t *)((char *)nn->qorder.p + pad16(wb));
            launch_query_order(lc, nn->sp, (const float *)nn->qfeat.p, nq, work, ord);
            order = ord;
            // a large chain index: the cell search, one warp per query (the query order's keys are the
            // cells)
            if (nn->sp.kind == GBO_SPACE_KINEMATIC_CHAIN && nn->sp.dim <= 10 && k <= 20 && nn->size >= 65536 &&
                nn->size < (1ll << 31))
            {
                if (auto st = ensure_chain_cells(nn, lc))
                    return st;
                NNChainCells &c = nn->ccells;
                const ChainCellArgs ci{(const int *)c.start.p,  (const int *)c.count.p, (const int64_t *)c.skey.p,
                                       (const float4 *)c.sfeat.p, nn->size,  (const uint4 *)c.box.p,
                                       (const int *)c.cstart.p,   (const uint4 *)c.cbox.p};
                if (launch_knn_ccell(lc, a, ci, nn->sp, qv, (const float *)nn->qfeat.p, nq, ord,
                                     work + 3 * kQueryKeys, k, idx, dist, (unsigned long long *)nn->fb_list.p, fb_n,
                                     ctr, part_d, part_k))
                {
                    launch_knn_exact(lc, a, nn->sp, qv, nq, k, prefix, idx, dist,
                                     (const unsigned long long *)nn->fb_list.p, fb_n, std::min<int64_t>(nq, 4096));
                    CHECK_LAUNCH();
                    return GBO_OK;
                }
            }
        }
        if (launch_knn_fp32(lc, a, nn->sp, qv, (const float *)nn->qfeat.p, nq, k, prefix, idx, dist,
                            (unsigned long long *)nn->fb_list.p, fb_n, ctr, part_d, part_k, P, order, thr))
        {
            // queries whose FP32 band overflowed: exact FP64 scan (count read on the device)
            launch_knn_exact(lc, a, nn->sp, qv, nq, k, prefix, idx, dist, (const unsigned long long *)nn->fb_list.p,
                             fb_n, std::min<int64_t>(nq, 4096));
            CHECK_LAUNCH();
            return GBO_OK;
        }
    }
    launch_knn_exact(lc, a, nn->sp, qv, nq, k, prefix, idx, dist, nullptr, nullptr, nq);
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_nn_nearest_r_count(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout, double r,
                                  int64_t *counts, gbo_stream stream)
{
    if (!nn || nq < 0 || (nq > 0 && (!q || !counts)) || !valid_layout(layout, nq, ld, nn->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad nearestR arguments");
    launch_radius(lcfg(stream), nn_args(nn), nn->sp, make_view(q, ld, layout), nq, r, counts, nullptr, nullptr,
                  nullptr);
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_nn_nearest_r_fill(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout, double r,
                                 const int64_t *offsets, int64_t *idx, double *dist, gbo_stream stream)
{
    if (!nn || nq < 0 || (nq > 0 && (!q || !offsets || !idx || !dist)) || !valid_layout(layout, nq, ld, nn->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad nearestR arguments");
    launch_radius(lcfg(stream), nn_args(nn), nn->sp, make_view(q, ld, layout), nq, r, nullptr, offsets, idx, dist);
    CHECK_LAUNCH();
    return GBO_OK;
}

// NearestNeighborsSqrtApprox::nearest (NearestNeighborsSqrtApprox.h:91-115) for nq queries made one after
// another. checks = 1 + floor(sqrt(n)) for the n present elements; *offset is the structure's offset
// before the first query and after the last. Positions count the present elements in insertion order
// (NearestNeighborsLinear's vector, whose remove erases); with removals a table of their keys is built
// on the host.
gbo_status gbo_nn_nearest_sqrt_approx(gbo_nn *nn, const double *q, int64_t nq, int64_t ld, int layout,
                                      uint64_t *offset, int64_t *idx, double *dist, gbo_stream stream)
{
    Trace trace("gbo_nn_nearest_sqrt_approx");
    if (!nn || !offset || nq < 0 || (nq > 0 && (!q || !idx || !dist)) ||
        !(layout == GBO_LAYOUT_SOA ? ld >= nq : (layout == GBO_LAYOUT_AOS && ld >= nn->sp.dim)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad nearest arguments");
    if (nq == 0)
        return GBO_OK;
    int64_t n = 0;
    if (auto st = gbo_nn_size(nn, &n))
        return st;
    if (n == 0)
        return fail(GBO_ERR_INVALID_ARGUMENT, "No elements found in nearest neighbors data structure");
    const int64_t checks = 1 + (int64_t)std::floor(std::sqrt((double)n));
    const cudaStream_t s = (cudaStream_t)stream;
    const int64_t *rank = nullptr;
    if (n != nn->size)
    {
        std::vector<unsigned char> alive((size_t)nn->size);
        CUDA_TRY(cudaStreamSynchronize(s));
        CUDA_TRY(cudaMemcpy(alive.data(), nn->alive, (size_t)nn->size, cudaMemcpyDeviceToHost));
        std::vector<int64_t> keys;
        keys.reserve((size_t)n);
        for (int64_t k = 0; k < nn->size; ++k)
            if (alive[(size_t)k])
                keys.push_back(k);
        if ((int64_t)keys.size() != n)
            return fail(GBO_ERR_INVALID_ARGUMENT, "element count changed during the call");
        if (auto st = nn->ranks.reserve(keys.size() * sizeof(int64_t), s))
            return st;
        CUDA_TRY(cudaMemcpyAsync(nn->ranks.p, keys.data(), keys.size() * sizeof(int64_t), cudaMemcpyHostToDevice, s));
        rank = (const int64_t *)nn->ranks.p;
    }
    launch_sqrt_approx(lcfg(stream), nn_args(nn), nn->sp, make_view(q, ld, layout), nq, n, checks,
                       (unsigned long long)*offset, rank, idx, dist);
    CHECK_LAUNCH();
    if (rank)
        CUDA_TRY(cudaStreamSynchronize(s));  // the key table is host memory's copy
    *offset = (*offset + (uint64_t)nq) % (uint64_t)checks;
    return GBO_OK;
}

gbo_status gbo_nn_error_stats(const gbo_nn *nn, float *max_abs_error, float *bound)
{
    if (!nn)
        return fail(GBO_ERR_INVALID_ARGUMENT, "nn is NULL");
    RunCounters h{};
    CUDA_TRY(cudaMemcpy(&h, nn->ctr.dev + nn->ctr.last, sizeof(h), cudaMemcpyDeviceToHost));
    if (max_abs_error)
    {
        float e;
        std::memcpy(&e, &h.max_err_bits, sizeof(e));
        *max_abs_error = e;
    }
    if (bound)
        *bound = nn->eps32;
    return GBO_OK;
}

gbo_status gbo_nn_stats(const gbo_nn *nn, uint64_t *queries, uint64_t *rechecked, uint64_t *fallbacks)
{
    if (!nn)
        return fail(GBO_ERR_INVALID_ARGUMENT, "nn is NULL");
    RunCounters h{};
    CUDA_TRY(cudaMemcpy(&h, nn->ctr.dev + nn->ctr.last, sizeof(h), cudaMemcpyDeviceToHost));
    if (queries)
        *queries = nn->queries;
    if (rechecked)
        *rechecked = h.rechecked;
    if (fallbacks)
        *fallbacks = h.fallbacks;
    return GBO_OK;
}

gbo_status gbo_nn_search_bytes(const gbo_nn *nn, uint64_t *bytes)
{
    if (!nn || !bytes)
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad search-bytes arguments");
    RunCounters h{};
    CUDA_TRY(cudaMemcpy(&h, nn->ctr.dev + nn->ctr.last, sizeof(h), cudaMemcpyDeviceToHost));
    *bytes = h.bytes;
    return GBO_OK;
}

gbo_status gbo_nn_add_host(gbo_nn *nn, const double *states, int64_t n, int64_t *first_key)
{
    if (!nn || n < 0 || (n > 0 && !states))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad add arguments");
    std::lock_guard<std::mutex> lk(nn->mu);
    const size_t b = (size_t)n * nn->sp.dim * sizeof(double);
    if (auto st = nn->pin.reserve(b + 16))
        return st;
    if (auto st = nn->dev.reserve(b + 16, nn->host_stream))
        return st;
    std::memcpy(nn->pin.p, states, b);
    CUDA_TRY(cudaMemcpyAsync(nn->dev.p, nn->pin.p, b, cudaMemcpyHostToDevice, nn->host_stream));
    if (auto st = gbo_nn_add(nn, (const double *)nn->dev.p, n, nn->sp.dim, GBO_LAYOUT_AOS, first_key,
                             nn->host_stream))
        return st;
    CUDA_TRY(cudaStreamSynchronize(nn->host_stream));
    return GBO_OK;
}

gbo_status gbo_nn_remove_host(gbo_nn *nn, const int64_t *keys, int64_t n)
{
    if (!nn || n < 0 || (n > 0 && !keys))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad remove arguments");
    std::lock_guard<std::mutex> lk(nn->mu);
    const size_t b = (size_t)n * sizeof(int64_t);
    if (auto st = nn->dev.reserve(b + 16, nn->host_stream))
        return st;
    CUDA_TRY(cudaMemcpyAsync(nn->dev.p, keys, b, cudaMemcpyHostToDevice, nn->host_stream));
    if (auto st = gbo_nn_remove(nn, (const int64_t *)nn->dev.p, n, nn->host_stream))
        return st;
    CUDA_TRY(cudaStreamSynchronize(nn->host_stream));
    return GBO_OK;
}

gbo_status gbo_nn_nearest_k_host(gbo_nn *nn, const double *q, int64_t nq, int k, int64_t *idx, double *dist)
{
    if (!nn || nq < 0 || k < 1 || (nq > 0 && (!q || !idx)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad nearestK arguments");
    std::lock_guard<std::mutex> lk(nn->mu);
    const size_t bq = (size_t)nq * nn->sp.dim * sizeof(double), bo = (size_t)nq * k * 8;
    if (auto st = nn->pin.reserve(std::max(bq, 2 * bo) + 16))
        return st;
    if (auto st = nn->dev.reserve(bq + 2 * bo + 32, nn->host_stream))
        return st;
    char *d = (char *)nn->dev.p;
    std::memcpy(nn->pin.p, q, bq);
    CUDA_TRY(cudaMemcpyAsync(d, nn->pin.p, bq, cudaMemcpyHostToDevice, nn->host_stream));
    int64_t *di = (int64_t *)(d + pad16(bq));
    double *dd = (double *)(d + pad16(bq) + bo);
    if (auto st = gbo_nn_nearest_k(nn, (const double *)d, nq, nn->sp.dim, GBO_LAYOUT_AOS, k, nullptr, di,
                                   dist ? dd : nullptr, nn->host_stream))
        return st;
    CUDA_TRY(cudaMemcpyAsync(nn->pin.p, di, bo, cudaMemcpyDeviceToHost, nn->host_stream));
    if (dist)
        CUDA_TRY(cudaMemcpyAsync((char *)nn->pin.p + bo, dd, bo, cudaMemcpyDeviceToHost, nn->host_stream));
    CUDA_TRY(cudaStreamSynchronize(nn->host_stream));
    std::memcpy(idx, nn->pin.p, bo);
    if (dist)
        std::memcpy(dist, (char *)nn->pin.p + bo, bo);
    return GBO_OK;
}

gbo_status gbo_nn_nearest_sqrt_approx_host(gbo_nn *nn, const double *q, int64_t nq, uint64_t *offset, int64_t *idx,
                                           double *dist)
{
    if (!nn || !offset || nq < 0 || (nq > 0 && (!q || !idx)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad nearest arguments");
    std::lock_guard<std::mutex> lk(nn->mu);
    const size_t bq = (size_t)nq * nn->sp.dim * sizeof(double), bo = (size_t)nq * 8;
    if (auto st = nn->pin.reserve(std::max(bq, 2 * bo) + 16))
        return st;
    if (auto st = nn->dev.reserve(bq + 2 * bo + 32, nn->host_stream))
        return st;
    char *d = (char *)nn->dev.p;
    std::memcpy(nn->pin.p, q, bq);
    CUDA_TRY(cudaMemcpyAsync(d, nn->pin.p, bq, cudaMemcpyHostToDevice, nn->host_stream));
    int64_t *di = (int64_t *)(d + pad16(bq));
    double *dd = (double *)(d + pad16(bq) + bo);
    if (auto st = gbo_nn_nearest_sqrt_approx(nn, (const double *)d, nq, nn->sp.dim, GBO_LAYOUT_AOS, offset, di, dd,
                                             nn->host_stream))
        return st;
    CUDA_TRY(cudaMemcpyAsync(nn->pin.p, di, bo, cudaMemcpyDeviceToHost, nn->host_stream));
    CUDA_TRY(cudaMemcpyAsync((char *)nn->pin.p + bo, dd, bo, cudaMemcpyDeviceToHost, nn->host_stream));
    CUDA_TRY(cudaStreamSynchronize(nn->host_stream));
    std::memcpy(idx, nn->pin.p, bo);
    if (dist)
        std::memcpy(dist, (char *)nn->pin.p + bo, bo);
    return GBO_OK;
}

gbo_status gbo_nn_nearest_r_host(gbo_nn *nn, const double *q, double r, int64_t cap, int64_t *count, int64_t *idx,
                                 double *dist)
{
    if (!nn || !q || !count || cap < 0 || (cap > 0 && (!idx || !dist)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad nearestR arguments");
    std::lock_guard<std::mutex> lk(nn->mu);
    const int dim = nn->sp.dim;
    if (auto st = nn->dev.reserve(64 + 16 * (size_t)(nn->size + 1) + 16 * (size_t)dim, nn->host_stream))
        return st;
    char *d = (char *)nn->dev.p;
    double *dq = (double *)d;
    int64_t *dcount = (int64_t *)(d + 16 * ((dim * 8 + 15) / 16));
    int64_t *doff = dcount + 1;
    int64_t *didx = dcount + 2;
    double *ddist = (double *)(didx + nn->size + 1);
    CUDA_TRY(cudaMemcpyAsync(dq, q, dim * sizeof(double), cudaMemcpyHostToDevice, nn->host_stream));
    CUDA_TRY(cudaMemsetAsync(doff, 0, sizeof(int64_t), nn->host_stream));
    if (auto st = gbo_nn_nearest_r_count(nn, dq, 1, dim, GBO_LAYOUT_AOS, r, dcount, nn->host_stream))
        return st;
    if (auto st = gbo_nn_nearest_r_fill(nn, dq, 1, dim, GBO_LAYOUT_AOS, r, doff, didx, ddist, nn->host_stream))
        return st;
    int64_t c = 0;
    CUDA_TRY(cudaMemcpyAsync(&c, dcount, sizeof(int64_t), cudaMemcpyDeviceToHost, nn->host_stream));
    CUDA_TRY(cudaStreamSynchronize(nn->host_stream));
    *count = c;
    const int64_t m = std::min(c, cap);
    if (m > 0)
    {
        CUDA_TRY(cudaMemcpy(idx, didx, m * sizeof(int64_t), cudaMemcpyDeviceToHost));
        CUDA_TRY(cudaMemcpy(dist, ddist, m * sizeof(double), cudaMemcpyDeviceToHost));
    }
    return GBO_OK;
}

gbo_status gbo_sample_uniform_host(gbo_sampler *s, int64_t n, double *out)
{
    if (!s || n < 0 || (n > 0 && !out))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sampleUniform arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    const size_t b = (size_t)n * s->sp.dim * sizeof(double);
    if (auto st = s->dev.reserve(b + 16, s->host_stream))
        return st;
    if (auto st = s->pin.reserve(b + 16))
        return st;
    if (auto st = gbo_sample_uniform(s, n, (double *)s->dev.p, s->sp.dim, GBO_LAYOUT_AOS, s->host_stream))
        return st;
    CUDA_TRY(cudaMemcpyAsync(s->pin.p, s->dev.p, b, cudaMemcpyDeviceToHost, s->host_stream));
    CUDA_TRY(cudaStreamSynchronize(s->host_stream));
    std::memcpy(out, s->pin.p, b);
    return GBO_OK;
}

gbo_status gbo_sample_valid_host(gbo_sampler *s, gbo_checker *c, int64_t n, unsigned attempts, double *out,
                                 uint8_t *ok)
{
    if (!s || !c || n < 0 || (n > 0 && (!out || !ok)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sampleValid arguments");
    if (n == 0)
        return GBO_OK;
    std::lock_guard<std::mutex> lk(s->mu);
    const size_t b = (size_t)n * s->sp.dim * sizeof(double);
    if (auto st = s->dev.reserve(b + (size_t)n + 16, s->host_stream))
        return st;
    double *d = (double *)s->dev.p;
    uint8_t *dok = (uint8_t *)s->dev.p + b;
    if (auto st = gbo_sample_valid(s, c, n, attempts, d, s->sp.dim, GBO_LAYOUT_AOS, dok, s->host_stream))
        return st;
    CUDA_TRY(cudaMemcpyAsync(out, d, b, cudaMemcpyDeviceToHost, s->host_stream));
    CUDA_TRY(cudaMemcpyAsync(ok, dok, (size_t)n, cudaMemcpyDeviceToHost, s->host_stream));
    CUDA_TRY(cudaStreamSynchronize(s->host_stream));
    return GBO_OK;
}

gbo_status gbo_sample_uniform_near_host(gbo_sampler *s, const double *near, double distance, int64_t n, double *out)
{
    if (!s || n < 0 || (n > 0 && (!out || !near)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sampleUniformNear arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    const size_t b = (size_t)n * s->sp.dim * sizeof(double);
    if (auto st = s->dev.reserve(2 * b + 32, s->host_stream))
        return st;
    if (auto st = s->pin.reserve(b + 16))
        return st;
    double *dn = (double *)s->dev.p, *dout = (double *)((char *)s->dev.p + pad16(b));
    std::memcpy(s->pin.p, near, b);
    CUDA_TRY(cudaMemcpyAsync(dn, s->pin.p, b, cudaMemcpyHostToDevice, s->host_stream));
    if (auto st = gbo_sample_uniform_near(s, dn, distance, n, s->sp.dim, GBO_LAYOUT_AOS, dout, s->host_stream))
        return st;
    CUDA_TRY(cudaMemcpyAsync(s->pin.p, dout, b, cudaMemcpyDeviceToHost, s->host_stream));
    CUDA_TRY(cudaStreamSynchronize(s->host_stream));
    std::memcpy(out, s->pin.p, b);
    return GBO_OK;
}

gbo_status gbo_sample_gaussian_host(gbo_sampler *s, const double *mean, double stddev, int64_t n, double *out)
{
    if (!s || n < 0 || (n > 0 && (!out || !mean)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sampleGaussian arguments");
    std::lock_guard<std::mutex> lk(s->mu);
    const size_t b = (size_t)n * s->sp.dim * sizeof(double);
    if (auto st = s->dev.reserve(2 * b + 32, s->host_stream))
        return st;
    if (auto st = s->pin.reserve(b + 16))
        return st;
    double *dm = (double *)s->dev.p, *dout = (double *)((char *)s->dev.p + pad16(b));
    std::memcpy(s->pin.p, mean, b);
    CUDA_TRY(cudaMemcpyAsync(dm, s->pin.p, b, cudaMemcpyHostToDevice, s->host_stream));
    if (auto st = gbo_sample_gaussian(s, dm, stddev, n, s->sp.dim, GBO_LAYOUT_AOS, dout, s->host_stream))
        return st;
    CUDA_TRY(cudaMemcpyAsync(s->pin.p, dout, b, cudaMemcpyDeviceToHost, s->host_stream));
    CUDA_TRY(cudaStreamSynchronize(s->host_stream));
    std::memcpy(out, s->pin.p, b);
    return GBO_OK;
}

// PRM::uniteComponents over a roadmap's edges in the order PRM adds them (PRM.cpp:580-609): boost's
// disjoint_sets, every vertex first its own set; union_set(n, m) links the two roots by rank (the root of
// higher rank becomes the parent of the other; on a tie the root of m's set becomes the parent and its
// rank grows), finds compress paths. root[v] = find_set(v) after the last union: the component tag that
// PRM::getPlannerData gives each vertex (PRM.cpp:734-754). Host memory, no device work.
gbo_status gbo_prm_component_roots(const int64_t *src, const int64_t *dst, int64_t n_edges, int64_t n_vertices,
                                   int64_t *root)
{
    if (n_edges < 0 || n_vertices < 0 || (n_edges && (!src || !dst)) || (n_vertices && !root))
        return GBO_ERR_INVALID_ARGUMENT;
    std::vector<int64_t> parent((size_t)n_vertices);
    std::vector<uint32_t> rank((size_t)n_vertices, 0);
    for (int64_t v = 0; v < n_vertices; ++v)
        parent[(size_t)v] = v;
    auto find = [&](int64_t x) {
        int64_t r = x;
        while (parent[(size_t)r] != r)
            r = parent[(size_t)r];
        while (parent[(size_t)x] != r)
        {
            const int64_t next = parent[(size_t)x];
            parent[(size_t)x] = r;
            x = next;
        }
        return r;
    };
    for (int64_t e = 0; e < n_edges; ++e)
    {
        if (src[e] < 0 || src[e] >= n_vertices || dst[e] < 0 || dst[e] >= n_vertices)
            return GBO_ERR_INVALID_ARGUMENT;
        const int64_t i = find(src[e]), j = find(dst[e]);
        if (i == j)
            continue;
        if (rank[(size_t)i] > rank[(size_t)j])
            parent[(size_t)j] = i;
        else
        {
            parent[(size_t)i] = j;
            if (rank[(size_t)i] == rank[(size_t)j])
                ++rank[(size_t)j];
        }
    }
    for (int64_t v = 0; v < n_vertices; ++v)
        root[v] = find(v);
    return GBO_OK;
}

gbo_status gbo_measure_fp32_peak(double *flops, gbo_stream stream)
{
    if (!flops)
        return fail(GBO_ERR_INVALID_ARGUMENT, "flops is NULL");
    if (auto st = ensure_device())
        return st;
    *flops = measure_fp32_peak(lcfg(stream));
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_sincos32(const double *theta, int64_t n, float *cos_out, float *sin_out, gbo_stream stream)
{
    if (n < 0 || (n > 0 && (!theta || !cos_out || !sin_out)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sincos32 arguments");
    if (auto st = ensure_device())
        return st;
    launch_sincos32(lcfg(stream), theta, n, cos_out, sin_out);
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_log_rn(const double *x, int64_t n, double *out, gbo_stream stream)
{
    if (n < 0 || n > (int64_t)INT32_MAX * 256 || (n > 0 && (!x || !out)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad log_rn arguments");
    if (auto st = ensure_device())
        return st;
    launch_log_rn(lcfg(stream), x, n, out);
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_sincos_cr(const double *x, int64_t n, double *sin_out, double *cos_out, gbo_stream stream)
{
    if (n < 0 || (n > 0 && (!x || !sin_out || !cos_out)))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad sincos_cr arguments");
    if (auto st = ensure_device())
        return st;
    launch_sincos_cr(lcfg(stream), x, n, sin_out, cos_out);
    CHECK_LAUNCH();
    return GBO_OK;
}

gbo_status gbo_checker_precision_stats(gbo_checker *c, const double *states, int64_t n, int64_t ld, int layout,
                                       gbo_precision_stats *out, gbo_stream stream)
{
    if (!c || !out || n < 0 || (n > 0 && !states) || !valid_layout(layout, n, ld, c->sp.dim))
        return fail(GBO_ERR_INVALID_ARGUMENT, "bad precision_stats arguments");
    if (c->wa.kind != GBO_CHECK_CHAIN_SEGMENTS && c->wa.kind != GBO_CHECK_DH_SPHERES)
        return fail(GBO_ERR_UNSUPPORTED, "this checker has no FP32 form");
    struct Tally
    {
        unsigned long long states, flips, ambiguous;
        unsigned int max_err_bits;
    } h{};
    void *d = nullptr;
    if (cudaMalloc(&d, sizeof(Tally)) != cudaSuccess)
        return fail(GBO_ERR_OUT_OF_MEMORY, "precision_stats buffer");
    LaunchCfg lc = lcfg(stream);
    cudaMemsetAsync(d, 0, sizeof(Tally), lc.stream);
    const bool launched = n > 0 && launch_precision_stats(lc, c->sp, c->wa, make_view(states, ld, layout), n, d);
    cudaMemcpyAsync(&h, d, sizeof(Tally), cudaMemcpyDeviceToHost, lc.stream);
    const cudaError_t e = cudaStreamSynchronize(lc.stream);
    cudaFree(d);
    if (e != cudaSuccess)
        return fail(GBO_ERR_CUDA, cudaGetErrorString(e));
    if (n > 0 && !launched)
        return fail(GBO_ERR_UNSUPPORTED, "precision statistics not available for this checker's size");
    float mx;
    std::memcpy(&mx, &h.max_err_bits, sizeof(mx));
    out->states = h.states;
    out->flips = h.flips;
    out->ambiguous = h.ambiguous;
    out->max_abs_err = mx;
    return GBO_OK;
}

gbo_status gbo_measure_fp64_peak(double *flops, gbo_stream stream)
{
    if (!flops)
        return fail(GBO_ERR_INVALID_ARGUMENT, "flops is NULL");
    if (auto st = ensure_device())
        return st;
    *flops = measure_fp64_peak(lcfg(stream));
    CHECK_LAUNCH();
    return GBO_OK;
}

}  // extern "C"

// ---------------------------------------------------------------- internal accessors (noalloc.cu)
namespace gbo
{
gbo_status internal_fail(gbo_status s, const char *msg)
{
    return fail(s, msg);
}

gbo_status internal_ensure_device(int *sm_count)
{
    if (auto st = ensure_device())
        return st;
    *sm_count = g_sm_count;
    return GBO_OK;
}

gbo_status internal_request_dim(const gbo_request *r, int *dim)
{
    if (r->kind == GBO_REQ_KNN)
    {
        if (!r->nn)
            return GBO_ERR_INVALID_ARGUMENT;
        *dim = r->nn->sp.dim;
        return GBO_OK;
    }
    if ((r->kind != GBO_REQ_VALIDITY && r->kind != GBO_REQ_MOTION) || !r->checker)
        return GBO_ERR_INVALID_ARGUMENT;
    *dim = r->checker->sp.dim;
    return GBO_OK;
}

bool internal_nn_view(const gbo_nn *nn, NNArgs *a, SpaceParams *sp, int *precision, int *features)
{
    if (!nn)
        return false;
    *a = nn_args(nn);
    *sp = nn->sp;
    *precision = nn->precision;
    *features = nn->F;
    return true;
}
}  // namespace gbo
