/*
 * ORACLE (test infrastructure only) — CPU restatement of OMPL's data-parallel inner loop.
 *
 * Parity is pinned: tests/test_oracle_golden.py checks every function below against fixtures
 * produced by OMPL's own sources compiled unmodified (oracle/ref/, tests/golden/make_golden.py),
 * bit for bit. Only tests/, the smoke check and the benchmark's CPU-baseline leg load this library;
 * the product library never links it.
 *
 * Build: g++ -O3 -ffp-contract=off -shared -fPIC (no -march flags), so FP64 results equal the
 * reference's default x86-64 build, which has no FMA and therefore never contracts.
 *
 * Reference citations are paths inside the OMPL source tree:
 *   RV  = src/ompl/base/spaces/src/RealVectorStateSpace.cpp
 *   SO2 = src/ompl/base/spaces/src/SO2StateSpace.cpp
 *   SS  = src/ompl/base/src/StateSpace.cpp
 *   DMV = src/ompl/base/src/DiscreteMotionValidator.cpp
 *   SI  = src/ompl/base/src/SpaceInformation.cpp
 *   KC  = demos/KinematicChain.h
 *   RNG = src/ompl/util/RandomNumbers.h
 *   NNL = src/ompl/datastructures/NearestNeighborsLinear.h
 */
#include "../oracle_api.h"
#include "../dh_arm.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <limits>
#include <queue>
#include <random>
#include <thread>
#include <utility>
#include <vector>

namespace
{
constexpr double kPi = 3.141592653589793238462643383279502884;  // boost::math::double_constants::pi
constexpr double kDblEps = std::numeric_limits<double>::epsilon();
constexpr double kFltEps = std::numeric_limits<float>::epsilon();
const double kNaN = std::numeric_limits<double>::quiet_NaN();

int g_threads = 1;

template <class F>
void parallel_rows(long n, F f)
{
    int t = (int)std::max<long>(1, std::min<long>(g_threads, n));
    if (t <= 1)
    {
        for (long i = 0; i < n; ++i)
            f(i);
        return;
    }
    std::atomic<long> next{0};
    const long chunk = 64;
    std::vector<std::thread> pool;
    for (int w = 0; w < t; ++w)
        pool.emplace_back([&] {
            for (;;)
            {
                long b = next.fetch_add(chunk);
                if (b >= n)
                    break;
                long e = std::min(n, b + chunk);
                for (long i = b; i < e; ++i)
                    f(i);
            }
        });
    for (auto &th : pool)
        th.join();
}

struct Space
{
    int kind, dim;
    std::vector<double> low, high;
    double link;
    double extent, lvs;
    unsigned factor;
};

// StateSpace::setup (SS:237-241): lvs = maxExtent * fraction; extent per kind:
// RV:167-176 (sqrt of summed squared ranges), SO2:69-72 (pi); the chain inherits RV's extent over
// its [-pi,pi] bounds (KC:94-97, no override); WRAP_L2 defines its extent as sqrt(sum pi^2).
Space make_space(const ora_space *d)
{
    Space s;
    s.kind = d->kind;
    s.dim = d->dim;
    s.link = d->link_length;
    s.factor = d->factor;
    s.low.resize(d->dim);
    s.high.resize(d->dim);
    for (int i = 0; i < d->dim; ++i)
    {
        if (d->kind == ORA_SPACE_REAL_VECTOR)
        {
            s.low[i] = d->low[i];
            s.high[i] = d->high[i];
        }
        else
        {
            s.low[i] = -kPi;
            s.high[i] = kPi;
        }
    }
    if (d->kind == ORA_SPACE_SO2)
        s.extent = kPi;
    else if (d->kind == ORA_SPACE_WRAP_L2)
    {
        double e = 0.0;
        for (int i = 0; i < d->dim; ++i)
            e += kPi * kPi;
        s.extent = std::sqrt(e);
    }
    else
    {
        double e = 0.0;
        for (int i = 0; i < d->dim; ++i)
        {
            double r = s.high[i] - s.low[i];
            e += r * r;
        }
        s.extent = std::sqrt(e);
    }
    s.lvs = s.extent * d->lvs_fraction;
    return s;
}

double distance(const Space &s, const double *a, const double *b)
{
    switch (s.kind)
    {
        case ORA_SPACE_SO2:
        {
            // SO2:114-126
            double d = std::fabs(a[0] - b[0]);
            return (d > kPi) ? 2.0 * kPi - d : d;
        }
        case ORA_SPACE_KINEMATIC_CHAIN:
        {
            // KC:105-121: workspace metric over the cumulative link directions
            double theta1 = 0., theta2 = 0., dx = 0., dy = 0., dist = 0.;
            for (int i = 0; i < s.dim; ++i)
            {
                theta1 += a[i];
                theta2 += b[i];
                dx += std::cos(theta1) - std::cos(theta2);
                dy += std::sin(theta1) - std::sin(theta2);
                dist += std::sqrt(dx * dx + dy * dy);
            }
            return dist * s.link;
        }
        case ORA_SPACE_WRAP_L2:
        {
            // L2 over per-joint shortest angular differences (a5.3 of the path's definition)
            double sum = 0.0;
            for (int i = 0; i < s.dim; ++i)
            {
                double d = std::fabs(a[i] - b[i]);
                if (d > kPi)
                    d = 2.0 * kPi - d;
                sum += d * d;
            }
            return std::sqrt(sum);
        }
        default:
        {
            // RV:230-242
            double dist = 0.0;
            for (int i = 0; i < s.dim; ++i)
            {
                double diff = a[i] - b[i];
                dist += diff * diff;
            }
            return std::sqrt(dist);
        }
    }
}

// One joint of the shortest-arc interpolation shared by SO2:134-153 and KC:150-176.
inline double interp_angle(double from, double to, double t)
{
    double diff = to - from;
    if (std::fabs(diff) <= kPi)
        return from + diff * t;
    if (diff > 0.0)
        diff = 2.0 * kPi - diff;
    else
        diff = -2.0 * kPi - diff;
    double v = from - diff * t;
    if (v > kPi)
        v -= 2.0 * kPi;
    else if (v < -kPi)
        v += 2.0 * kPi;
    return v;
}

void interpolate(const Space &s, const double *from, const double *to, double t, double *out)
{
    if (s.kind == ORA_SPACE_REAL_VECTOR)
    {
        // RV:257-265
        for (int i = 0; i < s.dim; ++i)
            out[i] = from[i] + (to[i] - from[i]) * t;
    }
    else
    {
        for (int i = 0; i < s.dim; ++i)
            out[i] = interp_angle(from[i], to[i], t);
    }
}

// SS:851-854
unsigned valid_segment_count(const Space &s, const double *a, const double *b)
{
    return s.factor * (unsigned)std::ceil(distance(s, a, b) / s.lvs);
}

void enforce_bounds(const Space &s, double *v)
{
    if (s.kind == ORA_SPACE_REAL_VECTOR)
    {
        // RV:188-198
        for (int i = 0; i < s.dim; ++i)
        {
            if (v[i] > s.high[i])
                v[i] = s.high[i];
            else if (v[i] < s.low[i])
                v[i] = s.low[i];
        }
        return;
    }
    // SO2:79-87 and KC:123-136 (identical per joint)
    for (int i = 0; i < s.dim; ++i)
    {
        double x = std::fmod(v[i], 2.0 * kPi);
        if (x < -kPi)
            x += 2.0 * kPi;
        else if (x >= kPi)
            x -= 2.0 * kPi;
        v[i] = x;
    }
}

// ---------------------------------------------------------------- validity checkers

// tests/resources/circles2D.h:141-151 (r2 precomputed as r*r, :51)
bool circles_valid(const ora_checker *c, const double *xy)
{
    for (long i = 0; i < c->n_obstacles; ++i)
    {
        const double *o = c->obstacles + 3 * i;
        double r2 = o[2] * o[2];
        double dx = o[0] - xy[0];
        double dy = o[1] - xy[1];
        if (dx * dx + dy * dy < r2)
            return false;
    }
    return true;
}

struct Seg
{
    double x0, y0, x1, y1;
};

// KC:251-276
bool segments_intersect(const Seg &s0, const Seg &s1)
{
    double s10_x = s0.x1 - s0.x0;
    double s10_y = s0.y1 - s0.y0;
    double s32_x = s1.x1 - s1.x0;
    double s32_y = s1.y1 - s1.y0;
    double denom = s10_x * s32_y - s32_x * s10_y;
    if (std::fabs(denom) < kDblEps)
        return false;
    bool denomPositive = denom > 0;
    double s02_x = s0.x0 - s1.x0;
    double s02_y = s0.y0 - s1.y0;
    double s_numer = s10_x * s02_y - s10_y * s02_x;
    if ((s_numer < kFltEps) == denomPositive)
        return false;
    double t_numer = s32_x * s02_y - s32_y * s02_x;
    if ((t_numer < kFltEps) == denomPositive)
        return false;
    if (((s_numer - denom > -kFltEps) == denomPositive) || ((t_numer - denom > kFltEps) == denomPositive))
        return false;
    return true;
}

// KC:209-249: forward kinematics into n link segments plus a 0.001 tip segment, then the
// all-pairs self test and the robot-vs-world test.
bool chain_valid(const Space &s, const ora_checker *c, const double *q)
{
    const int n = s.dim;
    Seg segs[64];
    double theta = 0., x = 0., y = 0., xN, yN;
    for (int i = 0; i < n; ++i)
    {
        theta += q[i];
        xN = x + std::cos(theta) * s.link;
        yN = y + std::sin(theta) * s.link;
        segs[i] = {x, y, xN, yN};
        x = xN;
        y = yN;
    }
    xN = x + std::cos(theta) * 0.001;
    yN = y + std::sin(theta) * 0.001;
    segs[n] = {x, y, xN, yN};
    const int m = n + 1;
    for (int i = 0; i < m; ++i)
        for (int j = i + 1; j < m; ++j)
            if (segments_intersect(segs[i], segs[j]))
                return false;
    for (int i = 0; i < m; ++i)
        for (long j = 0; j < c->n_obstacles; ++j)
        {
            const double *o = c->obstacles + 4 * j;
            Seg w{o[0], o[1], o[2], o[3]};
            if (segments_intersect(segs[i], w))
                return false;
        }
    return true;
}

bool is_valid(const Space &s, const ora_checker *c, const double *q)
{
    switch (c->kind)
    {
        case ORA_CHECK_CIRCLES:
            return circles_valid(c, q);
        case ORA_CHECK_CHAIN_SEGMENTS:
            return chain_valid(s, c, q);
        case ORA_CHECK_DH_SPHERES:
            return gbompl_oracle::dh_valid(c, q);
        default:
            return true;
    }
}

// DMV:48-91 (ordered variant). Returns result; fills lastValid.second, nd and the first invalid index.
bool check_motion_ordered(const Space &s, const ora_checker *c, const double *s1, const double *s2, double &last_t,
                          int &nd_out, int &first_j)
{
    bool result = true;
    int nd = (int)valid_segment_count(s, s1, s2);
    nd_out = nd;
    first_j = -1;
    if (nd > 1)
    {
        std::vector<double> test(s.dim);
        for (int j = 1; j < nd; ++j)
        {
            interpolate(s, s1, s2, (double)j / (double)nd, test.data());
            if (!is_valid(s, c, test.data()))
            {
                last_t = (double)(j - 1) / (double)nd;
                first_j = j;
                result = false;
                break;
            }
        }
    }
    if (result)
        if (!is_valid(s, c, s2))
        {
            last_t = (double)(nd - 1) / (double)nd;
            first_j = nd;
            result = false;
        }
    return result;
}

// DMV:93-145 (bisection variant): s2 first, then FIFO midpoint subdivision of [1, nd-1].
bool check_motion_bisect(const Space &s, const ora_checker *c, const double *s1, const double *s2)
{
    if (!is_valid(s, c, s2))
        return false;
    bool result = true;
    int nd = (int)valid_segment_count(s, s1, s2);
    std::queue<std::pair<int, int>> pos;
    if (nd >= 2)
    {
        pos.emplace(1, nd - 1);
        std::vector<double> test(s.dim);
        while (!pos.empty())
        {
            std::pair<int, int> x = pos.front();
            int mid = (x.first + x.second) / 2;
            interpolate(s, s1, s2, (double)mid / (double)nd, test.data());
            if (!is_valid(s, c, test.data()))
            {
                result = false;
                break;
            }
            pos.pop();
            if (x.first < mid)
                pos.emplace(x.first, mid - 1);
            if (x.second > mid)
                pos.emplace(mid + 1, x.second);
        }
    }
    return result;
}

// Exact k-nearest by (distance, insertion index), distance evaluated as distance(point, query)
// like NNL:159-172 (ElemSort calls df_(element, query)).
void knn_one(const Space &s, const double *pts, long npts, long limit, const double *q, int k, long *idx,
             double *dist)
{
    std::vector<std::pair<double, long>> all;
    long m = std::min(npts, limit);
    all.reserve(m);
    for (long i = 0; i < m; ++i)
        all.emplace_back(distance(s, pts + (size_t)i * s.dim, q), i);
    long kk = std::min<long>(k, m);
    std::partial_sort(all.begin(), all.begin() + kk, all.end());
    for (long j = 0; j < k; ++j)
    {
        idx[j] = j < kk ? all[j].second : -1;
        dist[j] = j < kk ? all[j].first : std::numeric_limits<double>::infinity();
    }
}
}  // namespace

extern "C" {

int ora_set_threads(int n)
{
    int old = g_threads;
    g_threads = n < 1 ? 1 : n;
    return old;
}

double ora_space_extent(const ora_space *d)
{
    return make_space(d).extent;
}

double ora_space_lvs(const ora_space *d)
{
    return make_space(d).lvs;
}

void ora_distance(const ora_space *d, const double *a, const double *b, long n, double *out)
{
    Space s = make_space(d);
    parallel_rows(n, [&](long i) { out[i] = distance(s, a + (size_t)i * s.dim, b + (size_t)i * s.dim); });
}

void ora_interpolate(const ora_space *d, const double *a, const double *b, const double *t, long n, double *out)
{
    Space s = make_space(d);
    parallel_rows(n, [&](long i) {
        interpolate(s, a + (size_t)i * s.dim, b + (size_t)i * s.dim, t[i], out + (size_t)i * s.dim);
    });
}

void ora_valid_segment_count(const ora_space *d, const double *a, const double *b, long n, unsigned *out)
{
    Space s = make_space(d);
    parallel_rows(n, [&](long i) { out[i] = valid_segment_count(s, a + (size_t)i * s.dim, b + (size_t)i * s.dim); });
}

void ora_enforce_bounds(const ora_space *d, double *states, long n)
{
    Space s = make_space(d);
    parallel_rows(n, [&](long i) { enforce_bounds(s, states + (size_t)i * s.dim); });
}

// RNG:72-76: uniformReal(lo, hi) = (hi - lo) * uniform01 + lo, with uniform01 the libstdc++
// uniform_real_distribution<double>(0,1) over std::mt19937 (RNG:190-191); seeding per
// RandomNumbers.cpp setLocalSeed (generator_.seed(localSeed)).
void ora_rng_uniform(unsigned seed, int kind, double lo, double hi, long n, double *out)
{
    std::mt19937 gen(seed);
    std::uniform_real_distribution<> uni{0, 1};
    for (long i = 0; i < n; ++i)
        out[i] = kind == 0 ? uni(gen) : (hi - lo) * uni(gen) + lo;
}

// RV:45-53 (RealVector, chain and wrap-L2 spaces use RealVectorStateSampler) and SO2:46-49.
void ora_sample_uniform(const ora_space *d, unsigned seed, long n, double *out)
{
    Space s = make_space(d);
    std::mt19937 gen(seed);
    std::uniform_real_distribution<> uni{0, 1};
    for (long i = 0; i < n; ++i)
        for (int k = 0; k < s.dim; ++k)
        {
            double lo = s.low[k], hi = s.high[k];
            out[(size_t)i * s.dim + k] = (hi - lo) * uni(gen) + lo;
        }
}

// RV:55-65 and SO2:51-56 (SO2 draws in [near-d, near+d] then wraps with enforceBounds).
void ora_sample_uniform_near(const ora_space *d, unsigned seed, const double *near, double distance_, long n,
                             double *out)
{
    Space s = make_space(d);
    std::mt19937 gen(seed);
    std::uniform_real_distribution<> uni{0, 1};
    for (long i = 0; i < n; ++i)
    {
        const double *nr = near + (size_t)i * s.dim;
        double *o = out + (size_t)i * s.dim;
        if (s.kind == ORA_SPACE_SO2)
        {
            double lo = nr[0] - distance_, hi = nr[0] + distance_;
            o[0] = (hi - lo) * uni(gen) + lo;
            enforce_bounds(s, o);
            continue;
        }
        for (int k = 0; k < s.dim; ++k)
        {
            double lo = std::max(s.low[k], nr[k] - distance_);
            double hi = std::min(s.high[k], nr[k] + distance_);
            o[k] = (hi - lo) * uni(gen) + lo;
        }
    }
}

// Natural log rounded to nearest, evaluated in double-double: x = 2^e m, m in [sqrt(1/2), sqrt(2)),
// s = (m - 1)/(m + 1), log m = 2 (s + s^3/3 + s^5/5 + ...) up to s^41/41 (terms from s^21 on in plain
// FP64), log x = e ln2 + log m; ln 2 and 1/(2k+1) split exactly into two doubles. Two-sum (Knuth) and
// fma two-product give the double-double operations.
namespace
{
struct DD
{
    double hi, lo;
};
DD two_sum(double a, double b)
{
    const double s = a + b, bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
DD fast_two_sum(double a, double b)
{
    const double s = a + b;
    return {s, b - (s - a)};
}
DD dd_add(DD a, DD b)
{
    DD s = two_sum(a.hi, b.hi);
    const DD t = two_sum(a.lo, b.lo);
    s.lo += t.hi;
    s = fast_two_sum(s.hi, s.lo);
    s.lo += t.lo;
    return fast_two_sum(s.hi, s.lo);
}
DD dd_mul(DD a, DD b)
{
    const double p = a.hi * b.hi;
    double e = std::fma(a.hi, b.hi, -p);
    e = std::fma(a.hi, b.lo, e);
    e = std::fma(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
DD dd_div(double a, DD b)
{
    const double q1 = a / b.hi;
    const DD p1 = dd_mul({q1, 0.0}, b);
    DD r = two_sum(a, -p1.hi);
    r.lo -= p1.lo;
    const double q2 = (r.hi + r.lo) / b.hi;
    const DD p2 = dd_mul({q2, 0.0}, b);
    const DD r2 = dd_add(r, {-p2.hi, -p2.lo});
    const double q3 = (r2.hi + r2.lo) / b.hi;
    return dd_add(fast_two_sum(q1, q2), {q3, 0.0});
}
double log_rn(double x)
{
    static const double kHi[21] = {0.0, 0x1.5555555555555p-2, 0x1.999999999999ap-3, 0x1.2492492492492p-3,
                                   0x1.c71c71c71c71cp-4, 0x1.745d1745d1746p-4, 0x1.3b13b13b13b14p-4,
                                   0x1.1111111111111p-4, 0x1.e1e1e1e1e1e1ep-5, 0x1.af286bca1af28p-5,
                                   0x1.8618618618618p-5, 0x1.642c8590b2164p-5, 0x1.47ae147ae147bp-5,
                                   0x1.2f684bda12f68p-5, 0x1.1a7b9611a7b96p-5, 0x1.0842108421084p-5,
                                   0x1.f07c1f07c1f08p-6, 0x1.d41d41d41d41dp-6, 0x1.bacf914c1bad0p-6,
                                   0x1.a41a41a41a41ap-6, 0x1.8f9c18f9c18fap-6};
    static const double kLo[10] = {0.0, 0x1.5555555555555p-56, -0x1.999999999999ap-57, 0x1.2492492492492p-57,
                                   0x1.c71c71c71c71cp-58, -0x1.745d1745d1746p-59, -0x1.3b13b13b13b14p-58,
                                   0x1.1111111111111p-60, 0x1.e1e1e1e1e1e1ep-61, 0x1.af286bca1af28p-59};
    int e = 0;
    double m = std::frexp(x, &e);
    if (m < 0x1.6a09e667f3bcdp-1)
    {
        m *= 2.0;
        --e;
    }
    const DD s = dd_div(m - 1.0, two_sum(m, 1.0));
    const DD z = dd_mul(s, s);
    double q = kHi[20];
    for (int k = 19; k >= 10; --k)
        q = std::fma(q, z.hi, kHi[k]);
    DD P{q, 0.0};
    for (int k = 9; k >= 1; --k)
        P = dd_add({kHi[k], kLo[k]}, dd_mul(z, P));
    DD lm = dd_add(s, dd_mul(dd_mul(s, z), P));
    lm.hi *= 2.0;
    lm.lo *= 2.0;
    return dd_add(dd_mul({(double)e, 0.0}, {0x1.62e42fefa39efp-1, 0x1.abc9e3b39803fp-56}), lm).hi;
}

// RNG:98-101 (gaussian = normalDist_(generator_) * stddev + mean) with log_mode 1: libstdc++'s
// normal_distribution restated (polar method of Marsaglia and Bray, cached second value), log
// replaced by log_rn. log_mode 0 uses std::normal_distribution itself, as OMPL.
struct Gaussian
{
    int log_mode = 0;
    std::normal_distribution<> nd{0, 1};
    bool saved_available = false;
    double saved = 0.0;
    double operator()(std::mt19937 &gen, std::uniform_real_distribution<> &uni)
    {
        if (log_mode == 0)
            return nd(gen);
        double ret;
        if (saved_available)
        {
            saved_available = false;
            ret = saved;
        }
        else
        {
            double x, y, r2;
            do
            {
                x = 2.0 * uni(gen) - 1.0;
                y = 2.0 * uni(gen) - 1.0;
                r2 = x * x + y * y;
            } while (r2 > 1.0 || r2 == 0.0);
            const double mult = std::sqrt(-2.0 * log_rn(r2) / r2);
            saved = x * mult;
            saved_available = true;
            ret = y * mult;
        }
        return ret * 1.0 + 0.0;
    }
};
}  // namespace

void ora_log_rn(const double *x, long n, double *out)
{
    for (long i = 0; i < n; ++i)
        out[i] = log_rn(x[i]);
}

// RV:67-82 (clamped to the bounds) and SO2:58-62 (wrapped by enforceBounds), interleaved with
// sampleUniform calls (RV:45-53, SO2:46-49) on one RNG.
void ora_sample_script(const ora_space *d, unsigned seed, const int *kinds, const long *counts, int nops,
                       const double *mean, double stddev, int log_mode, double *out)
{
    Space s = make_space(d);
    std::mt19937 gen(seed);
    std::uniform_real_distribution<> uni{0, 1};
    Gaussian gauss;
    gauss.log_mode = log_mode;
    long rows = 0, mrows = 0;
    for (int k = 0; k < nops; ++k)
        for (long i = 0; i < counts[k]; ++i)
        {
            double *o = out + (size_t)(rows++) * s.dim;
            if (kinds[k] != 1)
            {
                for (int j = 0; j < s.dim; ++j)
                    o[j] = (s.high[j] - s.low[j]) * uni(gen) + s.low[j];
                continue;
            }
            const double *m = mean + (size_t)(mrows++) * s.dim;
            for (int j = 0; j < s.dim; ++j)
            {
                double v = gauss(gen, uni) * stddev + m[j];
                if (s.kind != ORA_SPACE_SO2)
                {
                    if (v < s.low[j])
                        v = s.low[j];
                    else if (v > s.high[j])
                        v = s.high[j];
                }
                o[j] = v;
            }
            if (s.kind == ORA_SPACE_SO2)
                enforce_bounds(s, o);
        }
}

void ora_is_valid(const ora_space *d, const ora_checker *c, const double *states, long n, unsigned char *out)
{
    Space s = make_space(d);
    parallel_rows(n, [&](long i) { out[i] = is_valid(s, c, states + (size_t)i * s.dim) ? 1 : 0; });
}

void ora_check_motion(const ora_space *d, const ora_checker *c, const double *s1, const double *s2, long n,
                      unsigned char *ok, unsigned char *ok_bisect, double *last_t, double *last_state, int *nd,
                      int *first_j)
{
    Space s = make_space(d);
    parallel_rows(n, [&](long i) {
        const double *a = s1 + (size_t)i * s.dim, *b = s2 + (size_t)i * s.dim;
        double lt = kNaN;
        int ndi = 0, fj = -1;
        bool r = check_motion_ordered(s, c, a, b, lt, ndi, fj);
        if (ok)
            ok[i] = r ? 1 : 0;
        if (ok_bisect)
            ok_bisect[i] = check_motion_bisect(s, c, a, b) ? 1 : 0;
        if (last_t)
            last_t[i] = lt;
        if (nd)
            nd[i] = ndi;
        if (first_j)
            first_j[i] = fj;
        if (last_state)
        {
            double *o = last_state + (size_t)i * s.dim;
            if (r)
                for (int k = 0; k < s.dim; ++k)
                    o[k] = kNaN;
            else
                interpolate(s, a, b, lt, o);  // DMV:67-68 / :80-81
        }
    });
}

// SI:288-299 and SI:301-341
int ora_check_motion_states(const ora_space *d, const ora_checker *c, const double *states, long count,
                            long *first_invalid, int *ok_bisect)
{
    Space s = make_space(d);
    auto valid = [&](long i) { return is_valid(s, c, states + (size_t)i * s.dim); };
    if (ok_bisect)
    {
        bool res = true;
        if (count > 0)
        {
            if (count > 1)
            {
                if (!valid(0) || !valid(count - 1))
                    res = false;
                else if (count > 2)
                {
                    std::queue<std::pair<long, long>> pos;
                    pos.emplace(0, count - 1);
                    while (!pos.empty())
                    {
                        auto x = pos.front();
                        long mid = (x.first + x.second) / 2;
                        if (!valid(mid))
                        {
                            res = false;
                            break;
                        }
                        pos.pop();
                        if (x.first < mid - 1)
                            pos.emplace(x.first, mid);
                        if (x.second > mid + 1)
                            pos.emplace(mid, x.second);
                    }
                }
            }
            else
                res = valid(0);
        }
        *ok_bisect = res ? 1 : 0;
    }
    for (long i = 0; i < count; ++i)
        if (!valid(i))
        {
            *first_invalid = i;
            return 0;
        }
    return 1;
}

// SI:215-286 with alloc = true
long ora_get_motion_states(const ora_space *d, const double *s1, const double *s2, unsigned count, int endpoints,
                           double *out)
{
    Space s = make_space(d);
    count++;
    long added = 0;
    auto row = [&](long r) { return out + (size_t)r * s.dim; };
    if (count < 2)
    {
        if (endpoints)
        {
            std::copy(s1, s1 + s.dim, row(0));
            std::copy(s2, s2 + s.dim, row(1));
            return 2;
        }
        return 0;
    }
    const long size = (long)count + (endpoints ? 1 : -1);
    if (endpoints && size > 0)
    {
        std::copy(s1, s1 + s.dim, row(0));
        added++;
    }
    for (unsigned j = 1; j < count && added < size; ++j)
    {
        interpolate(s, s1, s2, (double)j / (double)count, row(added));
        added++;
    }
    if (added < size && endpoints)
    {
        std::copy(s2, s2 + s.dim, row(added));
        added++;
    }
    return added;
}

void ora_knn(const ora_space *d, int algo, const double *pts, long npts, const double *q, long nq, int k, long *idx,
             double *dist)
{
    (void)algo;  // the restatement implements the exact (distance, index) order only
    Space s = make_space(d);
    parallel_rows(nq, [&](long i) {
        knn_one(s, pts, npts, npts, q + (size_t)i * s.dim, k, idx + (size_t)i * k, dist + (size_t)i * k);
    });
}

void ora_knn_prefix(const ora_space *d, const double *pts, long npts, const double *q, const long *limit, long nq,
                    int k, long *idx, double *dist)
{
    Space s = make_space(d);
    parallel_rows(nq, [&](long i) {
        knn_one(s, pts, npts, limit[i], q + (size_t)i * s.dim, k, idx + (size_t)i * k, dist + (size_t)i * k);
    });
}

// NNL:135-142: keep distance(point, query) <= r, sorted ascending; ties by insertion index.
long ora_radius(const ora_space *d, int algo, const double *pts, long npts, const double *q, long nq, double r,
                long *counts, long *idx, double *dist, long cap)
{
    (void)algo;
    Space s = make_space(d);
    std::vector<std::vector<std::pair<double, long>>> res(nq);
    parallel_rows(nq, [&](long i) {
        const double *qq = q + (size_t)i * s.dim;
        for (long j = 0; j < npts; ++j)
        {
            double dd = distance(s, pts + (size_t)j * s.dim, qq);
            if (dd <= r)
                res[i].emplace_back(dd, j);
        }
        std::sort(res[i].begin(), res[i].end());
    });
    long total = 0;
    for (long i = 0; i < nq; ++i)
    {
        counts[i] = (long)res[i].size();
        for (auto &e : res[i])
        {
            if (idx && dist && total < cap)
            {
                idx[total] = e.second;
                dist[total] = e.first;
            }
            total++;
        }
    }
    return total;
}

}  // extern "C"
