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

// Uniform-grid broad phase for the DH sphere checker (a speed-up of this restatement only; the
// boolean is that of gbompl_oracle::dh_valid, which tests every robot sphere against every world
// obstacle). World sphere o is listed in every cell that its box [o - R, o + R] reaches, with R =
// r_o + r_robot + 1e-6 (a world box: its half extent + r_robot + 1e-6 per axis); cells are found with the monotone map floor((v - x0) / h), so a robot
// sphere centre inside that box always lands in a listed cell, and a centre outside every box
// (including outside the grid) is more than r_o + r_robot + 1e-6 from every world centre (more than
// r_robot + 1e-6 from every world box along some axis), where the
// FP64 narrow phase cannot report a hit. The narrow phase of the listed candidates is
// dh_valid's expression, evaluated on the same centres.
struct DhGrid
{
    double x0[3] = {0, 0, 0}, inv_h = 1.0;
    int nc = 0, stride = 4;
    bool boxes = false;
    std::vector<int> start, items;

    int cell_coord(double v, int a) const
    {
        double f = std::floor((v - x0[a]) * inv_h);
        return f < 0.0 ? -1 : (f >= (double)nc ? nc : (int)f);
    }

    void build(const ora_checker *c)
    {
        const long n = c->n_obstacles;
        if (n <= 0)
            return;
        boxes = c->kind == ORA_CHECK_DH_BOXES;
        stride = boxes ? 6 : 4;
        // reach of obstacle j along axis a: its radius (or half extent) + the robot sphere radius + 1e-6
        auto R_of = [&](const double *o, int a) { return (boxes ? o[3 + a] : o[3]) + c->sphere_radius + 1e-6; };
        double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
        for (long j = 0; j < n; ++j)
        {
            const double *o = c->obstacles + stride * j;
            for (int a = 0; a < 3; ++a)
            {
                lo[a] = std::min(lo[a], o[a] - R_of(o, a));
                hi[a] = std::max(hi[a], o[a] + R_of(o, a));
            }
        }
        nc = (int)std::min(64.0, std::max(4.0, std::ceil(1.5 * std::cbrt((double)n))));
        double ext = 0.0;
        for (int a = 0; a < 3; ++a)
            ext = std::max(ext, hi[a] - lo[a]);
        const double h = ext * (1.0 + 1e-9) / nc;
        inv_h = 1.0 / h;
        for (int a = 0; a < 3; ++a)
            x0[a] = lo[a];
        const size_t cells = (size_t)nc * nc * nc;
        std::vector<int> count(cells + 1, 0);
        auto each = [&](long j, auto f) {
            const double *o = c->obstacles + stride * j;
            int l[3], u[3];
            for (int a = 0; a < 3; ++a)
            {
                l[a] = std::max(0, cell_coord(o[a] - R_of(o, a), a));
                u[a] = std::min(nc - 1, cell_coord(o[a] + R_of(o, a), a));
            }
            for (int x = l[0]; x <= u[0]; ++x)
                for (int y = l[1]; y <= u[1]; ++y)
                    for (int z = l[2]; z <= u[2]; ++z)
                        f(((size_t)x * nc + y) * nc + z);
        };
        for (long j = 0; j < n; ++j)
            each(j, [&](size_t cell) { count[cell + 1]++; });
        start.assign(cells + 1, 0);
        for (size_t i = 0; i < cells; ++i)
            start[i + 1] = start[i] + count[i + 1];
        items.resize((size_t)start[cells]);
        std::vector<int> fill(start.begin(), start.end() - 1);
        for (long j = 0; j < n; ++j)
            each(j, [&](size_t cell) { items[(size_t)fill[cell]++] = (int)j; });
    }

    bool valid(const ora_checker *c, const double *q) const
    {
        const int ns = c->n_joints * c->spheres_per_link;
        double ctr[3 * 64 * 16];
        std::vector<double> big;
        double *cp = ctr;
        if (ns > 64 * 16)
        {
            big.resize(3 * (size_t)ns);
            cp = big.data();
        }
        gbompl_oracle::dh_sphere_centres(c, q, cp);
        const double rs = c->sphere_radius;
        for (int s = 0; s < ns; ++s)
        {
            const double *p = cp + 3 * s;
            int ix = cell_coord(p[0], 0), iy = cell_coord(p[1], 1), iz = cell_coord(p[2], 2);
            if (ix < 0 || iy < 0 || iz < 0 || ix >= nc || iy >= nc || iz >= nc)
                continue;
            const size_t cell = ((size_t)ix * nc + iy) * nc + iz;
            for (int t = start[cell]; t < start[cell + 1]; ++t)
                if (gbompl_oracle::dh_pair_hits(p, c->obstacles + stride * (size_t)items[(size_t)t], rs, boxes))
                    return false;
        }
        return true;
    }
};

// A checker as the batch calls use it: the description plus, for the DH arm, its grid.
struct Checker
{
    const ora_checker *c;
    DhGrid grid;
    bool use_grid = false;
};

Checker make_checker(const ora_checker *c, bool brute = false)
{
    Checker k;
    k.c = c;
    if ((c->kind == ORA_CHECK_DH_SPHERES || c->kind == ORA_CHECK_DH_BOXES) && !brute && c->n_obstacles > 64 &&
        c->spheres_per_link <= 16 &&
        c->n_joints <= 64)
    {
        k.grid.build(c);
        k.use_grid = true;
    }
    return k;
}

bool is_valid(const Space &s, const Checker &k, const double *q)
{
    const ora_checker *c = k.c;
    switch (c->kind)
    {
        case ORA_CHECK_CIRCLES:
            return circles_valid(c, q);
        case ORA_CHECK_CHAIN_SEGMENTS:
            return chain_valid(s, c, q);
        case ORA_CHECK_DH_SPHERES:
        case ORA_CHECK_DH_BOXES:
            return k.use_grid ? k.grid.valid(c, q) : gbompl_oracle::dh_valid(c, q);
        default:
            return true;
    }
}

// DMV:48-91 (ordered variant). Returns result; fills lastValid.second, nd and the first invalid index.
bool check_motion_ordered(const Space &s, const Checker &c, const double *s1, const double *s2, double &last_t,
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
bool check_motion_bisect(const Space &s, const Checker &c, const double *s1, const double *s2)
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

// Chain metric with per-row link directions precomputed: KC:105-121 evaluates cos/sin of
// theta = q_0 + ... + q_i of each argument inside the pair loop; here theta is accumulated in the
// same order once per row and the pair loop performs the same additions, square roots and final
// multiplication on the same values, so distances are bitwise those of distance().
struct ChainTrig
{
    int dim = 0;
    std::vector<double> cs;  // per row: cos(theta_0..theta_{dim-1}), then sin(...)
    const double *row(long r) const { return cs.data() + (size_t)r * 2 * dim; }
};

ChainTrig chain_trig(const Space &s, const double *rows, long n)
{
    ChainTrig t;
    t.dim = s.dim;
    t.cs.resize((size_t)n * 2 * s.dim);
    parallel_rows(n, [&](long r) {
        const double *q = rows + (size_t)r * s.dim;
        double *o = t.cs.data() + (size_t)r * 2 * s.dim;
        double theta = 0.;
        for (int i = 0; i < s.dim; ++i)
        {
            theta += q[i];
            o[i] = std::cos(theta);
            o[s.dim + i] = std::sin(theta);
        }
    });
    return t;
}

inline double chain_distance_pre(const Space &s, const double *a, const double *b)
{
    const int n = s.dim;
    double dx = 0., dy = 0., dist = 0.;
    for (int i = 0; i < n; ++i)
    {
        dx += a[i] - b[i];
        dy += a[n + i] - b[n + i];
        dist += std::sqrt(dx * dx + dy * dy);
    }
    return dist * s.link;
}

// distance(point j, query i) of the batch calls, with the chain's precomputed directions.
struct PairMetric
{
    const Space &s;
    const double *pts, *q;
    ChainTrig tp, tq;
    bool chain;
    PairMetric(const Space &s_, const double *p, long np, const double *q_, long nq)
        : s(s_), pts(p), q(q_), chain(s_.kind == ORA_SPACE_KINEMATIC_CHAIN)
    {
        if (chain)
        {
            tp = chain_trig(s, p, np);
            tq = chain_trig(s, q_, nq);
        }
    }
    double operator()(long j, long i) const
    {
        if (chain)
            return chain_distance_pre(s, tp.row(j), tq.row(i));
        return distance(s, pts + (size_t)j * s.dim, q + (size_t)i * s.dim);
    }
};

// Exact k nearest by (distance, insertion index) for every query, each query seeing the points
// [0, limit[i]) (all points when limit is null): tiles of 32 queries scan tiles of 2048 points so that
// a point tile stays in cache for the whole query tile. Points are visited in increasing index, so a
// point whose distance equals the current k-th never enters (the earlier index wins the tie), which is
// the (distance, index) order of knn_one.
void knn_blocked(const PairMetric &m, long npts, long nq, const long *limit, int k, long *idx, double *dist)
{
    const long QT = 32, PT = 2048;
    const long tiles = (nq + QT - 1) / QT;
    parallel_rows(tiles, [&](long t) {
        const long q0 = t * QT, q1 = std::min(nq, q0 + QT);
        std::vector<double> kd((size_t)(q1 - q0) * k);
        std::vector<long> ki((size_t)(q1 - q0) * k);
        std::vector<int> cnt((size_t)(q1 - q0), 0);
        long lmax = 0;
        for (long i = q0; i < q1; ++i)
            lmax = std::max(lmax, limit ? std::min(limit[i], npts) : npts);
        for (long p0 = 0; p0 < lmax; p0 += PT)
        {
            const long p1 = std::min(lmax, p0 + PT);
            for (long i = q0; i < q1; ++i)
            {
                const long lim = std::min(p1, limit ? std::min(limit[i], npts) : npts);
                double *D = kd.data() + (size_t)(i - q0) * k;
                long *I = ki.data() + (size_t)(i - q0) * k;
                int &c = cnt[(size_t)(i - q0)];
                for (long j = p0; j < lim; ++j)
                {
                    const double d = m(j, i);
                    if (c == k && !(d < D[k - 1]))
                        continue;
                    int pos = c < k ? c++ : k - 1;
                    while (pos > 0 && d < D[pos - 1])
                    {
                        D[pos] = D[pos - 1];
                        I[pos] = I[pos - 1];
                        --pos;
                    }
                    D[pos] = d;
                    I[pos] = j;
                }
            }
        }
        for (long i = q0; i < q1; ++i)
            for (int j = 0; j < k; ++j)
            {
                const int c = cnt[(size_t)(i - q0)];
                idx[(size_t)i * k + j] = j < c ? ki[(size_t)(i - q0) * k + j] : -1;
                dist[(size_t)i * k + j] =
                    j < c ? kd[(size_t)(i - q0) * k + j] : std::numeric_limits<double>::infinity();
            }
    });
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
    Checker k = make_checker(c);
    parallel_rows(n, [&](long i) { out[i] = is_valid(s, k, states + (size_t)i * s.dim) ? 1 : 0; });
}

void ora_is_valid_brute(const ora_space *d, const ora_checker *c, const double *states, long n, unsigned char *out)
{
    Space s = make_space(d);
    Checker k = make_checker(c, true);
    parallel_rows(n, [&](long i) { out[i] = is_valid(s, k, states + (size_t)i * s.dim) ? 1 : 0; });
}

void ora_check_motion(const ora_space *d, const ora_checker *c, const double *s1, const double *s2, long n,
                      unsigned char *ok, unsigned char *ok_bisect, double *last_t, double *last_state, int *nd,
                      int *first_j)
{
    Space s = make_space(d);
    Checker k = make_checker(c);
    parallel_rows(n, [&](long i) {
        const double *a = s1 + (size_t)i * s.dim, *b = s2 + (size_t)i * s.dim;
        double lt = kNaN;
        int ndi = 0, fj = -1;
        bool r = check_motion_ordered(s, k, a, b, lt, ndi, fj);
        if (ok)
            ok[i] = r ? 1 : 0;
        if (ok_bisect)
            ok_bisect[i] = check_motion_bisect(s, k, a, b) ? 1 : 0;
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
    Checker k = make_checker(c);
    auto valid = [&](long i) { return is_valid(s, k, states + (size_t)i * s.dim); };
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
    PairMetric m(s, pts, npts, q, nq);
    knn_blocked(m, npts, nq, nullptr, k, idx, dist);
}

// NearestNeighborsSqrtApprox.h:91-125: the structure is NearestNeighborsLinear's vector (insertion order,
// removals erase), checks_ = 1 + floor(sqrt(size)) after every add / remove; nearest() examines
// positions (j checks_ + offset_) % n for j < checks_, keeps the first strict minimum of
// distFun_(element, query), then offset_ = (offset_ + 1) % checks_.
unsigned long ora_nn_sqrt_approx(const ora_space *d, const double *pts, long npts, const long *remove, long nrem,
                                 const double *q, long nq, long *idx, double *dist)
{
    Space s = make_space(d);
    std::vector<long> data((size_t)npts);
    for (long i = 0; i < npts; ++i)
        data[(size_t)i] = i;
    for (long r = 0; r < nrem; ++r)
    {
        auto it = std::find(data.begin(), data.end(), remove[r]);
        if (it != data.end())
            data.erase(it);
    }
    const size_t n = data.size();
    const size_t checks = 1 + (size_t)std::floor(std::sqrt((double)n));
    size_t offset = 0;
    for (long i = 0; i < nq; ++i)
    {
        const double *qi = q + (size_t)i * s.dim;
        size_t pos = n;
        double dmin = 0.0;
        if (n > 0)
        {
            for (size_t j = 0; j < checks; ++j)
            {
                const size_t p = (j * checks + offset) % n;
                const double dd = distance(s, pts + (size_t)data[p] * s.dim, qi);
                if (pos == n || dmin > dd)
                {
                    pos = p;
                    dmin = dd;
                }
            }
            offset = (offset + 1) % checks;
        }
        idx[i] = pos == n ? -1 : data[pos];
        dist[i] = pos == n ? std::numeric_limits<double>::infinity() : dmin;
    }
    return n ? (unsigned long)offset : 0;
}

void ora_knn_prefix(const ora_space *d, const double *pts, long npts, const double *q, const long *limit, long nq,
                    int k, long *idx, double *dist)
{
    Space s = make_space(d);
    PairMetric m(s, pts, npts, q, nq);
    knn_blocked(m, npts, nq, limit, k, idx, dist);
}

// NNL:135-142: keep distance(point, query) <= r, sorted ascending; ties by insertion index.
long ora_radius(const ora_space *d, int algo, const double *pts, long npts, const double *q, long nq, double r,
                long *counts, long *idx, double *dist, long cap)
{
    (void)algo;
    Space s = make_space(d);
    PairMetric m(s, pts, npts, q, nq);
    std::vector<std::vector<std::pair<double, long>>> res(nq);
    parallel_rows(nq, [&](long i) {
        for (long j = 0; j < npts; ++j)
        {
            double dd = m(j, i);
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

namespace
{
// ------------------------------------------------ correctly rounded sin / cos (double-double)
// Used to measure how often the C library's sin/cos differ from the correctly rounded value
// (ora_trig_rounding). Method: Cody and Waite's additive reduction x = k*pi/2 + y with pi/2 split
// into four doubles (C1, C2: 33 significant bits, so k*C1 and k*C2 are exact for |k| < 2^20; C3, C4:
// 53 bits; x - k*C1 is exact by Sterbenz's lemma), y carried as a double-double; then the Taylor
// series sin y = y * sum (-1)^n y^2n/(2n+1)! (n <= 14) and cos y = sum (-1)^n y^2n/(2n)! (n <= 15)
// evaluated by Horner's rule in double-double (truncation < 1e-33 for |y| <= pi/4); the quadrant
// k mod 4 picks +-sin y or +-cos y. Constants: pi/2's splits and the coefficients rounded to
// double-doubles (hi = nearest double, lo = nearest double to the remainder), as derived from their
// definitions with 400-bit arithmetic. A result whose double-double is within 2^-98 relative of a
// rounding boundary is reported as undecided (never met on the tested arguments).
const double kC1 = 0x1.921fb54400000p+0, kC2 = 0x1.0b4611a600000p-34, kC3 = 0x1.3198a2e037073p-69,
             kC4 = 0x1.129024e088a68p-123, kTwoOverPi = 0x1.45f306dc9c883p-1;
const DD kSinC[15] = {{0x1.0000000000000p+0, 0.0},
                      {-0x1.5555555555555p-3, -0x1.5555555555555p-57},
                      {0x1.1111111111111p-7, 0x1.1111111111111p-63},
                      {-0x1.a01a01a01a01ap-13, -0x1.a01a01a01a01ap-73},
                      {0x1.71de3a556c734p-19, -0x1.c154f8ddc6c00p-73},
                      {-0x1.ae64567f544e4p-26, 0x1.c062e06d1f209p-80},
                      {0x1.6124613a86d09p-33, 0x1.f28e0cc748ebep-87},
                      {-0x1.ae7f3e733b81fp-41, -0x1.1d8656b0ee8cbp-97},
                      {0x1.952c77030ad4ap-49, 0x1.ac981465ddc6cp-103},
                      {-0x1.2f49b46814157p-57, -0x1.2650f61dbdcb4p-112},
                      {0x1.71b8ef6dcf572p-66, -0x1.d043ae40c4647p-120},
                      {-0x1.761b41316381ap-75, 0x1.3423c7d91404fp-130},
                      {0x1.3f3ccdd165fa9p-84, -0x1.58ddadf344487p-139},
                      {-0x1.d1ab1c2dccea3p-94, -0x1.054d0c78aea14p-149},
                      {0x1.259f98b4358adp-103, 0x1.eaf8c39dd9bc5p-157}};
const DD kCosC[16] = {{0x1.0000000000000p+0, 0.0},
                      {-0x1.0000000000000p-1, 0.0},
                      {0x1.5555555555555p-5, 0x1.5555555555555p-59},
                      {-0x1.6c16c16c16c17p-10, 0x1.f49f49f49f49fp-65},
                      {0x1.a01a01a01a01ap-16, 0x1.a01a01a01a01ap-76},
                      {-0x1.27e4fb7789f5cp-22, -0x1.cbbc05b4fa99ap-76},
                      {0x1.1eed8eff8d898p-29, -0x1.2aec959e14c06p-83},
                      {-0x1.93974a8c07c9dp-37, -0x1.05d6f8a2efd1fp-92},
                      {0x1.ae7f3e733b81fp-45, 0x1.1d8656b0ee8cbp-101},
                      {-0x1.6827863b97d97p-53, -0x1.eec01221a8b0bp-107},
                      {0x1.e542ba4020225p-62, 0x1.ea72b4afe3c2fp-120},
                      {-0x1.0ce396db7f853p-70, 0x1.aebcdbd20331cp-124},
                      {0x1.f2cf01972f578p-80, -0x1.9ada5fcc1ab14p-135},
                      {-0x1.88e85fc6a4e5ap-89, 0x1.71c37ebd16540p-143},
                      {0x1.0a18a2635085dp-98, 0x1.b9e2e28e1aa54p-153},
                      {-0x1.3932c5047d60ep-108, -0x1.832b7b530a627p-162}};

// Rounds a normalized double-double to the nearest double; `hard` is set when the double-double is
// too close to a rounding boundary for its own error (2^-98 relative) to settle the rounding.
double dd_round(DD v, bool &hard)
{
    const DD r = fast_two_sum(v.hi, v.lo);
    const double h = r.hi;
    if (h == 0.0 || !std::isfinite(h))
        return h;
    const double up = std::nextafter(h, HUGE_VAL) - h, dn = h - std::nextafter(h, -HUGE_VAL);
    const double tol = std::fabs(h) * 0x1p-98;
    if (std::fabs(std::fabs(r.lo) - 0.5 * (r.lo > 0 ? up : dn)) <= tol)
        hard = true;
    return h;
}

// sin and cos of x (|x| < 2^20) as double-doubles.
void dd_sincos(double x, DD &sn, DD &cs)
{
    const double k = std::nearbyint(x * kTwoOverPi);
    const double r = x - k * kC1;                     // exact
    DD y = two_sum(r, -(k * kC2));                    // k*C2 exact
    const double p3 = k * kC3, e3 = std::fma(k, kC3, -p3);
    y = dd_add(y, {-p3, -e3});
    y = dd_add(y, {-(k * kC4), 0.0});
    const DD z = dd_mul(y, y);
    DD s = kSinC[14];
    for (int n = 13; n >= 0; --n)
        s = dd_add(dd_mul(s, z), kSinC[n]);
    s = dd_mul(s, y);
    DD c = kCosC[15];
    for (int n = 14; n >= 0; --n)
        c = dd_add(dd_mul(c, z), kCosC[n]);
    const long q = (long)k & 3;
    const DD ns{-s.hi, -s.lo}, nc{-c.hi, -c.lo};
    sn = q == 0 ? s : (q == 1 ? c : (q == 2 ? ns : nc));
    cs = q == 0 ? c : (q == 1 ? ns : (q == 2 ? nc : s));
}
}  // namespace

extern "C" {

// Correctly rounded sin/cos (restatement above): out_s/out_c per argument; returns the number of
// arguments whose rounding the double-double could not settle (their outputs are the nearest
// double to the double-double).
long ora_sincos_rn(const double *x, long n, double *out_s, double *out_c)
{
    std::atomic<long> hard{0};
    parallel_rows(n, [&](long i) {
        DD s, c;
        dd_sincos(x[i], s, c);
        bool h = false;
        out_s[i] = dd_round(s, h);
        out_c[i] = dd_round(c, h);
        if (h)
            hard++;
    });
    return hard.load();
}

// How often the C library's sin and cos differ from the correctly rounded value on x[0..n):
// counts[0] = sin misrounded, counts[1] = cos misrounded, counts[2] = undecided roundings (skipped),
// counts[3] = largest difference in units in the last place seen.
void ora_trig_rounding(const double *x, long n, long *counts)
{
    std::atomic<long> ms{0}, mc{0}, hard{0}, worst{0};
    parallel_rows(n, [&](long i) {
        DD s, c;
        dd_sincos(x[i], s, c);
        bool h = false;
        const double rs = dd_round(s, h), rc = dd_round(c, h);
        if (h)
        {
            hard++;
            return;
        }
        const double ls = std::sin(x[i]), lc = std::cos(x[i]);
        auto ulps = [](double a, double b) {
            long d = 0;
            while (a != b && d < 1000)
            {
                a = std::nextafter(a, b);
                ++d;
            }
            return d;
        };
        if (ls != rs)
        {
            ms++;
            long u = ulps(ls, rs);
            long w = worst.load();
            while (u > w && !worst.compare_exchange_weak(w, u))
            {
            }
        }
        if (lc != rc)
        {
            mc++;
            long u = ulps(lc, rc);
            long w = worst.load();
            while (u > w && !worst.compare_exchange_weak(w, u))
            {
            }
        }
    });
    counts[0] = ms.load();
    counts[1] = mc.load();
    counts[2] = hard.load();
    counts[3] = worst.load();
}

// PRM roadmap (geometric/planners/prm/src/PRM.cpp:570-604 with KStrategy k, ConnectionStrategy.h:77-81,
// and the default connection filter): n_samples draws of the space's uniform sampler seeded with
// `seed` (the sampler of ora_sample_uniform); milestone m = the m-th valid sample; its neighbours are
// the k nearest among milestones 0..m-1 by (distance, index); every neighbour n is connected when
// the ordered DiscreteMotionValidator accepts the motion n -> m. Writes the milestones' sample
// indices (capacity n_samples) and the accepted edges (src = n, dst = m) in attempt order (m
// ascending, neighbours by increasing distance), at most edge_cap of them; returns the number of
// accepted edges; *candidates = connection attempts, *n_milestones = milestones.
long ora_prm_roadmap(const ora_space *d, const ora_checker *c, unsigned seed, long n_samples, int k,
                     long *n_milestones, long *sample_index, long *edge_src, long *edge_dst, long edge_cap,
                     long *candidates)
{
    Space s = make_space(d);
    Checker chk = make_checker(c);
    std::vector<double> samples((size_t)n_samples * s.dim);
    ora_sample_uniform(d, seed, n_samples, samples.data());
    std::vector<unsigned char> valid((size_t)n_samples);
    parallel_rows(n_samples, [&](long i) { valid[(size_t)i] = is_valid(s, chk, samples.data() + (size_t)i * s.dim); });
    std::vector<double> ms;
    long m = 0;
    for (long i = 0; i < n_samples; ++i)
        if (valid[(size_t)i])
        {
            sample_index[m++] = i;
            ms.insert(ms.end(), samples.begin() + (size_t)i * s.dim, samples.begin() + (size_t)(i + 1) * s.dim);
        }
    *n_milestones = m;
    samples.clear();
    samples.shrink_to_fit();
    std::vector<long> limit((size_t)m);
    for (long i = 0; i < m; ++i)
        limit[(size_t)i] = i;
    std::vector<long> nbr((size_t)m * k);
    std::vector<double> nd((size_t)m * k);
    PairMetric met(s, ms.data(), m, ms.data(), m);
    knn_blocked(met, m, m, limit.data(), k, nbr.data(), nd.data());
    std::vector<long> cs, cd;
    for (long i = 0; i < m; ++i)
        for (int j = 0; j < k; ++j)
            if (nbr[(size_t)i * k + j] >= 0)
            {
                cs.push_back(nbr[(size_t)i * k + j]);
                cd.push_back(i);
            }
    const long nc = (long)cs.size();
    *candidates = nc;
    std::vector<unsigned char> ok((size_t)nc);
    parallel_rows(nc, [&](long e) {
        double lt = kNaN;
        int ndi = 0, fj = -1;
        ok[(size_t)e] = check_motion_ordered(s, chk, ms.data() + (size_t)cs[(size_t)e] * s.dim,
                                             ms.data() + (size_t)cd[(size_t)e] * s.dim, lt, ndi, fj)
                            ? 1
                            : 0;
    });
    long ne = 0;
    for (long e = 0; e < nc; ++e)
        if (ok[(size_t)e])
        {
            if (ne < edge_cap)
            {
                edge_src[ne] = cs[(size_t)e];
                edge_dst[ne] = cd[(size_t)e];
            }
            ++ne;
        }
    return ne;
}

}  // extern "C"
