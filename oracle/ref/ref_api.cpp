/*
 * ORACLE (test infrastructure only): the oracle C API implemented with OMPL's OWN classes.
 *
 * oracle/ref/Makefile compiles this file together with OMPL's unmodified sources
 * (StateSpace, RealVectorStateSpace, SO2StateSpace, StateSampler, DiscreteMotionValidator,
 * SpaceInformation, RandomNumbers, ...) and the header-only NearestNeighbors* structures, and the
 * kinematic-chain space/checker from demos/KinematicChain.h, into oracle/_ref/libompl_ref.so.
 * Everything below only wires those classes to the C API; the arithmetic is OMPL's.
 *
 * Two pieces are not in OMPL's library sources and are supplied here:
 *   - the circle checker predicate, which lives in OMPL's test tree
 *     (tests/resources/circles2D.h:141-151, a header that also pulls in Eigen's QR solver);
 *   - the wrap-L2 joint space and the DH sphere arm, which have no OMPL counterpart.
 */
#include "ompl/base/SpaceInformation.h"
#include "ompl/base/DiscreteMotionValidator.h"
#include "ompl/base/spaces/RealVectorStateSpace.h"
#include "ompl/base/spaces/SO2StateSpace.h"
#include "ompl/datastructures/NearestNeighborsGNAT.h"
#include "ompl/datastructures/NearestNeighborsGNATNoThreadSafety.h"
#include "ompl/datastructures/NearestNeighborsLinear.h"
#include "ompl/datastructures/NearestNeighborsSqrtApprox.h"
#include "ompl/util/RandomNumbers.h"
#include "KinematicChain.h"

#include "../oracle_api.h"
#include "../dh_arm.h"

#include <cmath>
#include <limits>
#include <memory>
#include <vector>

namespace ob = ompl::base;

namespace
{
constexpr double kPi = boost::math::double_constants::pi;
const double kNaN = std::numeric_limits<double>::quiet_NaN();

// Joint space with wrap-around L2 (no OMPL counterpart): a RealVectorStateSpace on [-pi,pi]^dim whose
// distance is L2 over per-joint shortest angular differences, interpolation is the per-joint shortest
// arc (as KinematicChainSpace::interpolate) and extent is sqrt(sum pi^2).
class WrapL2Space : public ob::RealVectorStateSpace
{
public:
    explicit WrapL2Space(unsigned dim) : ob::RealVectorStateSpace(dim)
    {
        setBounds(-kPi, kPi);
    }
    double getMaximumExtent() const override
    {
        double e = 0.0;
        for (unsigned i = 0; i < dimension_; ++i)
            e += kPi * kPi;
        return std::sqrt(e);
    }
    double distance(const ob::State *a, const ob::State *b) const override
    {
        const double *x = a->as<StateType>()->values, *y = b->as<StateType>()->values;
        double sum = 0.0;
        for (unsigned i = 0; i < dimension_; ++i)
        {
            double d = std::fabs(x[i] - y[i]);
            if (d > kPi)
                d = 2.0 * kPi - d;
            sum += d * d;
        }
        return std::sqrt(sum);
    }
    void interpolate(const ob::State *from, const ob::State *to, double t, ob::State *state) const override
    {
        const double *f = from->as<StateType>()->values, *o = to->as<StateType>()->values;
        double *s = state->as<StateType>()->values;
        for (unsigned i = 0; i < dimension_; ++i)
        {
            double diff = o[i] - f[i];
            if (std::fabs(diff) <= kPi)
                s[i] = f[i] + diff * t;
            else
            {
                if (diff > 0.0)
                    diff = 2.0 * kPi - diff;
                else
                    diff = -2.0 * kPi - diff;
                s[i] = f[i] - diff * t;
                if (s[i] > kPi)
                    s[i] -= 2.0 * kPi;
                else if (s[i] < -kPi)
                    s[i] += 2.0 * kPi;
            }
        }
    }
    void enforceBounds(ob::State *state) const override
    {
        double *v = state->as<StateType>()->values;
        for (unsigned i = 0; i < dimension_; ++i)
        {
            double x = std::fmod(v[i], 2.0 * kPi);
            if (x < -kPi)
                x += 2.0 * kPi;
            else if (x >= kPi)
                x -= 2.0 * kPi;
            v[i] = x;
        }
    }
};

// Point robot vs circles; predicate of tests/resources/circles2D.h:141-151 (r2 = r*r, :51).
class CirclesChecker : public ob::StateValidityChecker
{
public:
    CirclesChecker(ob::SpaceInformation *si, const ora_checker *c) : ob::StateValidityChecker(si)
    {
        for (long i = 0; i < c->n_obstacles; ++i)
            circles_.push_back({c->obstacles[3 * i], c->obstacles[3 * i + 1], c->obstacles[3 * i + 2],
                                c->obstacles[3 * i + 2] * c->obstacles[3 * i + 2]});
    }
    bool isValid(const ob::State *state) const override
    {
        const double *xy = state->as<ob::RealVectorStateSpace::StateType>()->values;
        for (const auto &c : circles_)
        {
            double dx = c[0] - xy[0];
            double dy = c[1] - xy[1];
            if (dx * dx + dy * dy < c[3])
                return false;
        }
        return true;
    }

private:
    std::vector<std::array<double, 4>> circles_;
};

class DHChecker : public ob::StateValidityChecker
{
public:
    DHChecker(ob::SpaceInformation *si, const ora_checker *c) : ob::StateValidityChecker(si), c_(*c)
    {
    }
    bool isValid(const ob::State *state) const override
    {
        return gbompl_oracle::dh_valid(&c_, state->as<ob::RealVectorStateSpace::StateType>()->values);
    }

private:
    ora_checker c_;
};

// Forwards to the configured checker and counts calls, so the ordered DiscreteMotionValidator run
// reveals which checked state failed first.
class CountingChecker : public ob::StateValidityChecker
{
public:
    CountingChecker(ob::SpaceInformation *si, ob::StateValidityCheckerPtr inner)
      : ob::StateValidityChecker(si), inner_(std::move(inner))
    {
    }
    bool isValid(const ob::State *state) const override
    {
        ++calls;
        return inner_->isValid(state);
    }
    mutable long calls = 0;

private:
    ob::StateValidityCheckerPtr inner_;
};

struct Built
{
    Environment env;
    ob::StateSpacePtr space;
    ob::SpaceInformationPtr si;
    std::shared_ptr<CountingChecker> counter;
    unsigned dim = 0;
};

std::unique_ptr<Built> build(const ora_space *d, const ora_checker *c)
{
    auto b = std::make_unique<Built>();
    b->dim = d->dim;
    switch (d->kind)
    {
        case ORA_SPACE_SO2:
            b->space = std::make_shared<ob::SO2StateSpace>();
            break;
        case ORA_SPACE_KINEMATIC_CHAIN:
            if (c && c->kind == ORA_CHECK_CHAIN_SEGMENTS)
                for (long i = 0; i < c->n_obstacles; ++i)
                    b->env.emplace_back(c->obstacles[4 * i], c->obstacles[4 * i + 1], c->obstacles[4 * i + 2],
                                        c->obstacles[4 * i + 3]);
            b->space = std::make_shared<KinematicChainSpace>(d->dim, d->link_length, &b->env);
            break;
        case ORA_SPACE_WRAP_L2:
            b->space = std::make_shared<WrapL2Space>(d->dim);
            break;
        default:
        {
            auto rv = std::make_shared<ob::RealVectorStateSpace>(d->dim);
            ob::RealVectorBounds bounds(d->dim);
            for (int i = 0; i < d->dim; ++i)
            {
                bounds.low[i] = d->low[i];
                bounds.high[i] = d->high[i];
            }
            rv->setBounds(bounds);
            b->space = rv;
        }
    }
    b->space->setLongestValidSegmentFraction(d->lvs_fraction);
    b->space->setValidSegmentCountFactor(d->factor);
    b->si = std::make_shared<ob::SpaceInformation>(b->space);
    ob::StateValidityCheckerPtr inner;
    int kind = c ? c->kind : ORA_CHECK_ALL_VALID;
    if (kind == ORA_CHECK_CIRCLES)
        inner = std::make_shared<CirclesChecker>(b->si.get(), c);
    else if (kind == ORA_CHECK_CHAIN_SEGMENTS)
        inner = std::make_shared<KinematicChainValidityChecker>(b->si);
    else if (kind == ORA_CHECK_DH_SPHERES || kind == ORA_CHECK_DH_BOXES)
        inner = std::make_shared<DHChecker>(b->si.get(), c);
    else
        inner = std::make_shared<ob::AllValidStateValidityChecker>(b->si.get());
    b->counter = std::make_shared<CountingChecker>(b->si.get(), inner);
    b->si->setStateValidityChecker(b->counter);
    b->si->setup();
    return b;
}

struct StateRows
{
    const Built &b;
    std::vector<ob::State *> v;
    StateRows(const Built &bb, const double *rows, long n) : b(bb), v(n)
    {
        for (long i = 0; i < n; ++i)
        {
            v[i] = b.si->allocState();
            if (rows)
                b.space->copyFromReals(v[i], std::vector<double>(rows + (size_t)i * b.dim, rows + (size_t)(i + 1) * b.dim));
        }
    }
    ~StateRows()
    {
        for (auto *s : v)
            b.si->freeState(s);
    }
};

void to_row(const Built &b, const ob::State *s, double *out)
{
    std::vector<double> r;
    b.space->copyToReals(r, s);
    for (unsigned k = 0; k < b.dim; ++k)
        out[k] = r[k];
}

template <class Base>
class SeededSampler : public Base
{
public:
    SeededSampler(const ob::StateSpace *s, unsigned seed) : Base(s)
    {
        this->rng_.setLocalSeed(seed);
    }
};

ob::StateSamplerPtr seeded_sampler(const Built &b, int kind, unsigned seed)
{
    if (kind == ORA_SPACE_SO2)
        return std::make_shared<SeededSampler<ob::SO2StateSampler>>(b.space.get(), seed);
    return std::make_shared<SeededSampler<ob::RealVectorStateSampler>>(b.space.get(), seed);
}

std::unique_ptr<ompl::NearestNeighbors<long>> make_nn(int algo)
{
    switch (algo)
    {
        case ORA_NN_REF_GNAT:
            return std::make_unique<ompl::NearestNeighborsGNAT<long>>();
        case ORA_NN_REF_GNAT_NTS:
            return std::make_unique<ompl::NearestNeighborsGNATNoThreadSafety<long>>();
        case ORA_NN_REF_SQRT_APPROX:
            return std::make_unique<ompl::NearestNeighborsSqrtApprox<long>>();
        default:
            return std::make_unique<ompl::NearestNeighborsLinear<long>>();
    }
}
}  // namespace

extern "C" {

int ora_set_threads(int n)
{
    (void)n;  // the reference build runs single-threaded
    return 1;
}

double ora_space_extent(const ora_space *d)
{
    return build(d, nullptr)->space->getMaximumExtent();
}

double ora_space_lvs(const ora_space *d)
{
    return build(d, nullptr)->space->getLongestValidSegmentLength();
}

void ora_distance(const ora_space *d, const double *a, const double *b, long n, double *out)
{
    auto B = build(d, nullptr);
    StateRows A(*B, a, n), C(*B, b, n);
    for (long i = 0; i < n; ++i)
        out[i] = B->space->distance(A.v[i], C.v[i]);
}

void ora_interpolate(const ora_space *d, const double *a, const double *b, const double *t, long n, double *out)
{
    auto B = build(d, nullptr);
    StateRows A(*B, a, n), C(*B, b, n), O(*B, nullptr, 1);
    for (long i = 0; i < n; ++i)
    {
        B->space->interpolate(A.v[i], C.v[i], t[i], O.v[0]);
        to_row(*B, O.v[0], out + (size_t)i * B->dim);
    }
}

void ora_valid_segment_count(const ora_space *d, const double *a, const double *b, long n, unsigned *out)
{
    auto B = build(d, nullptr);
    StateRows A(*B, a, n), C(*B, b, n);
    for (long i = 0; i < n; ++i)
        out[i] = B->space->validSegmentCount(A.v[i], C.v[i]);
}

void ora_enforce_bounds(const ora_space *d, double *states, long n)
{
    auto B = build(d, nullptr);
    StateRows A(*B, states, n);
    for (long i = 0; i < n; ++i)
    {
        B->space->enforceBounds(A.v[i]);
        to_row(*B, A.v[i], states + (size_t)i * B->dim);
    }
}

void ora_rng_uniform(unsigned seed, int kind, double lo, double hi, long n, double *out)
{
    ompl::RNG rng(seed);
    for (long i = 0; i < n; ++i)
        out[i] = kind == 0 ? rng.uniform01() : rng.uniformReal(lo, hi);
}

void ora_sample_uniform(const ora_space *d, unsigned seed, long n, double *out)
{
    auto B = build(d, nullptr);
    auto smp = seeded_sampler(*B, d->kind, seed);
    StateRows O(*B, nullptr, 1);
    for (long i = 0; i < n; ++i)
    {
        smp->sampleUniform(O.v[0]);
        to_row(*B, O.v[0], out + (size_t)i * B->dim);
    }
}

void ora_sample_uniform_near(const ora_space *d, unsigned seed, const double *near, double distance, long n,
                             double *out)
{
    auto B = build(d, nullptr);
    auto smp = seeded_sampler(*B, d->kind, seed);
    StateRows N(*B, near, n), O(*B, nullptr, 1);
    for (long i = 0; i < n; ++i)
    {
        smp->sampleUniformNear(O.v[0], N.v[i], distance);
        to_row(*B, O.v[0], out + (size_t)i * B->dim);
    }
}

void ora_sample_script(const ora_space *d, unsigned seed, const int *kinds, const long *counts, int nops,
                       const double *mean, double stddev, int log_mode, double *out)
{
    (void)log_mode;  // OMPL's own RNG::gaussian only
    auto B = build(d, nullptr);
    auto smp = seeded_sampler(*B, d->kind, seed);
    StateRows O(*B, nullptr, 1);
    long rows = 0, mrows = 0;
    for (int k = 0; k < nops; ++k)
    {
        if (kinds[k] == 1)
        {
            StateRows M(*B, mean + (size_t)mrows * B->dim, counts[k]);
            for (long i = 0; i < counts[k]; ++i)
            {
                smp->sampleGaussian(O.v[0], M.v[i], stddev);
                to_row(*B, O.v[0], out + (size_t)(rows++) * B->dim);
            }
            mrows += counts[k];
        }
        else
            for (long i = 0; i < counts[k]; ++i)
            {
                smp->sampleUniform(O.v[0]);
                to_row(*B, O.v[0], out + (size_t)(rows++) * B->dim);
            }
    }
}

void ora_log_rn(const double *x, long n, double *out)
{
    for (long i = 0; i < n; ++i)
        out[i] = std::log(x[i]);  // the reference build has no rounded-to-nearest log; glibc's
}

void ora_is_valid(const ora_space *d, const ora_checker *c, const double *states, long n, unsigned char *out)
{
    auto B = build(d, c);
    StateRows S(*B, states, n);
    for (long i = 0; i < n; ++i)
        out[i] = B->si->isValid(S.v[i]) ? 1 : 0;
}

void ora_check_motion(const ora_space *d, const ora_checker *c, const double *s1, const double *s2, long n,
                      unsigned char *ok, unsigned char *ok_bisect, double *last_t, double *last_state, int *nd,
                      int *first_j)
{
    auto B = build(d, c);
    StateRows A(*B, s1, n), C(*B, s2, n), L(*B, nullptr, 1);
    for (long i = 0; i < n; ++i)
    {
        std::pair<ob::State *, double> lv(L.v[0], kNaN);
        B->counter->calls = 0;
        bool r = B->si->checkMotion(A.v[i], C.v[i], lv);
        long calls = B->counter->calls;
        int ndi = (int)B->space->validSegmentCount(A.v[i], C.v[i]);
        if (ok)
            ok[i] = r ? 1 : 0;
        if (ok_bisect)
            ok_bisect[i] = B->si->checkMotion(A.v[i], C.v[i]) ? 1 : 0;
        if (last_t)
            last_t[i] = lv.second;
        if (nd)
            nd[i] = ndi;
        if (first_j)
            first_j[i] = r ? -1 : (ndi > 1 ? (int)calls : ndi);
        if (last_state)
        {
            double *o = last_state + (size_t)i * B->dim;
            if (r)
                for (unsigned k = 0; k < B->dim; ++k)
                    o[k] = kNaN;
            else
                to_row(*B, L.v[0], o);
        }
    }
}

int ora_check_motion_states(const ora_space *d, const ora_checker *c, const double *states, long count,
                            long *first_invalid, int *ok_bisect)
{
    auto B = build(d, c);
    StateRows S(*B, states, count);
    if (ok_bisect)
        *ok_bisect = B->si->checkMotion(S.v, (unsigned)count) ? 1 : 0;
    unsigned fi = 0;
    bool r = B->si->checkMotion(S.v, (unsigned)count, fi);
    if (!r)
        *first_invalid = fi;
    return r ? 1 : 0;
}

long ora_get_motion_states(const ora_space *d, const double *s1, const double *s2, unsigned count, int endpoints,
                           double *out)
{
    auto B = build(d, nullptr);
    StateRows A(*B, s1, 1), C(*B, s2, 1);
    std::vector<ob::State *> states;
    unsigned added = B->si->getMotionStates(A.v[0], C.v[0], states, count, endpoints != 0, true);
    for (unsigned i = 0; i < added; ++i)
        to_row(*B, states[i], out + (size_t)i * B->dim);
    B->si->freeStates(states);
    return added;
}

static void knn_impl(const ora_space *d, int algo, const double *pts, long npts, const double *q, long nq, int k,
                     long *idx, double *dist)
{
    auto B = build(d, nullptr);
    StateRows P(*B, pts, npts), Q(*B, q, nq);
    auto nn = make_nn(algo);
    nn->setDistanceFunction([&](const long &a, const long &b) {
        const ob::State *sa = a >= 0 ? P.v[a] : Q.v[-1 - a];
        const ob::State *sb = b >= 0 ? P.v[b] : Q.v[-1 - b];
        return B->space->distance(sa, sb);
    });
    std::vector<long> all(npts);
    for (long i = 0; i < npts; ++i)
        all[i] = i;
    nn->add(all);
    std::vector<long> out;
    for (long i = 0; i < nq; ++i)
    {
        nn->nearestK(-1 - i, k, out);
        for (int j = 0; j < k; ++j)
        {
            bool have = j < (int)out.size();
            idx[(size_t)i * k + j] = have ? out[j] : -1;
            dist[(size_t)i * k + j] = have ? B->space->distance(P.v[out[j]], Q.v[i])
                                           : std::numeric_limits<double>::infinity();
        }
    }
}

void ora_knn(const ora_space *d, int algo, const double *pts, long npts, const double *q, long nq, int k, long *idx,
             double *dist)
{
    knn_impl(d, algo == ORA_NN_EXACT ? ORA_NN_REF_LINEAR : algo, pts, npts, q, nq, k, idx, dist);
}

// OMPL's own NearestNeighborsSqrtApprox: add all rows, remove some, then nearest() per query in order
unsigned long ora_nn_sqrt_approx(const ora_space *d, const double *pts, long npts, const long *remove, long nrem,
                                 const double *q, long nq, long *idx, double *dist)
{
    auto B = build(d, nullptr);
    StateRows P(*B, pts, npts), Q(*B, q, nq);
    ompl::NearestNeighborsSqrtApprox<long> nn;
    nn.setDistanceFunction([&](const long &a, const long &b) {
        const ob::State *sa = a >= 0 ? P.v[a] : Q.v[-1 - a];
        const ob::State *sb = b >= 0 ? P.v[b] : Q.v[-1 - b];
        return B->space->distance(sa, sb);
    });
    std::vector<long> all(npts);
    for (long i = 0; i < npts; ++i)
        all[i] = i;
    nn.add(all);
    for (long r = 0; r < nrem; ++r)
        nn.remove(remove[r]);
    for (long i = 0; i < nq; ++i)
    {
        const long e = nn.nearest(-1 - i);
        idx[i] = e;
        dist[i] = B->space->distance(P.v[e], Q.v[i]);
    }
    // the offset after the queries: offset_ is private, so it is recovered as (queries mod checks)
    const std::size_t n = (std::size_t)(npts - nrem);
    const std::size_t checks = n ? 1 + (std::size_t)std::floor(std::sqrt((double)n)) : 0;
    return checks ? (unsigned long)(nq % checks) : 0;
}

// PRM order (geometric/planners/prm/src/PRM.cpp:570-604): each milestone queries the structure, then
// is added to it, so query i sees exactly the milestones added before it.
void ora_knn_prefix(const ora_space *d, const double *pts, long npts, const double *q, const long *limit, long nq,
                    int k, long *idx, double *dist)
{
    auto B = build(d, nullptr);
    StateRows P(*B, pts, npts), Q(*B, q, nq);
    ompl::NearestNeighborsLinear<long> nn;
    nn.setDistanceFunction([&](const long &a, const long &b) {
        const ob::State *sa = a >= 0 ? P.v[a] : Q.v[-1 - a];
        const ob::State *sb = b >= 0 ? P.v[b] : Q.v[-1 - b];
        return B->space->distance(sa, sb);
    });
    long added = 0;
    std::vector<long> out;
    for (long i = 0; i < nq; ++i)
    {
        while (added < limit[i] && added < npts)
            nn.add(added++);
        nn.nearestK(-1 - i, k, out);
        for (int j = 0; j < k; ++j)
        {
            bool have = j < (int)out.size();
            idx[(size_t)i * k + j] = have ? out[j] : -1;
            dist[(size_t)i * k + j] = have ? B->space->distance(P.v[out[j]], Q.v[i])
                                           : std::numeric_limits<double>::infinity();
        }
    }
}

long ora_radius(const ora_space *d, int algo, const double *pts, long npts, const double *q, long nq, double r,
                long *counts, long *idx, double *dist, long cap)
{
    auto B = build(d, nullptr);
    StateRows P(*B, pts, npts), Q(*B, q, nq);
    auto nn = make_nn(algo == ORA_NN_EXACT ? ORA_NN_REF_LINEAR : algo);
    nn->setDistanceFunction([&](const long &a, const long &b) {
        const ob::State *sa = a >= 0 ? P.v[a] : Q.v[-1 - a];
        const ob::State *sb = b >= 0 ? P.v[b] : Q.v[-1 - b];
        return B->space->distance(sa, sb);
    });
    std::vector<long> all(npts);
    for (long i = 0; i < npts; ++i)
        all[i] = i;
    nn->add(all);
    std::vector<long> out;
    long total = 0;
    for (long i = 0; i < nq; ++i)
    {
        nn->nearestR(-1 - i, r, out);
        counts[i] = (long)out.size();
        for (long e : out)
        {
            if (idx && dist && total < cap)
            {
                idx[total] = e;
                dist[total] = B->space->distance(P.v[e], Q.v[i]);
            }
            total++;
        }
    }
    return total;
}

}  // extern "C"

/* Reference-build extra (not part of the shared oracle API): the demo's horn world,
 * createHornEnvironment(d, eps) of demos/KinematicChain.h:279-315, as (x0, y0, x1, y1) rows.
 * The demo also writes environment_<d>.dat into the working directory. Returns the row count. */
extern "C" long ora_ref_horn_environment(unsigned d, double eps, double *out, long cap)
{
    Environment env = createHornEnvironment(d, eps);
    long n = (long)env.size();
    for (long i = 0; i < n && i < cap; ++i)
    {
        out[4 * i + 0] = env[i].x0;
        out[4 * i + 1] = env[i].y0;
        out[4 * i + 2] = env[i].x1;
        out[4 * i + 3] = env[i].y1;
    }
    return n;
}
