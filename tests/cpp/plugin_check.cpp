// Builds the gbompl OMPL plugins against OMPL's own headers and objects and compares them with
// OMPL's DiscreteMotionValidator / StateValidityChecker / NearestNeighborsLinear on the same
// SpaceInformation. Without a GPU it checks that construction fails with ompl::Exception.
#include <ompl/base/DiscreteMotionValidator.h>
#include <ompl/base/SpaceInformation.h>
#include <ompl/base/samplers/UniformValidStateSampler.h>
#include <ompl/base/spaces/RealVectorStateSpace.h>
#include <ompl/datastructures/NearestNeighborsLinear.h>
#include <ompl/datastructures/NearestNeighborsSqrtApprox.h>

#include <cmath>
#include <cstdio>
#include <limits>
#include <random>

#include "gbompl_ompl.hpp"

namespace ob = ompl::base;

struct Circles : ob::StateValidityChecker
{
    Circles(ob::SpaceInformation *si, std::vector<double> c) : ob::StateValidityChecker(si), c_(std::move(c)) {}
    bool isValid(const ob::State *s) const override
    {
        const double *xy = s->as<ob::RealVectorStateSpace::StateType>()->values;
        for (size_t i = 0; i < c_.size(); i += 3)
        {
            double dx = c_[i] - xy[0], dy = c_[i + 1] - xy[1];
            if (dx * dx + dy * dy < c_[i + 2] * c_[i + 2])
                return false;
        }
        return true;
    }
    std::vector<double> c_;
};

// OMPL's own sampler with its stream seeded like RNG::setLocalSeed(seed)
struct SeededSampler : ob::RealVectorStateSampler
{
    SeededSampler(const ob::StateSpace *s, std::uint_fast32_t seed) : ob::RealVectorStateSampler(s)
    {
        rng_.setLocalSeed(seed);
    }
};

int main()
{
    std::mt19937_64 g(5);
    std::uniform_real_distribution<double> U(0, 1), R(0.02, 0.06);
    std::vector<double> world;
    for (int i = 0; i < 100; ++i)
        world.insert(world.end(), {U(g), U(g), R(g)});
    auto space = std::make_shared<ob::RealVectorStateSpace>(2);
    space->setBounds(0.0, 1.0);
    auto si = std::make_shared<ob::SpaceInformation>(space);
    si->setStateValidityChecker(std::make_shared<Circles>(si.get(), world));
    si->setStateValidityCheckingResolution(0.01);
    si->setup();
    gbompl::GpuContextPtr ctx;
    try
    {
        ctx = std::make_shared<gbompl::GpuContext>(space, GBO_SPACE_REAL_VECTOR);
        ctx->bindWorld(GBO_CHECK_CIRCLES, world, 3, {}, 0, 0.0, GBO_PRECISION_FP64);
    }
    catch (const ompl::Exception &e)
    {
        std::printf("NO_DEVICE %s\n", e.what());
        return 0;
    }
    gbompl::GpuStateValidityChecker gsvc(si, ctx);
    gbompl::GpuDiscreteMotionValidator gmv(si, ctx);
    ob::DiscreteMotionValidator ref(si);
    auto a = si->allocState(), b = si->allocState(), la = si->allocState(), lb = si->allocState();
    int mism = 0;
    for (int i = 0; i < 2000; ++i)
    {
        auto *va = a->as<ob::RealVectorStateSpace::StateType>()->values;
        auto *vb = b->as<ob::RealVectorStateSpace::StateType>()->values;
        va[0] = U(g); va[1] = U(g); vb[0] = U(g); vb[1] = U(g);
        mism += gsvc.isValid(a) != si->isValid(a);
        std::pair<ob::State *, double> l1(la, -7.0), l2(lb, -7.0);
        bool r1 = gmv.checkMotion(a, b, l1), r2 = ref.checkMotion(a, b, l2);
        mism += r1 != r2 || gmv.checkMotion(a, b) != ref.checkMotion(a, b);
        if (!r1 && !r2)
            mism += l1.second != l2.second || !space->equalStates(la, lb);
    }
    // nearest neighbours over State* elements
    std::vector<ob::State *> pts(3000);
    for (auto &p : pts)
    {
        p = si->allocState();
        auto *v = p->as<ob::RealVectorStateSpace::StateType>()->values;
        v[0] = U(g);
        v[1] = U(g);
    }
    gbompl::GpuNearestNeighbors<ob::State *> gnn(ctx, [](ob::State *const &s) { return (const ob::State *)s; }, 4096);
    ompl::NearestNeighborsLinear<ob::State *> lnn;
    auto df = [&](ob::State *const &x, ob::State *const &y) { return space->distance(x, y); };
    gnn.setDistanceFunction(df);
    lnn.setDistanceFunction(df);
    gnn.add(pts);
    lnn.add(pts);
    gnn.remove(pts[7]);
    lnn.remove(pts[7]);
    std::vector<ob::State *> n1, n2;
    for (int q = 0; q < 100; ++q)
    {
        gnn.nearestK(pts[q * 13], 10, n1);
        lnn.nearestK(pts[q * 13], 10, n2);
        mism += n1 != n2;
        gnn.nearestR(pts[q * 13], 0.05, n1);
        lnn.nearestR(pts[q * 13], 0.05, n2);
        mism += n1 != n2;
    }
    mism += gnn.size() != lnn.size();
    // NearestNeighborsSqrtApprox: the same round-robin subset, call after call
    gbompl::GpuNearestNeighborsSqrtApprox<ob::State *> gsq(ctx, [](ob::State *const &s) { return (const ob::State *)s; },
                                                          4096);
    ompl::NearestNeighborsSqrtApprox<ob::State *> lsq;
    gsq.setDistanceFunction(df);
    lsq.setDistanceFunction(df);
    gsq.add(pts);
    lsq.add(pts);
    gsq.remove(pts[3]);
    lsq.remove(pts[3]);
    for (int q = 0; q < 200; ++q)
        mism += gsq.nearest(pts[(q * 17) % pts.size()]) != lsq.nearest(pts[(q * 17) % pts.size()]);
    // UniformValidStateSampler: same seed, same calls (sample and sampleNear), same results (a few with
    // 2 attempts)
    space->setStateSamplerAllocator([](const ob::StateSpace *s) { return std::make_shared<SeededSampler>(s, 77); });
    ob::UniformValidStateSampler rvs(si.get());
    gbompl::GpuUniformValidStateSampler gvs(si.get(), ctx, 77);
    for (int i = 0; i < 300; ++i)
    {
        const unsigned att = i % 50 < 10 ? 2 : 100;
        rvs.setNrAttempts(att);
        gvs.setNrAttempts(att);
        const bool near = i % 7 == 3;  // sampleNear around a stored point, on the same stream
        const bool r1 = near ? rvs.sampleNear(a, pts[i], 0.1) : rvs.sample(a);
        const bool r2 = near ? gvs.sampleNear(b, pts[i], 0.1) : gvs.sample(b);
        mism += r1 != r2 || !space->equalStates(a, b);
    }
    std::vector<ob::State *> batch(500);
    for (auto &p : batch)
        p = si->allocState();
    std::vector<bool> bok;
    gvs.sampleBatch(batch, bok);
    for (size_t i = 0; i < batch.size(); ++i)
        mism += rvs.sample(a) != bok[i] || !space->equalStates(a, batch[i]);
    // sampleGaussian interleaved with sampleUniform: the stream positions agree exactly; a Gaussian
    // value may differ by a few ulps where glibc's log is not rounded to nearest (rarely)
    SeededSampler rs(space.get(), 91);
    gbompl::GpuStateSampler gs(space.get(), ctx, 91);
    int gauss_differ = 0;
    for (int i = 0; i < 400; ++i)
    {
        if (i % 7 == 3)
        {
            rs.sampleUniform(a);
            gs.sampleUniform(b);
            mism += !space->equalStates(a, b);
            continue;
        }
        auto *m = la->as<ob::RealVectorStateSpace::StateType>()->values;
        m[0] = U(g);
        m[1] = U(g);
        rs.sampleGaussian(a, la, 0.3);
        gs.sampleGaussian(b, la, 0.3);
        auto *va = a->as<ob::RealVectorStateSpace::StateType>()->values;
        auto *vb = b->as<ob::RealVectorStateSpace::StateType>()->values;
        for (int k = 0; k < 2; ++k)
        {
            gauss_differ += va[k] != vb[k];
            mism += std::fabs(va[k] - vb[k]) > 4 * std::numeric_limits<double>::epsilon();
        }
    }
    mism += gauss_differ > 8;
    std::printf("%s mismatches=%d valid=%u invalid=%u\n", mism ? "MISMATCH" : "MATCH", mism,
                gmv.getValidMotionCount(), gmv.getInvalidMotionCount());
    return mism ? 1 : 0;
}
