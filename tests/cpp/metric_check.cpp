// gbompl::MetricGuard (include/gbompl_ompl.hpp) against OMPL's RealVectorStateSpace, with no device:
// GpuNearestNeighbors accepts the space's own metric (NearestNeighbors.h:58-110) and throws
// ompl::Exception for any other, from setDistanceFunction when elements are stored, else from the
// first add that gives two elements to compare. Prints OK or the failed case.
#include <ompl/base/spaces/RealVectorStateSpace.h>

#include <cstdio>
#include <random>

#include "gbompl_ompl.hpp"

namespace ob = ompl::base;

int main()
{
    auto space = std::make_shared<ob::RealVectorStateSpace>(3);
    space->setBounds(-1.0, 1.0);
    std::mt19937 g(3);
    std::uniform_real_distribution<double> U(-1, 1);
    std::vector<ob::State *> pts(12);
    for (auto &p : pts)
    {
        p = space->allocState();
        for (int d = 0; d < 3; ++d)
            p->as<ob::RealVectorStateSpace::StateType>()->values[d] = U(g);
    }
    auto stateOf = [](ob::State *const &s) { return (const ob::State *)s; };
    auto own = [&](ob::State *const &a, ob::State *const &b) { return space->distance(a, b); };
    auto twice = [&](ob::State *const &a, ob::State *const &b) { return 2.0 * space->distance(a, b); };
    auto throws = [&](auto fn) {
        try
        {
            fn();
        }
        catch (const ompl::Exception &)
        {
            return true;
        }
        return false;
    };
    const std::vector<ob::State *> none, one(pts.begin(), pts.begin() + 1), many(pts.begin(), pts.begin() + 10);
    int fail = 0;
    {  // the space's metric, set before any element: the first add is checked and passes
        gbompl::MetricGuard<ob::State *> m(space.get(), stateOf);
        m.set(own, none);
        fail += throws([&] { m.check(none, many); }) ? 1 : 0;
    }
    {  // a foreign metric set on an empty container: the first add of two elements throws
        gbompl::MetricGuard<ob::State *> m(space.get(), stateOf);
        m.set(twice, none);
        fail += throws([&] { m.check(none, many); }) ? 0 : 2;
    }
    {  // a foreign metric set when elements are stored: setDistanceFunction throws
        gbompl::MetricGuard<ob::State *> m(space.get(), stateOf);
        fail += throws([&] { m.set(twice, many); }) ? 0 : 4;
    }
    {  // one element at a time: nothing to compare after the first add, the second add throws
        gbompl::MetricGuard<ob::State *> m(space.get(), stateOf);
        m.set(twice, none);
        fail += throws([&] { m.check(none, one); }) ? 8 : 0;
        fail += throws([&] { m.check(one, std::vector<ob::State *>{pts[5]}); }) ? 0 : 16;
    }
    {  // after the check passed, later adds are not checked again
        gbompl::MetricGuard<ob::State *> m(space.get(), stateOf);
        m.set(own, many);
        fail += throws([&] { m.check(many, std::vector<ob::State *>{pts[11]}); }) ? 32 : 0;
    }
    for (auto p : pts)
        space->freeState(p);
    if (fail)
        std::printf("FAIL %d\n", fail);
    else
        std::printf("OK\n");
    return fail ? 1 : 0;
}
