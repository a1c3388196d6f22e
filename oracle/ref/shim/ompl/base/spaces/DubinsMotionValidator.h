// Stand-in: a motion validator type SpaceInformation can name but the oracle never selects.
#pragma once
#include "ompl/base/MotionValidator.h"
#include <stdexcept>
namespace ompl { namespace base {
template <class T> class DubinsMotionValidator : public MotionValidator {
public:
    DubinsMotionValidator(SpaceInformation *si) : MotionValidator(si) {}
    bool checkMotion(const State *, const State *) const override { throw std::logic_error("not in the oracle build"); }
    bool checkMotion(const State *, const State *, std::pair<State *, double> &) const override
    { throw std::logic_error("not in the oracle build"); }
};
} }
