// Stand-in: constrained planning is off the path; SpaceInformation only names these two types.
#pragma once
#include "ompl/base/StateSpace.h"
#include "ompl/base/MotionValidator.h"
#include <stdexcept>
namespace ompl { namespace base {
class ConstrainedStateSpace : public StateSpace { public: ~ConstrainedStateSpace() override = default; };
class ConstrainedMotionValidator : public MotionValidator {
public:
    ConstrainedMotionValidator(SpaceInformation *si) : MotionValidator(si) {}
    bool checkMotion(const State *, const State *) const override { throw std::logic_error("not in the oracle build"); }
    bool checkMotion(const State *, const State *, std::pair<State *, double> &) const override
    { throw std::logic_error("not in the oracle build"); }
};
} }
