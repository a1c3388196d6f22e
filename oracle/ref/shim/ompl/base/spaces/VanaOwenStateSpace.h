// Stand-in: SpaceInformation::setDefaultMotionValidator only dynamic_casts to this type, which the
// oracle never instantiates; an abstract polymorphic declaration is all that translation unit needs.
#pragma once
#include "ompl/base/StateSpace.h"
namespace ompl { namespace base { class VanaOwenStateSpace : public StateSpace { public: ~VanaOwenStateSpace() override = default; }; } }
