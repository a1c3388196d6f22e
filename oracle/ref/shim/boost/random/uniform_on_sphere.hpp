// Stand-in for boost::uniform_on_sphere. Only RNG::uniformNormalVector uses it, which is off the
// sampling/validity/motion/kNN path; calling it through this stand-in throws.
#pragma once
#include <vector>
namespace boost { template <class R = double, class C = std::vector<R>> struct uniform_on_sphere {
    explicit uniform_on_sphere(int = 2) {}
    void reset() {}
}; }
