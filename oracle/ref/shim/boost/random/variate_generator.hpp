// Stand-in for boost::variate_generator (see uniform_on_sphere.hpp): construction is allowed, use throws.
#pragma once
#include <stdexcept>
#include <vector>
namespace boost { template <class G, class D> struct variate_generator {
    variate_generator(G, D) {}
    std::vector<double> operator()() { throw std::runtime_error("uniform_on_sphere is not available in the oracle build"); }
    D &distribution() { static D d; return d; }
}; }
