// Stand-in for Boost.Math constants: the few named constants the hot-path sources use.
#pragma once
namespace boost { namespace math {
namespace double_constants {
constexpr double pi = 3.141592653589793238462643383279502884;
constexpr double half_pi = 1.570796326794896619231321691639751442;
constexpr double two_pi = 6.283185307179586476925286766559005768;
constexpr double sixth_pi = 0.5235987755982988730771072305465838140;
}
namespace constants {
template <class T> constexpr T pi() { return static_cast<T>(3.141592653589793238462643383279502884L); }
template <class T> constexpr T half_pi() { return static_cast<T>(1.570796326794896619231321691639751442L); }
template <class T> constexpr T two_pi() { return static_cast<T>(6.283185307179586476925286766559005768L); }
template <class T> constexpr T e() { return static_cast<T>(2.718281828459045235360287471352662498L); }
}
} }
#ifndef BOOST_ASSERT_MSG
#define BOOST_ASSERT_MSG(expr, msg) ((void)0)
#endif
