/*
 * Stand-in for <boost/math/special_functions/gamma.hpp>; the reference calls
 * only boost::math::lgamma (src/utils.cpp:103-106).  The C library's lgamma is
 * used instead.  ORACLE / TEST INFRASTRUCTURE.
 */
#ifndef BMG_SHIM_BOOST_MATH_GAMMA_HPP_
#define BMG_SHIM_BOOST_MATH_GAMMA_HPP_

#include <cmath>

namespace boost {
namespace math {
inline double lgamma(double x) { return std::lgamma(x); }
}  // namespace math
}  // namespace boost

#endif
