/*
 * Stand-in for boost::math::signbit (Boost is absent in this image); used
 * only by the pinning harness oracle/ref_harness.cpp.  Test infrastructure.
 */
#ifndef ORACLE_SHIM_BOOST_SIGN_HPP
#define ORACLE_SHIM_BOOST_SIGN_HPP
#include <cmath>
namespace boost { namespace math { using std::signbit; } }
#endif
