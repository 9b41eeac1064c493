// Type-only stand-in for boost::math::cubic_b_spline<Real>.
//
// Test infrastructure only. The reference's forces.h / update.h name this type
// in the signatures of their spline ("fast-CMD") functions, which the oracle
// never calls; the stand-in lets those translation units compile when Boost is
// not installed. Evaluating it is an error, so it aborts.
#ifndef QTIP_ORACLE_CUBIC_B_SPLINE_SHIM_HPP
#define QTIP_ORACLE_CUBIC_B_SPLINE_SHIM_HPP
#include <cstdlib>

namespace boost {
namespace math {
template <class Real>
class cubic_b_spline {
  public:
    cubic_b_spline() = default;
    template <class It>
    cubic_b_spline(It, It, Real, Real) {}
    Real operator()(Real) const { std::abort(); }
    Real prime(Real) const { std::abort(); }
};
}  // namespace math
}  // namespace boost
#endif
