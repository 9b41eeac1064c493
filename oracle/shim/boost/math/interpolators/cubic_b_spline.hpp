// Stand-in for boost::math::cubic_b_spline<Real> (Boost is not installed here).
//
// Test infrastructure only: it lets the reference's sources compile and run
// their spline ("fast-CMD") path in the oracle's reference build. It keeps the
// documented interface -- values on a uniform grid, left end point and step,
// optional end slopes; operator() and prime() -- and evaluates the clamped
// uniform cubic B-spline interpolant with the oracle's own restatement
// (qo_spline_build / qo_spline_eval in oracle/qtip_oracle.c, linked in from
// liboracle.so). Whether Boost estimates missing end slopes the same way is
// not pinned (no Boost here).
#ifndef QTIP_ORACLE_CUBIC_B_SPLINE_SHIM_HPP
#define QTIP_ORACLE_CUBIC_B_SPLINE_SHIM_HPP
#include <cmath>
#include <cstddef>
#include <limits>
#include <vector>

extern "C" {
int qo_spline_build(const double *y, int n, double step, double dl, double dr, double *c);
double qo_spline_eval(const double *c, int n, double start, double step, double x, double *deriv);
}

namespace boost {
namespace math {
template <class Real>
class cubic_b_spline {
  public:
    cubic_b_spline() = default;
    template <class It>
    cubic_b_spline(It f, It end, Real left_endpoint, Real step_size,
                   Real left_endpoint_derivative = std::numeric_limits<Real>::quiet_NaN(),
                   Real right_endpoint_derivative = std::numeric_limits<Real>::quiet_NaN())
        : a_(left_endpoint), h_(step_size) {
        std::vector<double> y;
        for (; f != end; ++f) y.push_back((double)*f);
        n_ = (int)y.size();
        c_.assign(y.size() + 2, 0.0);
        qo_spline_build(y.data(), n_, (double)h_, (double)left_endpoint_derivative,
                        (double)right_endpoint_derivative, c_.data());
    }
    Real operator()(Real x) const { return (Real)qo_spline_eval(c_.data(), n_, a_, h_, (double)x, nullptr); }
    Real prime(Real x) const {
        double d = 0.0;
        qo_spline_eval(c_.data(), n_, a_, h_, (double)x, &d);
        return (Real)d;
    }

  private:
    double a_ = 0.0, h_ = 1.0;
    int n_ = 0;
    std::vector<double> c_;
};
}  // namespace math
}  // namespace boost
#endif
