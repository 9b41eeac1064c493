// boost::math::cubic_b_spline<Real> for builds of the drop-in where Boost.Math
// is not installed. The build adds this directory with -idirafter, so an
// installed Boost takes precedence; the drop-in only names the type in the
// reference's signatures and calls its documented interface (constructor from
// knot values, left end point and step with optional end slopes; operator()
// and prime()).
//
// Interpolant: the clamped uniform cubic B-spline through the knot values,
// s(x) = sum_{j=-1}^{n} c_j B((x - a)/h - j) with B the centred cubic B-spline,
// (c_{i-1} + 4 c_i + c_{i+1}) / 6 = y_i at the knots and the end slopes
// (c_1 - c_{-1}) / 2h and (c_n - c_{n-2}) / 2h; end slopes not given are
// estimated by five-point one-sided differences.
#ifndef QTG_COMPAT_CUBIC_B_SPLINE_HPP
#define QTG_COMPAT_CUBIC_B_SPLINE_HPP
#include <cmath>
#include <cstddef>
#include <iterator>
#include <limits>
#include <stdexcept>
#include <vector>

namespace boost {
namespace math {

template <class Real>
class cubic_b_spline {
  public:
    cubic_b_spline() = default;

    template <class BidiIterator>
    cubic_b_spline(BidiIterator f, BidiIterator end_p, Real left_endpoint, Real step_size,
                   Real left_endpoint_derivative = std::numeric_limits<Real>::quiet_NaN(),
                   Real right_endpoint_derivative = std::numeric_limits<Real>::quiet_NaN())
        : a_(left_endpoint), h_(step_size) {
        std::vector<Real> y(f, end_p);
        solve(y, left_endpoint_derivative, right_endpoint_derivative);
    }

    cubic_b_spline(const Real *const f, std::size_t length, Real left_endpoint, Real step_size,
                   Real left_endpoint_derivative = std::numeric_limits<Real>::quiet_NaN(),
                   Real right_endpoint_derivative = std::numeric_limits<Real>::quiet_NaN())
        : a_(left_endpoint), h_(step_size) {
        std::vector<Real> y(f, f + length);
        solve(y, left_endpoint_derivative, right_endpoint_derivative);
    }

    Real operator()(Real x) const {
        Real u;
        const Real *c = segment(x, &u);
        const Real v = 1 - u, u2 = u * u, u3 = u2 * u;
        return (v * v * v * c[0] + (3 * u3 - 6 * u2 + 4) * c[1] + (-3 * u3 + 3 * u2 + 3 * u + 1) * c[2] +
                u3 * c[3]) / 6;
    }

    Real prime(Real x) const {
        Real u;
        const Real *c = segment(x, &u);
        const Real v = 1 - u, u2 = u * u;
        return (-v * v * c[0] + (3 * u2 - 4 * u) * c[1] + (-3 * u2 + 2 * u + 1) * c[2] + u2 * c[3]) / (2 * h_);
    }

  private:
    Real a_ = 0, h_ = 1;
    std::vector<Real> c_;  // c_{-1} .. c_n

    // the four coefficients around x's interval and x's fraction in it
    const Real *segment(Real x, Real *u) const {
        const int n = (int)c_.size() - 2;
        const Real t = (x - a_) / h_;
        if (!(t >= -1e-12 * n && t <= (n - 1) * (1 + 1e-12)))
            throw std::domain_error("cubic_b_spline: abscissa outside the knots");
        int i = (int)std::floor(t);
        if (i < 0) i = 0;
        if (i > n - 2) i = n - 2;
        *u = t - i;
        return c_.data() + i;
    }

    void solve(const std::vector<Real> &y, Real dl, Real dr) {
        const int n = (int)y.size();
        if (n < 5 || !(h_ > 0)) throw std::invalid_argument("cubic_b_spline: need >= 5 values and a positive step");
        if (std::isnan(dl)) dl = (-25 * y[0] + 48 * y[1] - 36 * y[2] + 16 * y[3] - 3 * y[4]) / (12 * h_);
        if (std::isnan(dr))
            dr = (25 * y[n - 1] - 48 * y[n - 2] + 36 * y[n - 3] - 16 * y[n - 4] + 3 * y[n - 5]) / (12 * h_);
        // rows: (0) 4 x0 + 2 x1 = 6 y0 + 2h dl; (i) x_{i-1} + 4 x_i + x_{i+1} = 6 y_i;
        // (n-1) 2 x_{n-2} + 4 x_{n-1} = 6 y_{n-1} - 2h dr. Eliminate the sub-diagonal,
        // keeping the modified super-diagonal g and right side r.
        std::vector<Real> g(n), r(n);
        g[0] = Real(2) / 4;
        r[0] = (6 * y[0] + 2 * h_ * dl) / 4;
        for (int i = 1; i < n; ++i) {
            const Real lo = i == n - 1 ? 2 : 1, up = 1;
            const Real den = 4 - lo * g[i - 1];
            g[i] = up / den;
            const Real rhs = 6 * y[i] - (i == n - 1 ? 2 * h_ * dr : 0);
            r[i] = (rhs - lo * r[i - 1]) / den;
        }
        c_.assign(n + 2, 0);
        Real *x = c_.data() + 1;
        x[n - 1] = r[n - 1];
        for (int i = n - 2; i >= 0; --i) x[i] = r[i] - g[i] * x[i + 1];
        c_[0] = x[1] - 2 * h_ * dl;
        c_[n + 1] = x[n - 2] + 2 * h_ * dr;
    }
};

}  // namespace math
}  // namespace boost
#endif
