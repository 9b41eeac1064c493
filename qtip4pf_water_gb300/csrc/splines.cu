// Tabulated pair corrections ("fast-CMD" splines) on GB300: replaces the spline
// loop of get_forces_wspline (forces.cpp:634-691, pair term get_spline
// forces.cpp:452-466). Every atom pair of a configuration whose minimum-image
// separation is inside its type's cutoff (O-O, O-H, H-H; r^2 < cut^2 strictly,
// as forces.cpp:664-686) adds s(r) to the energy and -s'(r) r_ij / r to atom i
// (+ to atom j), s the type's cubic spline.
//
// The spline is a uniform cubic B-spline interpolant of values y_0 .. y_{n-1}
// on knots x_i = start + i h with clamped end slopes (the construction
// Boost.Math's cubic_b_spline documents): s(x) = sum_j c_j B((x - start)/h - j),
// j = -1 .. n, B the centred cubic B-spline; (c_{i-1} + 4 c_i + c_{i+1}) / 6 =
// y_i at every knot and (c_1 - c_{-1}) / 2h, (c_n - c_{n-2}) / 2h the end
// slopes. The coefficients are solved on the host (tridiagonal system) when a
// table is attached; end slopes not given are estimated by five-point
// one-sided differences. Kernel: thread per atom i of a force evaluation, the
// evaluation's atoms staged through shared memory in tiles, each pair taken
// from both sides (each thread writes only its own atom's force: no atomics,
// a fixed summation order), half of each pair energy from each side.
#include <math.h>

#include <vector>

#include "qtg_internal.h"

namespace qtg {

namespace {

constexpr int ST = 128;  // atoms per block and per shared-memory tile

template <typename R>
struct V3 {
    R x, y, z;
};

// uniform cubic B-spline: value and derivative (per unit of t) from the four
// coefficients around interval i0 (cf points at c_{i0-1}), fraction u in [0, 1)
template <typename R>
__device__ __forceinline__ void bspline_eval(const double *cf, R u, R *val, R *dval) {
    const R c0 = (R)__ldg(cf), c1 = (R)__ldg(cf + 1), c2 = (R)__ldg(cf + 2), c3 = (R)__ldg(cf + 3);
    const R v = (R)1 - u, u2 = u * u, u3 = u2 * u;
    const R w0 = v * v * v, w1 = (R)3 * u3 - (R)6 * u2 + (R)4, w2 = (R)-3 * u3 + (R)3 * u2 + (R)3 * u + (R)1;
    *val = (w0 * c0 + w1 * c1 + w2 * c2 + u3 * c3) * ((R)1 / (R)6);
    const R d0 = -v * v, d1 = (R)3 * u2 - (R)4 * u, d2 = (R)-3 * u2 + (R)2 * u + (R)1;
    *dval = (d0 * c0 + d1 * c1 + d2 * c2 + u2 * c3) * (R)0.5;
}

template <typename R>
__device__ __forceinline__ R round_half_away(R x);
template <>
__device__ __forceinline__ double round_half_away<double>(double x) {
    return round(x);
}
template <>
__device__ __forceinline__ float round_half_away<float>(float x) {
    return roundf(x);
}

template <typename R>
__global__ void __launch_bounds__(ST) k_pair_splines(SplineArgs a) {
    const Job J = a.jobs[blockIdx.y];
    const PairSplines &T = a.tables[J.sys];
    if (!T.on) return;
    const SysDev &S = a.sys[J.sys];
    const int na = 3 * S.n_mols;
    const double *pos = a.pos + J.pos_off;
    __shared__ V3<R> tile[ST];
    const int i = blockIdx.x * ST + threadIdx.x;
    const bool act = i < na;
    R box[3], ibox[3];
    for (int d = 0; d < 3; ++d) {
        box[d] = (R)S.box[d];
        ibox[d] = (R)S.inv_box[d];
    }
    // FP64: the raw coordinates, differences and minimum images as the reference
    // forms them; FP32: coordinates wrapped into the box in FP64 first, so their
    // single-precision differences carry the box's absolute resolution
    auto load = [&](int k) {
        V3<R> v;
        double x = pos[3 * k], y = pos[3 * k + 1], z = pos[3 * k + 2];
        if (sizeof(R) == 4) {
            x -= S.box[0] * floor(x * S.inv_box[0]);
            y -= S.box[1] * floor(y * S.inv_box[1]);
            z -= S.box[2] * floor(z * S.inv_box[2]);
        }
        v.x = (R)x;
        v.y = (R)y;
        v.z = (R)z;
        return v;
    };
    V3<R> pi = act ? load(i) : V3<R>{0, 0, 0};
    const int ti = act ? (i % 3 == 0 ? 0 : 1) : 0;
    R fx = 0, fy = 0, fz = 0, e = 0;
    for (int j0 = 0; j0 < na; j0 += ST) {
        __syncthreads();
        if (j0 + threadIdx.x < na) tile[threadIdx.x] = load(j0 + threadIdx.x);
        __syncthreads();
        if (!act) continue;
        const int nj = min(ST, na - j0);
        for (int jj = 0; jj < nj; ++jj) {
            const int j = j0 + jj;
            if (j == i) continue;
            R dx = pi.x - tile[jj].x, dy = pi.y - tile[jj].y, dz = pi.z - tile[jj].z;
            dx -= box[0] * round_half_away<R>(dx * ibox[0]);
            dy -= box[1] * round_half_away<R>(dy * ibox[1]);
            dz -= box[2] * round_half_away<R>(dz * ibox[2]);
            const R r2 = dx * dx + dy * dy + dz * dz;
            const int t = ti + (j % 3 == 0 ? 0 : 1);  // 0 O-O, 1 O-H, 2 H-H
            const SplineType &st = T.t[t];
            if (!(r2 < (R)st.cut_sq) || st.n < 2) continue;
            const R r = sqrt(r2);
            R tt = (r - (R)st.start) * (R)st.inv_step;
            int i0 = (int)floor(tt);
            i0 = max(0, min(i0, st.n - 2));
            const R u = tt - (R)i0;
            R val, dval;
            bspline_eval<R>(a.coef + st.coef_off + i0, u, &val, &dval);
            const R fp = dval * (R)st.inv_step / r;  // s'(r) / r
            fx -= fp * dx;
            fy -= fp * dy;
            fz -= fp * dz;
            e += (R)0.5 * val;
        }
    }
    if (act) {
        double *o = a.out + J.out_off + 3 * i;
        o[0] += (double)fx;
        o[1] += (double)fy;
        o[2] += (double)fz;
        if (a.out_prop) {
            double *p = a.out_prop + J.out_off + 3 * i;
            p[0] += (double)fx;
            p[1] += (double)fy;
            p[2] += (double)fz;
        }
    }
    __shared__ double red[ST / 32];
    const double be = block_sum((double)e, red);
    if (threadIdx.x == 0) atomicAdd(a.energy + J.slot, be);
}

}  // namespace

void launch_pair_splines(const SplineArgs &a, bool mixed, cudaStream_t s, unsigned long long *launches) {
    if (a.n_jobs <= 0) return;
    const dim3 g((3 * a.max_mols + ST - 1) / ST, a.n_jobs);
    if (mixed) k_pair_splines<float><<<g, ST, 0, s>>>(a);
    else k_pair_splines<double><<<g, ST, 0, s>>>(a);
    if (launches) ++*launches;
}

// Coefficients c_{-1} .. c_n (n + 2 values) of the clamped uniform cubic
// B-spline interpolant of y_0 .. y_{n-1}, step h. Slopes given as NaN are
// estimated by five-point one-sided differences (n >= 5). Thomas algorithm on
// the n x n system for c_0 .. c_{n-1}; rows 0 and n-1 carry the end conditions
// (c_{-1} = c_1 - 2 h y'_0 and c_n = c_{n-2} + 2 h y'_{n-1} substituted).
bool bspline_coefficients(const double *y, int n, double h, double dl, double dr, double *c) {
    if (n < 5 || !(h > 0)) return false;
    if (isnan(dl)) dl = (-25.0 * y[0] + 48.0 * y[1] - 36.0 * y[2] + 16.0 * y[3] - 3.0 * y[4]) / (12.0 * h);
    if (isnan(dr))
        dr = (25.0 * y[n - 1] - 48.0 * y[n - 2] + 36.0 * y[n - 3] - 16.0 * y[n - 4] + 3.0 * y[n - 5]) / (12.0 * h);
    std::vector<double> sub(n, 1.0), dia(n, 4.0), sup(n, 1.0), rhs(n);
    for (int i = 0; i < n; ++i) rhs[i] = 6.0 * y[i];
    sup[0] = 2.0;
    rhs[0] += 2.0 * h * dl;
    sub[n - 1] = 2.0;
    rhs[n - 1] -= 2.0 * h * dr;
    for (int i = 1; i < n; ++i) {
        const double w = sub[i] / dia[i - 1];
        dia[i] -= w * sup[i - 1];
        rhs[i] -= w * rhs[i - 1];
    }
    std::vector<double> x(n);
    x[n - 1] = rhs[n - 1] / dia[n - 1];
    for (int i = n - 2; i >= 0; --i) x[i] = (rhs[i] - sup[i] * x[i + 1]) / dia[i];
    for (int i = 0; i < n; ++i) c[i + 1] = x[i];
    c[0] = x[1] - 2.0 * h * dl;
    c[n + 1] = x[n - 2] + 2.0 * h * dr;
    return true;
}

}  // namespace qtg
