// qTIP4P/F force evaluation on GB300 (replaces forces.cpp:25-630).
//
// A launch evaluates a batch of "jobs" (one configuration of one system each;
// all beads of all replicas at once). Per job:
//   k_prep     charge sites (M, H1, H2) wrapped into the box with their charges,
//              wrapped oxygen positions, and per-site phase tables
//              exp(i 2 pi m s_d), m = 0..k_max, d = x,y,z (complex recursion from
//              exp(i 2 pi s_d), charge folded into the x factor);
//   k_real     real-space Ewald between sites of different molecules; grid =
//              (i-site tiles) x (j-chunks) x jobs, j-sites staged through shared
//              memory, each thread owns one i-site and writes one partial force
//              per j-chunk (no atomics, deterministic);
//   k_ksk      structure factors S(k) = sum_i q_i exp(i k.r_i); grid = (k tiles)
//              x (site chunks) x jobs, one thread per k-vector, site chunks staged
//              in shared memory, 32-site partial sums promoted to FP64;
//   k_kforce   reciprocal-space site forces; grid = (i-site tiles) x (k-chunks)
//              x jobs, (k, 2 c_k k, S(k)) broadcast from shared memory, S(k)
//              summed over the site-chunk partials in fixed order;
//   k_combine  per molecule: partial site forces summed in fixed order, same-
//              molecule real-space pairs (erfc - 1), quartic-Morse bonds, HOH
//              angle (FP64 difference vectors), M-site chain rule;
//   k_lj       O-O Lennard-Jones over the CSR Verlet list, one warp per row.
//   k_lj_dense O-O Lennard-Jones of the device stepper (mixed), all pairs from shared memory.
// The kernels are templated on the arithmetic type: double for the parity
// mode, float (FP64 accumulation across tiles/chunks/planes) for the mixed
// mode. Mode-1 jobs compute the directional derivative of the intermolecular
// Ewald forces along a per-dof direction (the Suzuki-Chin force gradient).
#include <math.h>

#include <algorithm>
#include <string>

#include "qtg_internal.h"

namespace qtg {

namespace {

template <typename R> struct V4;
template <> struct __align__(16) V4<float> { float x, y, z, w; };
template <> struct __align__(16) V4<double> { double x, y, z, w; };
template <typename R> struct V2;
template <> struct __align__(8) V2<float> { float x, y; };
template <> struct __align__(16) V2<double> { double x, y; };

__device__ __forceinline__ double f_erfc(double x) { return erfc(x); }
__device__ __forceinline__ double f_exp(double x) { return exp(x); }
__device__ __forceinline__ float f_rint(float x) { return rintf(x); }
__device__ __forceinline__ double f_rint(double x) { return rint(x); }
__device__ __forceinline__ double f_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ double f_acos(double x) { return acos(x); }
__device__ __forceinline__ void f_sincospi(double t, double *s, double *c) { sincospi(t, s, c); }

template <typename R> __device__ __forceinline__ R sys_box(const SysDev &S, int d);
template <> __device__ __forceinline__ float sys_box<float>(const SysDev &S, int d) { return S.boxf[d]; }
template <> __device__ __forceinline__ double sys_box<double>(const SysDev &S, int d) { return S.box[d]; }
template <typename R> __device__ __forceinline__ R sys_ibox(const SysDev &S, int d);
template <> __device__ __forceinline__ float sys_ibox<float>(const SysDev &S, int d) { return S.inv_boxf[d]; }
template <> __device__ __forceinline__ double sys_ibox<double>(const SysDev &S, int d) { return S.inv_box[d]; }

__device__ __forceinline__ int chunk_lo(int n, int c, int nc) { return (int)(((long long)n * c) / nc); }

// Real-space pair kernel pieces. For FP32: 1/r, exp(-x^2) and 1/(1 + p x) from
// the approximate special-function instructions of PTX (rsqrt.approx,
// ex2.approx, rcp.approx: relative errors of a few ulp), and erfc(x) =
// t P(t) exp(-x^2), t = 1 / (1 + p x), the rational approximation of
// Abramowitz & Stegun, Handbook of Mathematical Functions, eq. 7.1.26 (absolute
// error <= 1.5e-7, which bounds the accuracy of the whole term), reusing the
// Gaussian the force needs anyway. For FP64 the library functions are used.
__device__ __forceinline__ float rsqrt_approx(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float ex2_approx(float x) {
    float y;
    asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rcp_approx(float x) {
    float y;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
constexpr float AS_P = 0.3275911f;  // A&S 7.1.26
__device__ __forceinline__ float as_poly(float t) {
    return fmaf(fmaf(fmaf(fmaf(1.061405429f, t, -1.453152027f), t, 1.421413741f), t, -0.284496736f), t,
                0.254829592f);
}
__device__ __forceinline__ void pair_terms(float r2, float kap, float kap2, float *inv, float *ex, float *ec) {
    const float iv = rsqrt_approx(r2);
    const float x = kap * (r2 * iv);
    const float e = ex2_approx(-kap2 * r2 * 1.4426950408889634f);
    const float t = rcp_approx(fmaf(AS_P, x, 1.0f));
    *inv = iv;
    *ex = e;
    *ec = t * as_poly(t) * e;
}
__device__ __forceinline__ void pair_terms(double r2, double kap, double kap2, double *inv, double *ex, double *ec) {
    const double r = sqrt(r2);
    *inv = 1.0 / r;
    *ex = exp(-kap2 * r2);
    *ec = erfc(kap * r);
}

// ---- k_prep (FP64 form; the FP32 form is k_prep_f32) ---------------------------
template <typename R>
__global__ void __launch_bounds__(128) k_prep(EvalArgs a) {
    const Job J = a.jobs[blockIdx.y];
    const SysDev &S = a.sys[J.sys];
    const int ns = S.n_sites;
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s == 0) a.energy[J.slot] = 0.0;
    if (s >= ns) return;
    const int mol = s / 3, kind = s - 3 * mol;
    const double *q = a.pos + J.pos_off;
    const double g = a.c.gamma_vs;
    double x[3], u[3] = {0.0, 0.0, 0.0};
    if (a.sites_are_input || kind != 0) {
        for (int d = 0; d < 3; ++d) x[d] = q[3 * s + d];
        if (J.mode == 1)
            for (int d = 0; d < 3; ++d) u[d] = a.dir[J.pos_off + 3 * s + d];
    } else {
        // M site (forces.cpp:558-564)
        for (int d = 0; d < 3; ++d)
            x[d] = g * q[9 * mol + d] + 0.5 * (1.0 - g) * (q[9 * mol + 3 + d] + q[9 * mol + 6 + d]);
        if (J.mode == 1) {
            const double *v = a.dir + J.pos_off;
            for (int d = 0; d < 3; ++d)
                u[d] = g * v[9 * mol + d] + 0.5 * (1.0 - g) * (v[9 * mol + 3 + d] + v[9 * mol + 6 + d]);
        }
        // wrapped oxygen position for the Lennard-Jones kernel
        V4<R> o;
        double w[3];
        for (int d = 0; d < 3; ++d) {
            const double t = q[9 * mol + d] * S.inv_box[d];
            w[d] = (t - floor(t)) * S.box[d];
        }
        o.x = (R)w[0];
        o.y = (R)w[1];
        o.z = (R)w[2];
        o.w = (R)0;
        reinterpret_cast<V4<R> *>(a.opos)[J.site_off / 3 + mol] = o;
    }
    const double chg = a.charge[S.chg_off + s];
    double frac[3];
    for (int d = 0; d < 3; ++d) {
        const double t = x[d] * S.inv_box[d];
        frac[d] = t - floor(t);
    }
    V4<R> sv;
    sv.x = (R)(frac[0] * S.box[0]);
    sv.y = (R)(frac[1] * S.box[1]);
    sv.z = (R)(frac[2] * S.box[2]);
    sv.w = (R)chg;
    reinterpret_cast<V4<R> *>(a.sites)[J.site_off + s] = sv;
    if (J.mode == 1) {
        V4<R> tv;
        tv.x = (R)u[0];
        tv.y = (R)u[1];
        tv.z = (R)u[2];
        tv.w = (R)0;
        reinterpret_cast<V4<R> *>(a.tan_sites)[J.site_off + s] = tv;
    }
    // phase table exp(i 2 pi m frac_d), layout [(d * (kmax+1) + m) * ns + s], by
    // complex recursion from exp(i 2 pi frac_d) (as forces.cpp:233-240 does),
    // reseeded every 4 powers from a directly evaluated phase whose argument
    // 2 m frac_d is reduced in FP64, so rounding does not accumulate with m (the
    // FP32 tables of k_prep_f32 reduce it exactly in fixed point)
    const int km1 = S.k_max + 1;
    V2<R> *ph = reinterpret_cast<V2<R> *>(a.phase) + J.phase_off;
    for (int d = 0; d < 3; ++d) {
        R s1, c1;
        {
            double t = 2.0 * frac[d];
            t -= 2.0 * floor(0.5 * t + 0.5);  // in [-1, 1)
            f_sincospi((R)t, &s1, &c1);
        }
        const R qd = (d == 0) ? (R)chg : (R)1;
        R cr = (R)1, ci = (R)0;
        for (int m = 0; m < km1; ++m) {
            if (m > 0 && (m & 3) == 0) {
                double t = 2.0 * m * frac[d];
                t -= 2.0 * floor(0.5 * t + 0.5);
                f_sincospi((R)t, &ci, &cr);
            }
            V2<R> e;
            e.x = cr * qd;
            e.y = ci * qd;
            ph[(size_t)(d * km1 + m) * ns + s] = e;
            const R nr = cr * c1 - ci * s1;
            ci = cr * s1 + ci * c1;
            cr = nr;
        }
    }
}

// FP32 form of k_prep with one thread per (site, dimension): each dimension of
// the M site, the box fraction, the fixed-point fraction and the phase-table
// rows depend on that dimension alone. Blocks are dimension-major (a block's
// threads share d), so the phase rows are written by consecutive sites.
__global__ void __launch_bounds__(128) k_prep_f32(EvalArgs a) {
    pdl_wait();  // the positions of the ring step ahead
    const Job J = a.jobs[blockIdx.y];
    const SysDev &S = a.sys[J.sys];
    const int ns = S.n_sites;
    const int tiles = (3 * a.max_mols + 127) / 128;
    const int d = blockIdx.x / tiles;
    const int s = (blockIdx.x - d * tiles) * 128 + threadIdx.x;
    if (s == 0 && d == 0) a.energy[J.slot] = 0.0;
    if (s >= ns) return;
    const int mol = s / 3, kind = s - 3 * mol;
    const double *q = a.pos + J.pos_off;
    const double g = a.c.gamma_vs, h = 0.5 * (1.0 - g);
    double x, u = 0.0;
    // box fractions in 32-bit fixed point: the low 32 bits of round(x 2^32 / L), an
    // FP64 product (exact scaling by 2^32 of x / L rounded once) and one conversion;
    // the wrapped FP32 coordinates follow from the fixed-point value
    if (a.sites_are_input || kind != 0) {
        x = q[3 * s + d];
        if (J.mode == 1) u = a.dir[J.pos_off + 3 * s + d];
    } else {
        // M site (forces.cpp:558-564)
        x = fma(g, q[9 * mol + d], h * (q[9 * mol + 3 + d] + q[9 * mol + 6 + d]));
        if (J.mode == 1) {
            const double *v = a.dir + J.pos_off;
            u = fma(g, v[9 * mol + d], h * (v[9 * mol + 3 + d] + v[9 * mol + 6 + d]));
        }
        // wrapped oxygen position for the Lennard-Jones kernel and the skin test
        const unsigned FO = (unsigned)__double2ll_rn(q[9 * mol + d] * S.fix_scale[d]);
        float *o = reinterpret_cast<float *>(a.opos) + 4 * ((size_t)J.site_off / 3 + mol);
        o[d] = (float)FO * S.fixf[d];
        if (d == 0) o[3] = 0.f;
    }
    const unsigned F = (unsigned)__double2ll_rn(x * S.fix_scale[d]);
    float *sv = reinterpret_cast<float *>(a.sites) + 4 * ((size_t)J.site_off + s);
    float xf = (float)F * S.fixf[d];
    if (a.rl_on && !a.sites_are_input && kind != 0) {
        // (pair-list real space) an H site follows its molecule's wrapped M site across the box boundary
        // (the wrapped fixed-point difference is the M-H minimum image), so the
        // FP32 positions of a molecule's sites stay together: one minimum image per
        // molecule pair serves all nine site pairs in k_real_list
        const double xm = fma(g, q[9 * mol + d], h * (q[9 * mol + 3 + d] + q[9 * mol + 6 + d]));
        const unsigned FM = (unsigned)__double2ll_rn(xm * S.fix_scale[d]);
        xf = fmaf((float)(int)(F - FM), S.fixf[d], (float)FM * S.fixf[d]);
    }
    sv[d] = xf;
    int *fx = reinterpret_cast<int *>(a.sites_fix + J.site_off + s);
    fx[d] = (int)F;
    if (a.rfix) a.rfix[3 * ((size_t)J.site_off + s) + d] = 0;  // k_real_half adds into it
    float cf = 1.f;
    if (d == 0) {
        cf = (float)a.charge[S.chg_off + s];
        sv[3] = cf;
        fx[3] = __float_as_int(cf);
    }
    if (J.mode == 1) {
        float *tv = reinterpret_cast<float *>(a.tan_sites) + 4 * ((size_t)J.site_off + s);
        tv[d] = (float)u;
        if (d == 0) tv[3] = 0.f;
    }
    // phase row d: exp(i 2 pi m frac) by complex recursion, reseeded every 4 powers
    // from the exact fixed-point argument m F (see k_prep)
    const int km1 = S.k_max + 1;
    float2 *ph = reinterpret_cast<float2 *>(a.phase) + J.phase_off;
    float s1, c1;
    sincospif((float)(int)F * 4.656612873077393e-10f, &s1, &c1);
    const float qd = cf;  // the charge in row 0 (x), 1 in the y and z rows
    float cr = 1.f, ci = 0.f;
    for (int m = 0; m < km1; ++m) {
        if (m > 0 && (m & 3) == 0) sincospif((float)(int)((unsigned)m * F) * 4.656612873077393e-10f, &ci, &cr);
        ph[(size_t)(d * km1 + m) * ns + s] = make_float2(cr * qd, ci * qd);
        const float nr = cr * c1 - ci * s1;
        ci = cr * s1 + ci * c1;
        cr = nr;
    }
}

void launch_prep_f32(const EvalArgs &a, cudaStream_t s) {
    const int tiles = (3 * a.max_mols + 127) / 128;
    launch_pdl(k_prep_f32, dim3(3 * tiles, a.n_jobs), dim3(128), 0, s, a);
}

// Running sum s (+ compensation c) += v, Kahan's compensated summation.
template <typename R>
__device__ __forceinline__ void kahan_add(R &s, R &c, R v) {
    const R y = v - c;
    const R t = s + y;
    c = (t - s) - y;
    s = t;
}

// Partial site-force planes: FP64 in the FP64 form; FP32 in the mixed form
// (each plane is a compensated FP32 sum rounded once; k_combine_f32 adds the
// planes with compensation), which halves their traffic and keeps the plane
// sum off the FP64 pipe.
template <typename R>
__device__ __forceinline__ void store_plane(double *part, size_t at3, R x, R y, R z);
template <>
__device__ __forceinline__ void store_plane<double>(double *part, size_t at3, double x, double y, double z) {
    part[at3] = x;
    part[at3 + 1] = y;
    part[at3 + 2] = z;
}
template <>
__device__ __forceinline__ void store_plane<float>(double *part, size_t at3, float x, float y, float z) {
    float *p = reinterpret_cast<float *>(part) + at3;
    p[0] = x;
    p[1] = y;
    p[2] = z;
}

// ---- k_real: intermolecular real-space Ewald ----------------------------------
constexpr int RT = 128;

template <typename R, int MODE>
__global__ void __launch_bounds__(RT) k_real(EvalArgs a) {
    const int rj = blockIdx.y, jb = blockIdx.z;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int ns = S.n_sites;
    if (blockIdx.x * RT >= ns) return;
    const int i = blockIdx.x * RT + threadIdx.x;
    const bool act = i < ns;
    const int j0 = chunk_lo(ns, rj, a.n_rj), j1 = chunk_lo(ns, rj + 1, a.n_rj);
    const V4<R> *sites = reinterpret_cast<const V4<R> *>(a.sites) + J.site_off;
    const V4<R> *tans = reinterpret_cast<const V4<R> *>(a.tan_sites) + J.site_off;
    __shared__ V4<R> sj[RT];
    __shared__ V4<R> uj[MODE == 1 ? RT : 1];
    __shared__ double red[RT / 32];
    const R L0 = sys_box<R>(S, 0), L1 = sys_box<R>(S, 1), L2 = sys_box<R>(S, 2);
    const R I0 = sys_ibox<R>(S, 0), I1 = sys_ibox<R>(S, 1), I2 = sys_ibox<R>(S, 2);
    const R rc2 = (R)S.rc_sq, kap = (R)S.kappa, kap2 = (R)(S.kappa * S.kappa), pref = (R)S.ewald_pref;
    V4<R> si;
    si.x = si.y = si.z = si.w = (R)0;
    V4<R> ui = si;
    if (act) {
        si = sites[i];
        if (MODE == 1) ui = tans[i];
    }
    const int mlo = (i / 3) * 3;  // first site of i's molecule
    double Fx = 0.0, Fy = 0.0, Fz = 0.0, E = 0.0;
    for (int t0 = j0; t0 < j1; t0 += RT) {
        __syncthreads();
        if (t0 + threadIdx.x < j1) {
            sj[threadIdx.x] = sites[t0 + threadIdx.x];
            if (MODE == 1) uj[threadIdx.x] = tans[t0 + threadIdx.x];
        }
        __syncthreads();
        const int nj = min(RT, j1 - t0);
        R fx = 0, fy = 0, fz = 0, e = 0;
        if (act) {
            for (int jj = 0; jj < nj; ++jj) {
                if ((unsigned)(t0 + jj - mlo) < 3u) continue;  // same molecule
                const V4<R> b = sj[jj];
                R dx = si.x - b.x, dy = si.y - b.y, dz = si.z - b.z;
                dx -= L0 * f_rint(dx * I0);
                dy -= L1 * f_rint(dy * I1);
                dz -= L2 * f_rint(dz * I2);
                const R r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rc2) {
                    R inv, ex, ec;
                    pair_terms(r2, kap, kap2, &inv, &ex, &ec);
                    const R qq = si.w * b.w;
                    const R en = qq * inv * ec;
                    const R hq = qq * pref * ex;
                    const R phi = (en + hq) * inv * inv;
                    if (MODE == 0) {
                        e += en;
                        fx += phi * dx;
                        fy += phi * dy;
                        fz += phi * dz;
                    } else {
                        // d/d(eps) of phi(r^2) r along u = u_i - u_j:
                        // phi' = dphi/d(r^2) = -1.5 phi / r^2 - kappa^2 hq / r^2
                        const V4<R> ub = uj[jj];
                        const R ux = ui.x - ub.x, uy = ui.y - ub.y, uz = ui.z - ub.z;
                        const R ru = dx * ux + dy * uy + dz * uz;
                        const R dphi = (-(R)1.5 * phi - kap2 * hq) * inv * inv;
                        const R c2 = (R)2 * dphi * ru;
                        fx += phi * ux + c2 * dx;
                        fy += phi * uy + c2 * dy;
                        fz += phi * uz + c2 * dz;
                    }
                }
            }
        }
        Fx += (double)fx;
        Fy += (double)fy;
        Fz += (double)fz;
        E += (double)e;
    }
    if (act) store_plane<R>(a.part, 3 * ((size_t)rj * a.total_sites + J.site_off + i), (R)Fx, (R)Fy, (R)Fz);
    if (MODE == 0) {
        const double t = block_sum(0.5 * E, red);
        if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
    }
}

// FP32 form of k_real<float, 0> (energies and forces): the pair term is
// q_i q_j [A, (A + B) / r^2] with A = erfc(kappa r) / r and
// B = (2 kappa / sqrt(pi)) exp(-kappa^2 r^2); q_i is factored out of the sums,
// the same-molecule exclusion joins the cutoff predicate, and each 128-site
// tile's FP32 sums are added into Kahan-compensated FP32 running sums (FP64
// only when the plane is written).
__global__ void __launch_bounds__(RT) k_real_f32(EvalArgs a) {
    const int rj = blockIdx.y, jb = blockIdx.z;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int ns = S.n_sites;
    if (blockIdx.x * RT >= ns) return;
    const int i = blockIdx.x * RT + threadIdx.x;
    const bool act = i < ns;
    const int j0 = chunk_lo(ns, rj, a.n_rj), j1 = chunk_lo(ns, rj + 1, a.n_rj);
    const float4 *sites = reinterpret_cast<const float4 *>(a.sites) + J.site_off;
    __shared__ float4 sj[RT];
    __shared__ double red[RT / 32];
    const float L0 = S.boxf[0], L1 = S.boxf[1], L2 = S.boxf[2];
    const float I0 = S.inv_boxf[0], I1 = S.inv_boxf[1], I2 = S.inv_boxf[2];
    const float rc2 = (float)S.rc_sq, ka = (float)(0.3275911 * S.kappa);
    const float cex = (float)(-S.kappa * S.kappa * 1.4426950408889634), pref = (float)S.ewald_pref;
    float4 si = make_float4(0.f, 0.f, 0.f, 0.f);
    if (act) si = sites[i];
    const int mlo = (i / 3) * 3;  // first site of i's molecule
    float Sx = 0.f, Sy = 0.f, Sz = 0.f, Se = 0.f, Cx = 0.f, Cy = 0.f, Cz = 0.f, Ce = 0.f;
    for (int t0 = j0; t0 < j1; t0 += RT) {
        __syncthreads();
        if (t0 + threadIdx.x < j1) sj[threadIdx.x] = sites[t0 + threadIdx.x];
        __syncthreads();
        const int nj = min(RT, j1 - t0);
        const int moff = mlo - t0;  // same molecule: (unsigned)(jj - moff) < 3
        float fx = 0.f, fy = 0.f, fz = 0.f, e = 0.f;
        if (act) {
#pragma unroll 4
            for (int jj = 0; jj < nj; ++jj) {
                const float4 b = sj[jj];
                float dx = si.x - b.x, dy = si.y - b.y, dz = si.z - b.z;
                dx = fmaf(-L0, rintf(dx * I0), dx);
                dy = fmaf(-L1, rintf(dy * I1), dy);
                dz = fmaf(-L2, rintf(dz * I2), dz);
                const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                if (r2 < rc2 && (unsigned)(jj - moff) >= 3u) {
                    const float iv = rsqrt_approx(r2);
                    const float ex = ex2_approx(cex * r2);
                    const float t = rcp_approx(fmaf(ka, r2 * iv, 1.0f));
                    const float A = (t * as_poly(t)) * ex * iv;
                    const float w = b.w * fmaf(pref, ex, A) * (iv * iv);
                    e = fmaf(b.w, A, e);
                    fx = fmaf(w, dx, fx);
                    fy = fmaf(w, dy, fy);
                    fz = fmaf(w, dz, fz);
                }
            }
        }
        kahan_add(Sx, Cx, fx);
        kahan_add(Sy, Cy, fy);
        kahan_add(Sz, Cz, fz);
        kahan_add(Se, Ce, e);
    }
    const double qi = (double)si.w;
    if (act)
        store_plane<float>(a.part, 3 * ((size_t)rj * a.total_sites + J.site_off + i), si.w * (Sx - Cx),
                           si.w * (Sy - Cy), si.w * (Sz - Cz));
    const double t = block_sum(0.5 * qi * ((double)Se - (double)Ce), red);
    if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
}

// ---- real-space pair list (mixed form, beads beyond the half-interaction kernel) ----
// The reference's real-space sum (forces.cpp:589-608) visits every site pair of
// different molecules and keeps those within r_c. For large beads the pairs
// within r_c are found through a list per (slot) configuration: row i holds, in
// ascending order, every molecule j != i that had a site pair within r_c + RL_SKIN
// when the list was built. The list stays complete while no two sites have moved
// by more than RL_SKIN between them since the build, the Verlet argument of
// neighbour.cpp applied to sites: k_rlist_test rebuilds it when the two largest
// site displacements sum to more than the skin (or were never measured).
// k_prep_f32 keeps a molecule's FP32 sites together (H sites follow the wrapped M
// site). While every site lies within RL_SPREAD of its M site and r_c +
// 2 RL_SPREAD <= L/2 (the context's eligibility test), the M-M minimum image of a
// molecule pair is the minimum image of each of its site pairs within r_c, so one
// image serves nine pairs; a configuration with a wider molecule ("wide", found by
// k_rlist_test) takes a minimum image per site pair instead, in the build and in
// the force sum.
constexpr int RL_ROWS = 8;  // rows (warps) per block of k_rlist_rows
constexpr int RLW = 4;      // molecules (warps) per block of k_real_list

struct RlBox {
    float L0, L1, L2, I0, I1, I2;
};
__device__ __forceinline__ RlBox rl_box(const SysDev &S) {
    return {S.boxf[0], S.boxf[1], S.boxf[2], S.inv_boxf[0], S.inv_boxf[1], S.inv_boxf[2]};
}
// minimum image of a difference vector
__device__ __forceinline__ void rl_image(const RlBox &B, float &dx, float &dy, float &dz) {
    dx = fmaf(-B.L0, rintf(dx * B.I0), dx);
    dy = fmaf(-B.L1, rintf(dy * B.I1), dy);
    dz = fmaf(-B.L2, rintf(dz * B.I2), dz);
}

// The list's validity and the molecules' spread, RLT_SITES sites a block, any
// number of blocks a configuration: the two largest site displacements since
// the build (compared as the bit patterns of their non-negative squares, a NaN
// above all) are merged over the blocks with two atomic maxima (a block's largest
// either becomes the maximum or bids, through the smaller of itself and the
// maximum it displaced, for the second), and the block that arrives last on the
// configuration's ticket decides, re-arms the state and, when the list is
// rebuilt, adds the configuration to the launch's list of rebuilding ones.
constexpr int RLT_SITES = 2048;
__global__ void __launch_bounds__(256) k_rlist_test(EvalArgs a) {
    const Job J = a.jobs[blockIdx.y];
    const SysDev &S = a.sys[J.sys];
    const int ns = S.n_sites;
    const float4 *sites = reinterpret_cast<const float4 *>(a.sites) + J.site_off;
    const float4 *ref = a.rl_ref + J.site_off;
    const RlBox B = rl_box(S);
    constexpr float sp2 = RL_SPREAD * RL_SPREAD;
    unsigned m1 = 0u, m2 = 0u;
    int wide = 0;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < ns; k += gridDim.x * blockDim.x) {
        const float4 p = sites[k], r = ref[k];
        float dx = p.x - r.x, dy = p.y - r.y, dz = p.z - r.z;
        rl_image(B, dx, dy, dz);
        const unsigned d2 = __float_as_uint(fmaf(dx, dx, fmaf(dy, dy, dz * dz)));
        if (d2 > m1) {
            m2 = m1;
            m1 = d2;
        } else if (d2 > m2) {
            m2 = d2;
        }
        const int kind = k % 3;
        if (kind) {
            const float4 m = sites[k - kind];
            const float hx = p.x - m.x, hy = p.y - m.y, hz = p.z - m.z;
            if (!(fmaf(hx, hx, fmaf(hy, hy, hz * hz)) <= sp2)) wide = 1;
        }
    }
    for (int o = 16; o > 0; o >>= 1) {
        const unsigned b1 = __shfl_xor_sync(0xffffffffu, m1, o), b2 = __shfl_xor_sync(0xffffffffu, m2, o);
        const unsigned n1 = max(m1, b1), n2 = max(min(m1, b1), max(m2, b2));
        m1 = n1;
        m2 = n2;
    }
    __shared__ unsigned red[2][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) {
        red[0][w] = m1;
        red[1][w] = m2;
    }
    wide = __syncthreads_or(wide);
    if (threadIdx.x != 0) return;
    unsigned t1 = 0u, t2 = 0u;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
        const unsigned n1 = max(t1, red[0][k]), n2 = max(min(t1, red[0][k]), max(t2, red[1][k]));
        t1 = n1;
        t2 = n2;
    }
    uint4 *st = a.rl_state + J.slot;  // (largest, second, wide, ticket)
    const unsigned o = atomicMax(&st->x, t1);
    atomicMax(&st->y, max(t2, min(t1, o)));
    if (wide) atomicOr(&st->z, 1u);
    __threadfence();
    if (atomicAdd(&st->w, 1u) != gridDim.x - 1) return;
    __threadfence();
    const unsigned g1 = atomicExch(&st->x, 0u), g2 = atomicExch(&st->y, 0u), wd = atomicExch(&st->z, 0u);
    atomicExch(&st->w, 0u);
    a.rl_wide[J.slot] = wd ? 1 : 0;
    if (!(sqrtf(__uint_as_float(g1)) + sqrtf(__uint_as_float(g2)) <= RL_SKIN))
        a.rl_jobs[atomicAdd(a.rl_count, 1)] = blockIdx.y;
}

// Whether some site pair of molecules (a0, a1, a2) and (b0, b1, b2) lies within
// R (R2 = R^2). Not WIDE: the M-M image for all nine pairs, after an M-M
// prefilter at R + 2 RL_SPREAD (P2); WIDE: a minimum image per pair.
template <bool WIDE>
__device__ __forceinline__ bool rl_near(const float4 *sites, int j, const float4 &a0, const float4 &a1,
                                        const float4 &a2, const RlBox &B, float R2, float P2) {
    const float4 b0 = sites[3 * j];
    float sx = 0.f, sy = 0.f, sz = 0.f;
    if (!WIDE) {
        sx = B.L0 * rintf((a0.x - b0.x) * B.I0);
        sy = B.L1 * rintf((a0.y - b0.y) * B.I1);
        sz = B.L2 * rintf((a0.z - b0.z) * B.I2);
        const float dx = a0.x - sx - b0.x, dy = a0.y - sy - b0.y, dz = a0.z - sz - b0.z;
        if (!(fmaf(dx, dx, fmaf(dy, dy, dz * dz)) < P2)) return false;
    }
    const float4 b1 = sites[3 * j + 1], b2 = sites[3 * j + 2];
    const float4 ai[3] = {a0, a1, a2}, bj[3] = {b0, b1, b2};
    float m = 3.4e38f;
#pragma unroll
    for (int u = 0; u < 3; ++u)
#pragma unroll
        for (int v = 0; v < 3; ++v) {
            float ex = ai[u].x - sx - bj[v].x, ey = ai[u].y - sy - bj[v].y, ez = ai[u].z - sz - bj[v].z;
            if (WIDE) rl_image(B, ex, ey, ez);
            m = fminf(m, fmaf(ex, ex, fmaf(ey, ey, ez * ez)));
        }
    return m < R2;
}

// Rows of the rebuilding jobs' lists, a warp per row i over a fixed grid of
// (rebuilding job, RL_ROWS rows) items: the 32 lanes test 32 molecules j at a
// time and a ballot places the hits in ascending j.
__global__ void __launch_bounds__(32 * RL_ROWS) k_rlist_rows(EvalArgs a, int row_blocks) {
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long n_items = (long long)(*a.rl_count) * row_blocks;
    for (long long it = blockIdx.x; it < n_items; it += gridDim.x) {
        const Job J = a.jobs[a.rl_jobs[it / row_blocks]];
        const SysDev &S = a.sys[J.sys];
        const int N = S.n_mols, i = (int)(it % row_blocks) * RL_ROWS + w;
        if (i >= N) continue;
        const float4 *sites = reinterpret_cast<const float4 *>(a.sites) + J.site_off;
        const RlBox B = rl_box(S);
        const float R = sqrtf(S.rc_sqf) + RL_SKIN, R2 = R * R;
        const float P = R + 2.0f * RL_SPREAD, P2 = P * P;
        const bool wide = a.rl_wide[J.slot] != 0;
        const float4 a0 = sites[3 * i], a1 = sites[3 * i + 1], a2 = sites[3 * i + 2];
        // the build's positions, for the next displacement tests
        if (lane < 3) a.rl_ref[J.site_off + 3 * i + lane] = lane == 0 ? a0 : (lane == 1 ? a1 : a2);
        unsigned short *row = a.rl_list + ((size_t)J.site_off / 3 + i) * a.rl_cap;
        int cnt = 0;
        for (int j0 = 0; j0 < N; j0 += 32) {
            const int j = j0 + lane;
            bool hit = false;
            if (j < N && j != i)
                hit = wide ? rl_near<true>(sites, j, a0, a1, a2, B, R2, P2)
                           : rl_near<false>(sites, j, a0, a1, a2, B, R2, P2);
            const unsigned bal = __ballot_sync(0xffffffffu, hit);
            if (hit) {
                const int at = cnt + __popc(bal & ((1u << lane) - 1u));
                if (at < a.rl_cap) row[at] = (unsigned short)j;
            }
            cnt += __popc(bal);
        }
        if (lane == 0) {
            a.rl_cnt[(size_t)J.site_off / 3 + i] = min(cnt, a.rl_cap);
            if (cnt > a.rl_cap) atomicOr(a.status, (unsigned)ST_RLIST_OVERFLOW);
        }
    }
}

// One site pair of k_real_list: the FP32 pair term of k_real_f32 with the
// cutoff applied through the j charge (branch-free), accumulated into the i
// site's sums; MI: the difference vector takes its own minimum image.
struct RlPair {
    float rc2, ka, cex, pref;
};
template <bool MI>
__device__ __forceinline__ void rl_pair(float ax, float ay, float az, const float4 b, const RlBox &B,
                                        const RlPair &K, float &fx, float &fy, float &fz, float &e) {
    float dx = ax - b.x, dy = ay - b.y, dz = az - b.z;
    if (MI) rl_image(B, dx, dy, dz);
    const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
    const float iv = rsqrt_approx(r2);
    const float ex = ex2_approx(K.cex * r2);
    const float t = rcp_approx(fmaf(K.ka, r2 * iv, 1.0f));
    const float A = (t * as_poly(t)) * ex * iv;
    const float qb = r2 < K.rc2 ? b.w : 0.0f;
    const float wq = qb * fmaf(K.pref, ex, A) * (iv * iv);
    e = fmaf(qb, A, e);
    fx = fmaf(wq, dx, fx);
    fy = fmaf(wq, dy, fy);
    fz = fmaf(wq, dz, fz);
}

// A lane's share of row i in k_real_list: listed molecules lo + lane, lo + lane
// + 32, ... below hi; nine site pairs each (WIDE: a minimum image per pair, else
// the i sites shifted by the M-M image once per j).
template <bool WIDE>
__device__ __forceinline__ void rl_row(const float4 *sites, const unsigned short *row, int lo, int hi,
                                       const float4 &a0, const float4 &a1, const float4 &a2, const RlBox &B,
                                       const RlPair &K, float (&f)[9], float &e0, float &e1, float &e2) {
    for (int k = lo + (threadIdx.x & 31); k < hi; k += 32) {
        const int j = row[k];
        const float4 b0 = __ldg(sites + 3 * j), b1 = __ldg(sites + 3 * j + 1), b2 = __ldg(sites + 3 * j + 2);
        float sx = 0.f, sy = 0.f, sz = 0.f;
        if (!WIDE) {
            sx = B.L0 * rintf((a0.x - b0.x) * B.I0);
            sy = B.L1 * rintf((a0.y - b0.y) * B.I1);
            sz = B.L2 * rintf((a0.z - b0.z) * B.I2);
        }
        const float x0 = a0.x - sx, y0 = a0.y - sy, z0 = a0.z - sz;
        const float x1 = a1.x - sx, y1 = a1.y - sy, z1 = a1.z - sz;
        const float x2 = a2.x - sx, y2 = a2.y - sy, z2 = a2.z - sz;
        rl_pair<WIDE>(x0, y0, z0, b0, B, K, f[0], f[1], f[2], e0);
        rl_pair<WIDE>(x0, y0, z0, b1, B, K, f[0], f[1], f[2], e0);
        rl_pair<WIDE>(x0, y0, z0, b2, B, K, f[0], f[1], f[2], e0);
        rl_pair<WIDE>(x1, y1, z1, b0, B, K, f[3], f[4], f[5], e1);
        rl_pair<WIDE>(x1, y1, z1, b1, B, K, f[3], f[4], f[5], e1);
        rl_pair<WIDE>(x1, y1, z1, b2, B, K, f[3], f[4], f[5], e1);
        rl_pair<WIDE>(x2, y2, z2, b0, B, K, f[6], f[7], f[8], e2);
        rl_pair<WIDE>(x2, y2, z2, b1, B, K, f[6], f[7], f[8], e2);
        rl_pair<WIDE>(x2, y2, z2, b2, B, K, f[6], f[7], f[8], e2);
    }
}

// Real-space Ewald over the pair list (energies and forces): a warp per
// (molecule i, chunk rj of its row), a lane per listed molecule j at a time. The
// warp's sums are reduced by shuffles in a fixed order and written as plane rj
// (deterministic, no atomics on forces).
__global__ void __launch_bounds__(32 * RLW) k_real_list(EvalArgs a) {
    const int rj = blockIdx.y, w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const Job J = a.jobs[blockIdx.z];
    const SysDev &S = a.sys[J.sys];
    const int N = S.n_mols;
    if ((int)blockIdx.x * RLW >= N) return;
    const int i = blockIdx.x * RLW + w;
    const bool act = i < N;
    const float4 *sites = reinterpret_cast<const float4 *>(a.sites) + J.site_off;
    const RlBox B = rl_box(S);
    const RlPair K = {S.rc_sqf, S.kaf, S.cexf, S.ewald_preff};
    float4 a0 = make_float4(0.f, 0.f, 0.f, 0.f), a1 = a0, a2 = a0;
    int lo = 0, hi = 0;
    if (act) {
        a0 = sites[3 * i];
        a1 = sites[3 * i + 1];
        a2 = sites[3 * i + 2];
        const int c = a.rl_cnt[(size_t)J.site_off / 3 + i];
        lo = chunk_lo(c, rj, a.n_rj);
        hi = chunk_lo(c, rj + 1, a.n_rj);
    }
    const unsigned short *row = a.rl_list + ((size_t)J.site_off / 3 + i) * a.rl_cap;
    float f[9], e0 = 0.f, e1 = 0.f, e2 = 0.f;
#pragma unroll
    for (int k = 0; k < 9; ++k) f[k] = 0.f;
    if (a.rl_wide[J.slot]) rl_row<true>(sites, row, lo, hi, a0, a1, a2, B, K, f, e0, e1, e2);
    else rl_row<false>(sites, row, lo, hi, a0, a1, a2, B, K, f, e0, e1, e2);
    float e = 0.5f * (a0.w * e0 + a1.w * e1 + a2.w * e2);
#pragma unroll
    for (int k = 0; k < 9; ++k) f[k] = warp_sum(f[k]);
    e = warp_sum(e);
    if (act && lane < 3) {
        // lane p stores site p (selects: a lane-dependent index into f would go
        // through local memory)
        const float q = lane == 0 ? a0.w : (lane == 1 ? a1.w : a2.w);
        const float fx = lane == 0 ? f[0] : (lane == 1 ? f[3] : f[6]);
        const float fy = lane == 0 ? f[1] : (lane == 1 ? f[4] : f[7]);
        const float fz = lane == 0 ? f[2] : (lane == 1 ? f[5] : f[8]);
        store_plane<float>(a.part, 3 * ((size_t)rj * a.total_sites + J.site_off + 3 * i + lane), q * fx, q * fy,
                           q * fz);
    }
    __shared__ double red[RLW];
    if (lane == 0) red[w] = act ? (double)e : 0.0;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int k = 0; k < RLW; ++k) t += red[k];
        atomicAdd(&a.energy[J.slot], t);
    }
}

// Half-interaction form of k_real_f32 (energies and forces, beads of at most
// HALF_MAX_TILES tiles of 32 sites): every site pair is evaluated once. A warp
// holds tile J of a bead in registers (one site a lane) and visits the tiles at
// ring distances d = 1 .. T/2 from it (distance T/2 of an even ring only from
// the first half of the tiles); the visited tile's sites and their force
// accumulators rotate through the lanes by shuffles, 32 steps bringing them
// back home. The stationary tile's own pairs (d = 0) are taken from both sides.
// Sites are read as 32-bit fixed-point box fractions (k_prep), whose wrapped
// integer differences are minimum-image separations to 2^-32 of the box.
// Both sides' site forces are added into one array a configuration (a.rfix,
// zeroed by k_prep_f32) as 64-bit fixed point (2^-40 Hartree/bohr) by integer
// atomics: the visited sites' sums after each visit, the stationary sites' Kahan
// sums over the block's distance chunk ch at the end. Integer addition is
// associative, so the totals are the same bits whatever order the warps finish
// in; k_combine_f32 reads the array after the float planes of the other terms.
constexpr int HW = 4;  // warps per block
constexpr float RFIX_SCALE = 1099511627776.0f;  // 2^40: fixed-point units of the real-space site forces
__device__ __forceinline__ void rfix_add(long long *p, float x, float y, float z) {
    atomicAdd(reinterpret_cast<unsigned long long *>(p), (unsigned long long)__float2ll_rn(x * RFIX_SCALE));
    atomicAdd(reinterpret_cast<unsigned long long *>(p + 1), (unsigned long long)__float2ll_rn(y * RFIX_SCALE));
    atomicAdd(reinterpret_cast<unsigned long long *>(p + 2), (unsigned long long)__float2ll_rn(z * RFIX_SCALE));
}
__global__ void __launch_bounds__(32 * HW) k_real_half(EvalArgs a, int n_ch) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ch = blockIdx.y, jb = blockIdx.z;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int ns = S.n_sites, T = (ns + 31) / 32;
    const int tJ = blockIdx.x * HW + warp;
    if (tJ >= T) return;
    const int maxd = T / 2;
    const int d0 = chunk_lo(maxd + 1, ch, n_ch), d1 = chunk_lo(maxd + 1, ch + 1, n_ch);
    // sites as 32-bit fixed-point box fractions: the wrapped difference of two
    // fractions is the minimum image, one integer subtraction and one conversion
    // a component (scaled by L / 2^32)
    const int4 *sites = a.sites_fix + J.site_off;
    const float X0 = S.fixf[0], X1 = S.fixf[1], X2 = S.fixf[2];
    const float rc2 = S.rc_sqf, ka = S.kaf, cex = S.cexf, pref = S.ewald_preff;
    const int s = tJ * 32 + lane, ms = s / 3;
    const bool vs = s < ns;
    // the visited tile twice over, so that step r of lane l reads entry l + r
    __shared__ int4 vis[HW][64];
    int4 ps = make_int4(0, 0, 0, 0);
    if (vs) ps = sites[s];
    const float qs = __int_as_float(ps.w);
    auto disp = [&](const int4 &pm, float &dx, float &dy, float &dz) {
        dx = (float)(int)((unsigned)ps.x - (unsigned)pm.x) * X0;
        dy = (float)(int)((unsigned)ps.y - (unsigned)pm.y) * X1;
        dz = (float)(int)((unsigned)ps.z - (unsigned)pm.z) * X2;
    };
    // w = q_s q_m (A + B) / r^2 along d = r_s - r_m; returns q_s q_m A (the pair energy)
    auto pair = [&](const int4 &pm, float &dx, float &dy, float &dz, float &w) -> float {
        disp(pm, dx, dy, dz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        w = 0.f;
        if (!(r2 < rc2)) return 0.f;
        const float iv = rsqrt_approx(r2);
        const float ex = ex2_approx(cex * r2);
        const float t = rcp_approx(fmaf(ka, r2 * iv, 1.0f));
        const float A = (t * as_poly(t)) * ex * iv;
        const float qq = qs * __int_as_float(pm.w);
        w = qq * fmaf(pref, ex, A) * (iv * iv);
        return qq * A;
    };
    // the same pair without a branch (the test-free loop between distant tiles):
    // a pair beyond r_c is evaluated at r_c and weighted by zero
    auto pair_nb = [&](const int4 &pm, float &dx, float &dy, float &dz, float &w) -> float {
        disp(pm, dx, dy, dz);
        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
        const bool in = r2 < rc2;
        const float rr = in ? r2 : rc2;
        const float iv = rsqrt_approx(rr);
        const float ex = ex2_approx(cex * rr);
        const float t = rcp_approx(fmaf(ka, rr * iv, 1.0f));
        const float A = (t * as_poly(t)) * ex * iv;
        const float qq = in ? qs * __int_as_float(pm.w) : 0.f;
        w = qq * fmaf(pref, ex, A) * (iv * iv);
        return qq * A;
    };
    float Sx = 0.f, Sy = 0.f, Sz = 0.f, Cx = 0.f, Cy = 0.f, Cz = 0.f, e = 0.f;
    for (int d = d0; d < d1; ++d) {
        float fx = 0.f, fy = 0.f, fz = 0.f;
        if (d == 0) {  // the tile's own pairs, from both sides
            for (int r = 1; r < 32; ++r) {
                const int src = (lane + r) & 31;
                int4 pm;
                pm.x = __shfl_sync(0xffffffffu, ps.x, src);
                pm.y = __shfl_sync(0xffffffffu, ps.y, src);
                pm.z = __shfl_sync(0xffffffffu, ps.z, src);
                pm.w = __shfl_sync(0xffffffffu, ps.w, src);
                const int m = tJ * 32 + src;
                if (!vs || m >= ns || m / 3 == ms) continue;
                float dx, dy, dz, w;
                e += 0.5f * pair(pm, dx, dy, dz, w);
                fx = fmaf(w, dx, fx);
                fy = fmaf(w, dy, fy);
                fz = fmaf(w, dz, fz);
            }
        } else {
            const int tI = (tJ + d) % T;
            const bool active = !((T % 2 == 0) && d == maxd && tJ >= maxd);
            const int m0 = tI * 32;
            int4 pm = make_int4(0, 0, 0, 0);
            if (active && m0 + lane < ns) pm = sites[m0 + lane];
            float mx = 0.f, my = 0.f, mz = 0.f;
            // tiles two or more apart share no molecule (a molecule's three sites lie in
            // at most two consecutive tiles): between two full tiles every pair counts
            const bool plain = d >= 2 && (tJ + 1) * 32 <= ns && m0 + 32 <= ns;
            if (active && plain) {
                // the visited sites are read from the warp's shared-memory copy (one
                // 16-byte load a step); only their force accumulators rotate
                vis[warp][lane] = pm;
                vis[warp][lane + 32] = pm;
                __syncwarp();
                const int4 *vr = &vis[warp][lane];
                const int nx = (lane + 1) & 31;
                if (S.fix_cubic) {
                    // cubic box: distances in fixed-point units u = L / 2^32 (the integer
                    // differences themselves), constants scaled to match; forces come out
                    // in units of 1 / u^2 and energies of 1 / u, rescaled once at the end
                    const float rc2u = S.rc2u, cexu = S.cexu, kau = S.kau, prefu = S.prefu;
                    float eu = 0.f;
#pragma unroll 4
                    for (int r = 0; r < 32; ++r) {
                        const int4 pv = vr[r];
                        const float dx = (float)(int)((unsigned)ps.x - (unsigned)pv.x);
                        const float dy = (float)(int)((unsigned)ps.y - (unsigned)pv.y);
                        const float dz = (float)(int)((unsigned)ps.z - (unsigned)pv.z);
                        const float r2 = fmaf(dx, dx, fmaf(dy, dy, dz * dz));
                        const bool in = r2 < rc2u;
                        const float rr = in ? r2 : rc2u;
                        const float iv = rsqrt_approx(rr);
                        const float ex = ex2_approx(cexu * rr);
                        const float t = rcp_approx(fmaf(kau, rr * iv, 1.0f));
                        const float A = (t * as_poly(t)) * ex * iv;
                        const float qq = in ? qs * __int_as_float(pv.w) : 0.f;
                        const float w = qq * fmaf(prefu, ex, A) * (iv * iv);
                        eu = fmaf(qq, A, eu);
                        fx = fmaf(w, dx, fx);
                        fy = fmaf(w, dy, fy);
                        fz = fmaf(w, dz, fz);
                        mx = fmaf(-w, dx, mx);
                        my = fmaf(-w, dy, my);
                        mz = fmaf(-w, dz, mz);
                        mx = __shfl_sync(0xffffffffu, mx, nx);
                        my = __shfl_sync(0xffffffffu, my, nx);
                        mz = __shfl_sync(0xffffffffu, mz, nx);
                    }
                    const float s2 = S.s2u;
                    fx *= s2;
                    fy *= s2;
                    fz *= s2;
                    mx *= s2;
                    my *= s2;
                    mz *= s2;
                    e = fmaf(eu, S.invu, e);
                } else {
#pragma unroll 4
                    for (int r = 0; r < 32; ++r) {
                        const int4 pv = vr[r];
                        float dx, dy, dz, w;
                        e += pair_nb(pv, dx, dy, dz, w);
                        fx = fmaf(w, dx, fx);
                        fy = fmaf(w, dy, fy);
                        fz = fmaf(w, dz, fz);
                        mx = fmaf(-w, dx, mx);
                        my = fmaf(-w, dy, my);
                        mz = fmaf(-w, dz, mz);
                        mx = __shfl_sync(0xffffffffu, mx, nx);
                        my = __shfl_sync(0xffffffffu, my, nx);
                        mz = __shfl_sync(0xffffffffu, mz, nx);
                    }
                }
                __syncwarp();
            } else if (active) {
                for (int r = 0; r < 32; ++r) {
                    const int m = m0 + ((lane + r) & 31);
                    if (vs && m < ns && m / 3 != ms) {
                        float dx, dy, dz, w;
                        e += pair(pm, dx, dy, dz, w);
                        fx = fmaf(w, dx, fx);
                        fy = fmaf(w, dy, fy);
                        fz = fmaf(w, dz, fz);
                        mx = fmaf(-w, dx, mx);
                        my = fmaf(-w, dy, my);
                        mz = fmaf(-w, dz, mz);
                    }
                    // hand the visited site and its force one lane down
                    const int nx = (lane + 1) & 31;
                    pm.x = __shfl_sync(0xffffffffu, pm.x, nx);
                    pm.y = __shfl_sync(0xffffffffu, pm.y, nx);
                    pm.z = __shfl_sync(0xffffffffu, pm.z, nx);
                    pm.w = __shfl_sync(0xffffffffu, pm.w, nx);
                    mx = __shfl_sync(0xffffffffu, mx, nx);
                    my = __shfl_sync(0xffffffffu, my, nx);
                    mz = __shfl_sync(0xffffffffu, mz, nx);
                }
            }
            if (m0 + lane < ns) rfix_add(a.rfix + 3 * ((size_t)J.site_off + m0 + lane), mx, my, mz);
        }
        kahan_add(Sx, Cx, fx);
        kahan_add(Sy, Cy, fy);
        kahan_add(Sz, Cz, fz);
    }
    if (vs) rfix_add(a.rfix + 3 * ((size_t)J.site_off + s), Sx - Cx, Sy - Cy, Sz - Cz);
    for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
    if (lane == 0) atomicAdd(&a.energy[J.slot], (double)e);
}

// ---- k_ksk: structure factors ---------------------------------------------------
// One thread per group of <= 4 consecutive |kz| of one (kx, ky) column, each
// |kz| covering the pair kz = +|kz|, -|kz|; the column factor X(kx) Y(ky) of a
// site is formed once and multiplied by Z and conj(Z) with shared products. Sites are staged through shared memory in chunks of CH; each
// chunk's partial sums (registers, working precision) are added to FP64 running
// sums kept in shared memory.
// Asynchronous global -> shared copies (cp.async) of B = 8 or 16 bytes; an invalid
// source copies nothing and zero-fills the destination.
template <int B>
__device__ __forceinline__ void cp_async(void *dst, const void *src, bool valid) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int n = valid ? B : 0;
    if constexpr (B == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(n) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;\n" ::"r"(d), "l"(src), "n"(B), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

constexpr int KT = 128;  // threads (k groups) per block
constexpr int CH = 32;   // sites per shared-memory chunk


// KZ: |kz| values per group (each covering +kz and -kz), the context's group width.
// The FP32 energy/force form (G3) accumulates, per |kz| and with A = X Y = Ar + i Ai
// the site's column factor, the four sums T1 = sum Ar Zr, T2 = sum Ai Zi,
// U = sum (Ar + Ai) Zr and V = sum (Ar + Ai) Zi (Gauss's three-multiplication
// complex product, whose third products (Ar + Ai)(Zr +- Zi) are U +- V, with T1 and
// T2 shared by +kz and -kz): four FMAs for the pair instead of eight. Then
// S(+kz) = T1 - T2 + i (U + V - T1 - T2) and S(-kz) = T1 + T2 + i (U - V - T1 + T2).
template <typename R, int MODE, int KZ>
__global__ void __launch_bounds__(KT) k_ksk(EvalArgs a) {
    const int sc = blockIdx.y, jb = blockIdx.z;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    // the FP32 energy/force form runs over the half set (kx = 0, ky < 0 columns left out)
    const bool half = sizeof(R) == 4 && MODE == 0;
    const int ng = half ? S.n_grp_half : S.n_grp, ns = S.n_sites, km1 = S.k_max + 1;
    if (blockIdx.x * KT >= ng) return;
    const int t = blockIdx.x * KT + threadIdx.x;
    const bool act = t < ng;
    const int s0 = chunk_lo(ns, sc, a.n_sc), s1 = chunk_lo(ns, sc + 1, a.n_sc);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // two buffers (chunk i computed while chunk i + 1 is copied in)
    V4<R> *ush = reinterpret_cast<V4<R> *>(smem_raw);      // [2][CH] (mode 1)
    V2<R> *tab = reinterpret_cast<V2<R> *>(ush + 2 * CH);  // [2][3*km1][CH+1]
    constexpr bool G3 = sizeof(R) == 4 && MODE == 0;
    KGroup G;
    G.col = G.kz0 = G.n = 0;
    KCol C;
    C.kx = C.ky = C.m = C.k_begin = 0;
    if (act) {
        G = a.kgrp[S.grp_off + t];
        C = a.kcol[S.col_off + G.col];
    }
    const int ax = C.kx, ay = abs(C.ky);
    const R sy = C.ky < 0 ? (R)-1 : (R)1;
    const R bz = (R)(2.0 * PI_REF * S.inv_box[2]);
    const R kx = (R)(2.0 * PI_REF * C.kx * S.inv_box[0]), ky = (R)(2.0 * PI_REF * C.ky * S.inv_box[1]);
    // the group's |kz| values az = kz0 .. kz0 + n - 1; each covers kz = +az and -az
    int zrow[KZ];
    R kzr[KZ];
#pragma unroll
    for (int g = 0; g < KZ; ++g) {
        zrow[g] = (2 * km1 + min(G.kz0 + g, km1 - 1)) * (CH + 1);
        kzr[g] = bz * (R)(G.kz0 + g);
    }
    // compensated running sums over the chunk totals, [g][0] for +az, [g][1] for -az
    R Sr[KZ][2], Si[KZ][2], Cr[KZ][2], Ci[KZ][2], dSr[KZ][2], dSi[KZ][2], dCr[KZ][2], dCi[KZ][2];
#pragma unroll
    for (int g = 0; g < KZ; ++g)
#pragma unroll
        for (int h = 0; h < 2; ++h) Sr[g][h] = Si[g][h] = Cr[g][h] = Ci[g][h] = dSr[g][h] = dSi[g][h] = dCr[g][h] = dCi[g][h] = (R)0;
    const V2<R> *ph = reinterpret_cast<const V2<R> *>(a.phase) + J.phase_off;
    const V4<R> *tans = reinterpret_cast<const V4<R> *>(a.tan_sites) + J.site_off;
    const int rows = 3 * km1, nchunk = s1 > s0 ? (s1 - s0 + CH - 1) / CH : 0;
    // copies of chunk ci's phase rows (and tangents) into buffer ci & 1, zero past s1
    auto stage = [&](int ci) {
        const int c0 = s0 + ci * CH;
        V2<R> *tb = tab + (ci & 1) * rows * (CH + 1);
        for (int idx = threadIdx.x; idx < rows * CH; idx += KT) {
            const int row = idx / CH, c = idx - row * CH, s = c0 + c;
            cp_async<sizeof(V2<R>)>(tb + row * (CH + 1) + c, ph + (size_t)row * ns + min(s, s1 - 1), s < s1);
        }
        if (MODE == 1 && threadIdx.x < CH) {
            const int s = c0 + threadIdx.x;
            const V4<R> *src = tans + min(s, s1 - 1);
            V4<R> *dst = ush + (ci & 1) * CH + threadIdx.x;
            if constexpr (sizeof(V4<R>) == 16) {
                cp_async<16>(dst, src, s < s1);
            } else {
                cp_async<16>(dst, src, s < s1);
                cp_async<16>(reinterpret_cast<unsigned char *>(dst) + 16, reinterpret_cast<const unsigned char *>(src) + 16,
                             s < s1);
            }
        }
        cp_async_commit();
    };
    if (nchunk > 0) stage(0);
    for (int ci = 0; ci < nchunk; ++ci) {
        const int c0 = s0 + ci * CH;
        __syncthreads();  // every thread is done with buffer (ci + 1) & 1
        if (ci + 1 < nchunk) stage(ci + 1);
        else cp_async_commit();
        cp_async_wait<1>();  // this thread's copies of chunk ci have landed
        __syncthreads();     // and every other thread's
        const V2<R> *tab_c = tab + (ci & 1) * rows * (CH + 1);
        const V4<R> *ush_c = ush + (ci & 1) * CH;
        const int nc = min(CH, s1 - c0);
        R sr[KZ][2], si[KZ][2], dsr[KZ][2], dsi[KZ][2];
#pragma unroll
        for (int g = 0; g < KZ; ++g)
#pragma unroll
            for (int h = 0; h < 2; ++h) sr[g][h] = si[g][h] = dsr[g][h] = dsi[g][h] = (R)0;
        auto site = [&](int c) {
            const V2<R> x = tab_c[ax * (CH + 1) + c], y = tab_c[(km1 + ay) * (CH + 1) + c];
            const R yi = sy * y.y;
            const R pr = x.x * y.x - x.y * yi, pi = x.x * yi + x.y * y.x;
            if constexpr (G3) {
                const float ps = (float)(pr + pi);
#pragma unroll
                for (int g = 0; g < KZ; ++g) {
                    const V2<R> z = tab_c[zrow[g] + c];
                    sr[g][0] = fmaf((float)pr, (float)z.x, sr[g][0]);  // T1
                    sr[g][1] = fmaf((float)pi, (float)z.y, sr[g][1]);  // T2
                    si[g][0] = fmaf(ps, (float)z.x, si[g][0]);         // U
                    si[g][1] = fmaf(ps, (float)z.y, si[g][1]);         // V
                }
                return;
            }
            R kxyu = (R)0, uz = (R)0;
            if (MODE == 1) {
                const V4<R> u = ush_c[c];
                kxyu = kx * u.x + ky * u.y;
                uz = u.z;
            }
#pragma unroll
            for (int g = 0; g < KZ; ++g) {
                const V2<R> z = tab_c[zrow[g] + c];
                if (MODE == 0) {
                    // A Z (kz = +az) and A conj(Z) (kz = -az) accumulated by FMAs alone
                    sr[g][0] = fma(pr, z.x, sr[g][0]);
                    sr[g][0] = fma(-pi, z.y, sr[g][0]);
                    si[g][0] = fma(pi, z.x, si[g][0]);
                    si[g][0] = fma(pr, z.y, si[g][0]);
                    sr[g][1] = fma(pr, z.x, sr[g][1]);
                    sr[g][1] = fma(pi, z.y, sr[g][1]);
                    si[g][1] = fma(pi, z.x, si[g][1]);
                    si[g][1] = fma(-pr, z.y, si[g][1]);
                } else {
                    // A Z (kz = +az) and A conj(Z) (kz = -az) share their products
                    const R t1 = pr * z.x, t2 = pi * z.x;
                    const R erp = t1 - pi * z.y, eip = t2 + pr * z.y;
                    const R erm = t1 + pi * z.y, eim = t2 - pr * z.y;
                    sr[g][0] += erp;
                    si[g][0] += eip;
                    sr[g][1] += erm;
                    si[g][1] += eim;
                    const R kup = kxyu + kzr[g] * uz, kum = kxyu - kzr[g] * uz;
                    dsr[g][0] -= kup * eip;
                    dsi[g][0] += kup * erp;
                    dsr[g][1] -= kum * eim;
                    dsi[g][1] += kum * erm;
                }
            }
        };
        if (nc == CH) {  // a full chunk: a fixed trip count, unrolled
#pragma unroll 4
            for (int c = 0; c < CH; ++c) site(c);
        } else {
            for (int c = 0; c < nc; ++c) site(c);
        }
#pragma unroll
        for (int g = 0; g < KZ; ++g)
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                kahan_add(Sr[g][h], Cr[g][h], sr[g][h]);
                kahan_add(Si[g][h], Ci[g][h], si[g][h]);
                if (MODE == 1) {
                    kahan_add(dSr[g][h], dCr[g][h], dsr[g][h]);
                    kahan_add(dSi[g][h], dCi[g][h], dsi[g][h]);
                }
            }
    }
    if (act) {
#pragma unroll
        for (int g = 0; g < KZ; ++g) {
            if (g < G.n) {
                const int az = G.kz0 + g;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    if (h == 1 && az == 0) continue;  // kz = 0 has one entry
                    const int kz = h ? -az : az;
                    const size_t at = (size_t)sc * a.total_k + J.sk_off + C.k_begin + (kz + C.m);
                    if constexpr (G3) {
                        // FP32 form: the compensated pair (S, C) of S(kz) itself, from the
                        // (sum, compensation) pairs of T1, T2, U and V
                        const float t1 = (float)Sr[g][0], t2 = (float)Sr[g][1], u1 = (float)Cr[g][0], u2 = (float)Cr[g][1];
                        const float us = (float)Si[g][0], vs = (float)Si[g][1], uc = (float)Ci[g][0], vc = (float)Ci[g][1];
                        float4 o;
                        if (h == 0) {
                            o = make_float4(t1 - t2, ((us + vs) - t1) - t2, u1 - u2, ((uc + vc) - u1) - u2);
                        } else {
                            o = make_float4(t1 + t2, ((us - vs) - t1) + t2, u1 + u2, ((uc - vc) - u1) + u2);
                        }
                        reinterpret_cast<float4 *>(a.skp)[at] = o;
                    } else
                        a.skp[at] = make_double2((double)Sr[g][h] - (double)Cr[g][h], (double)Si[g][h] - (double)Ci[g][h]);
                    if (MODE == 1)
                        a.dskp[at] = make_double2((double)dSr[g][h] - (double)dCr[g][h],
                                                  (double)dSi[g][h] - (double)dCi[g][h]);
                }
            }
        }
    }
}

// Sum of the structure-factor partials of every k (FP64, fixed order), the
// reciprocal-space energy sum_k c_k |S(k)|^2, and the force weights 2 c_k S(k)
// (and 2 c_k dS(k)) in the working precision for k_kforce. One thread per k.
template <typename R, int MODE>
__global__ void __launch_bounds__(128) k_sk_reduce(EvalArgs a) {
    pdl_launch_dependents();  // the k-force may start its staging of the phase rows
    pdl_wait();               // the structure-factor partials of k_ksk
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    // FP32 energy/force form: the half set, each kx = 0, ky > 0 vector standing for
    // itself and its conjugate partner (|S|^2 and the force are the same for both),
    // one block per force batch (whole columns, <= 128 vectors), so that the block
    // also packs the batch's +-kz weights for k_kforce_f32
    const bool half = sizeof(R) == 4 && MODE == 0;
    int k, nk, kb0 = 0;
    if (half) {
        if ((int)blockIdx.x >= S.n_batch_half) return;
        const KBatch B = a.kbatch[S.batch_off + blockIdx.x];
        kb0 = B.k0;
        k = B.k0 + threadIdx.x;
        nk = B.k1;
    } else {
        nk = S.n_kvec;
        if (blockIdx.x * 128 >= nk) return;
        k = blockIdx.x * 128 + threadIdx.x;
    }
    __shared__ double red[4];
    __shared__ float2 wl[128];
    __shared__ float redf[4];
    double e = 0.0;
    float ef = 0.f;  // FP32 form: the k's energy term, summed over the block in FP32
    if (k < nk) {
        const KVec kv = a.kvec[S.kvec_off + k];
        const double w = 2.0 * kv.coef * ((half && kv.twin) ? 2.0 : 1.0);
        double sr = 0.0, si = 0.0, dr = 0.0, di = 0.0;
        if (sizeof(R) == 4 && MODE == 0) {
            // FP32 form: the site chunks' compensated pairs (S, C), summed in chunk
            // order with compensation in FP32; FP64 only for the energy
            const float4 *pk = reinterpret_cast<const float4 *>(a.skp) + J.sk_off + k;
            float xs = 0.f, xc = 0.f, ys = 0.f, yc = 0.f;
            int sc = 0;
            for (; sc + 4 <= a.n_sc; sc += 4) {  // four chunks' loads in flight, then their sums in order
                float4 p[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) p[u] = pk[(size_t)(sc + u) * a.total_k];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    kahan_add(xs, xc, p[u].x - p[u].z);
                    kahan_add(ys, yc, p[u].y - p[u].w);
                }
            }
            for (; sc < a.n_sc; ++sc) {
                const float4 p = pk[(size_t)sc * a.total_k];
                kahan_add(xs, xc, p.x - p.z);
                kahan_add(ys, yc, p.y - p.w);
            }
            const float fr = xs - xc, fi = ys - yc, wf = (float)w;
            ef = 0.5f * wf * fmaf(fr, fr, fi * fi);
            V2<R> v;
            v.x = (R)(wf * fr);
            v.y = (R)(wf * fi);
            reinterpret_cast<V2<R> *>(a.wsk)[J.sk_off + k] = v;
            wl[threadIdx.x] = make_float2(wf * fr, wf * fi);
        } else {
        for (int sc = 0; sc < a.n_sc; ++sc) {
            const size_t at = (size_t)sc * a.total_k + J.sk_off + k;
            const double2 p = a.skp[at];
            sr += p.x;
            si += p.y;
            if (MODE == 1) {
                const double2 d = a.dskp[at];
                dr += d.x;
                di += d.y;
            }
        }
        e = 0.5 * w * (sr * sr + si * si);
        V2<R> *ws = reinterpret_cast<V2<R> *>(a.wsk) + J.sk_off;
        V2<R> v;
        v.x = (R)(w * sr);
        v.y = (R)(w * si);
        ws[k] = v;
        if (MODE == 1) {
            V2<R> *wd = reinterpret_cast<V2<R> *>(a.wdsk) + J.sk_off;
            v.x = (R)(w * dr);
            v.y = (R)(w * di);
            wd[k] = v;
        }
        }
    }
    if (half && a.wpk && a.kpk) {
        // the batch's packed weights: slot of |kz| = az of a column holds, with
        // s = W(+az) + W(-az) and d = W(+az) - W(-az), P1 = (s.x, d.y, d.x, s.y) and
        // P2 = az (d.x, s.y, s.x, d.y) (az = 0: P1 = (W, 0, 0))
        __syncthreads();
        const int code = k < nk ? a.kpk[S.kvec_off + k] : -1;
        if (code >= 0) {
            const int slot = code >> 8, az = code & 255;
            const float2 wp = wl[threadIdx.x];
            float4 *o = a.wpk + 2 * ((size_t)J.sk_off + kb0 + slot);
            if (az == 0) {
                o[0] = make_float4(wp.x, wp.y, 0.f, 0.f);
            } else {
                const float2 wm = wl[threadIdx.x - 2 * az];
                const float sx = wp.x + wm.x, sy = wp.y + wm.y, dx = wp.x - wm.x, dy = wp.y - wm.y;
                const float fa = (float)az;
                o[0] = make_float4(sx, dy, dx, sy);
                o[1] = make_float4(fa * dx, fa * sy, fa * sx, fa * dy);
            }
        }
    }
    if (half) {  // the block's FP32 partial, added to the FP64 energy
        float t = warp_sum(ef);
        const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
        if (lane == 0) redf[w] = t;
        __syncthreads();
        if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], (double)(((redf[0] + redf[1]) + redf[2]) + redf[3]));
    } else if (MODE == 0) {
        const double t = block_sum(e, red);
        if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
    }
}

// k_sk_reduce's grid: FP32 energy/force form one block per force batch, else per 128 k
template <typename R, int MODE>
void launch_sk_reduce(const EvalArgs &a, cudaStream_t s) {
    const bool half = sizeof(R) == 4 && MODE == 0;
    const dim3 g(half ? a.max_batch : (a.max_kvec + 127) / 128, a.n_jobs);
    launch_pdl(k_sk_reduce<R, MODE>, g, dim3(128), 0, s, a);
}

// ---- k_kforce: reciprocal-space site forces -------------------------------------
// One thread per site; the block walks batches of whole k columns. Per batch
// the vectors' 2 c_k S(k) (and 2 c_k dS(k)) are summed over the structure-factor
// partials and staged in shared memory; per column a site forms X(kx) Y(ky)
// once, then for each kz the value v = Im(conj(2 c_k S) e_i), accumulating
// sum_kz v and sum_kz kz v: since kx and ky are constant along a column,
// F_x = b_x kx sum v, F_y = b_y ky sum v, F_z = b_z sum kz v.
constexpr int FT = 128;  // threads (sites) per block
constexpr int KB = 128;  // k-vectors per batch (at most)

template <typename R, int MODE>
__global__ void __launch_bounds__(FT) k_kforce(EvalArgs a) {
    const int kc = blockIdx.y, jb = blockIdx.z;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    // FP32 energy/force form: the half set, whose weights k_sk_reduce<float, 0> writes
    const int nb = (sizeof(R) == 4 && MODE == 0) ? S.n_batch_half : S.n_batch, ns = S.n_sites, km1 = S.k_max + 1;
    if (blockIdx.x * FT >= ns) return;
    const int i = blockIdx.x * FT + threadIdx.x;
    const bool act = i < ns;
    const int bt0 = chunk_lo(nb, kc, a.n_kc), bt1 = chunk_lo(nb, kc + 1, a.n_kc);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // 16-byte elements first so every array stays aligned for vector access
    KCol *cs = reinterpret_cast<KCol *>(smem_raw);  // [KB]
    V2<R> *ss = reinterpret_cast<V2<R> *>(cs + KB);  // [KB] 2 c_k S(k)
    V2<R> *ds = ss + KB;                             // [KB] 2 c_k dS(k)
    V2<R> *zr = ds + KB;                             // [km1][FT] my Z(kz) row
    const V2<R> *ph = reinterpret_cast<const V2<R> *>(a.phase) + J.phase_off;
    for (int m = 0; m < km1; ++m) {
        V2<R> v;
        v.x = v.y = (R)0;
        if (act) v = ph[(size_t)(2 * km1 + m) * ns + i];
        zr[m * FT + threadIdx.x] = v;
    }
    V4<R> ui;
    ui.x = ui.y = ui.z = ui.w = (R)0;
    if (MODE == 1 && act) ui = reinterpret_cast<const V4<R> *>(a.tan_sites)[J.site_off + i];
    const R bx = (R)(2.0 * PI_REF * S.inv_box[0]), by = (R)(2.0 * PI_REF * S.inv_box[1]),
            bz = (R)(2.0 * PI_REF * S.inv_box[2]);
    // per-batch sums added into Kahan-compensated running sums in the working precision
    R Fx = 0, Fy = 0, Fz = 0, Cx = 0, Cy = 0, Cz = 0;
    const int ii = act ? i : 0;
    const V2<R> *wsk = reinterpret_cast<const V2<R> *>(a.wsk) + J.sk_off;
    const V2<R> *wdsk = reinterpret_cast<const V2<R> *>(a.wdsk) + J.sk_off;
    for (int bt = bt0; bt < bt1; ++bt) {
        const KBatch B = a.kbatch[S.batch_off + bt];
        __syncthreads();
        for (int idx = threadIdx.x; idx < B.c1 - B.c0; idx += FT) cs[idx] = a.kcol[S.col_off + B.c0 + idx];
        for (int idx = threadIdx.x; idx < B.k1 - B.k0; idx += FT) {
            ss[idx] = wsk[B.k0 + idx];
            if (MODE == 1) ds[idx] = wdsk[B.k0 + idx];
        }
        __syncthreads();
        R fx = 0, fy = 0, fz = 0;
        for (int cc = 0; cc < B.c1 - B.c0; ++cc) {
            const KCol C = cs[cc];
            const V2<R> x = ph[(size_t)C.kx * ns + ii];
            const V2<R> y = ph[(size_t)(km1 + abs(C.ky)) * ns + ii];
            const R yi = C.ky < 0 ? -y.y : y.y;
            const R pr = x.x * y.x - x.y * yi, pi = x.x * yi + x.y * y.x;
            R kxyu = (R)0;
            if (MODE == 1) kxyu = bx * (R)C.kx * ui.x + by * (R)C.ky * ui.y;
            const int kb = C.k_begin - B.k0 + C.m;  // smem index of kz = 0
            R v = 0, vz = 0;
            {   // kz = 0: Z = 1
                const V2<R> sk = ss[kb];
                R val = sk.x * pi - sk.y * pr;
                if (MODE == 1) {
                    const V2<R> d = ds[kb];
                    val = (d.x * pi - d.y * pr) + kxyu * (sk.x * pr + sk.y * pi);
                }
                v += val;
            }
            // kz = +az and -az share the products of A Z and A conj(Z)
            for (int az = 1; az <= C.m; ++az) {
                const V2<R> z = zr[az * FT + threadIdx.x];
                const R t1 = pr * z.x, t2 = pi * z.x;
                const R erp = t1 - pi * z.y, eip = t2 + pr * z.y;
                const R erm = t1 + pi * z.y, eim = t2 - pr * z.y;
                const V2<R> sp = ss[kb + az], sm = ss[kb - az];
                R vp = sp.x * eip - sp.y * erp, vm = sm.x * eim - sm.y * erm;
                if (MODE == 1) {
                    const V2<R> dp = ds[kb + az], dm = ds[kb - az];
                    const R kup = kxyu + bz * (R)az * ui.z, kum = kxyu - bz * (R)az * ui.z;
                    vp = (dp.x * eip - dp.y * erp) + kup * (sp.x * erp + sp.y * eip);
                    vm = (dm.x * eim - dm.y * erm) + kum * (sm.x * erm + sm.y * eim);
                }
                v += vp + vm;
                vz += (R)az * (vp - vm);
            }
            fx += bx * (R)C.kx * v;
            fy += by * (R)C.ky * v;
            fz += bz * vz;
        }
        kahan_add(Fx, Cx, fx);
        kahan_add(Fy, Cy, fy);
        kahan_add(Fz, Cz, fz);
    }
    if (act) store_plane<R>(a.part, 3 * ((size_t)(a.n_rj + kc) * a.total_sites + J.site_off + i), Fx - Cx, Fy - Cy, Fz - Cz);
}

// FP32 form of k_kforce<float, 0> with the kz sums rearranged. Per site and
// column, with A = X(kx) Y(ky) = pr + i pi, Z = Z(|kz|) = zx + i zy and the
// column's weights W(+kz), W(-kz) (W = 2 c_k S(k)), the value summed above is
//   vp + vm = pr [zy dx - zx sy] + pi [zx sx + zy dy],
//   vp - vm = pr [zy sx - zx dy] + pi [zx dx + zy sy],
// with sx, sy = W(+kz) + W(-kz) and dx, dy = W(+kz) - W(-kz) (x, y: real and
// imaginary parts). So four per-site sums over |kz| -- U1 = sum (zx sx + zy dy),
// U2 = sum (zy dx - zx sy), U3 = sum kz (zx dx + zy sy), U4 = sum kz (zy sx - zx dy)
// -- take eight FMAs per +-kz pair, and A enters once per column:
// sum v = pi (U1 + W0x) + pr (U2 - W0y), sum kz v = pi U3 + pr U4 (W0: kz = 0).
// The batch's weights are staged as (sx, dy, dx, sy) and kz (dx, sy, sx, dy);
// a site's Z(1 .. ZM) stays in registers, its X and Y rows in shared memory.
template <int ZM, int SPT>  // SPT: sites per thread (the block's weights serve SPT x FT sites)
__global__ void __launch_bounds__(FT) k_kforce_f32(EvalArgs a) {
    constexpr int NS = SPT * FT;  // sites per block
    const int kc = blockIdx.y, jb = blockIdx.z;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    // the half set, whose weights k_sk_reduce<float, 0> writes
    const int nb = S.n_batch_half, ns = S.n_sites, km1 = S.k_max + 1;
    if (blockIdx.x * NS >= ns) return;
    const int bt0 = chunk_lo(nb, kc, a.n_kc), bt1 = chunk_lo(nb, kc + 1, a.n_kc);
    __shared__ float4 P1[KB], P2[KB];
    __shared__ int4 cs[KB];      // kx, ky, m, packed slot of kz = 0
    __shared__ float2 cb[KB];    // b_x kx, b_y ky
    extern __shared__ float2 xyrow[];  // [2 km1][NS]: this block's sites' X(0 .. k_max), Y(0 .. k_max)
    const float2 *ph = reinterpret_cast<const float2 *>(a.phase) + J.phase_off;
    int site[SPT];
    float2 z[SPT][ZM];
#pragma unroll
    for (int u = 0; u < SPT; ++u) {
        site[u] = blockIdx.x * NS + u * FT + threadIdx.x;
        const int ii = site[u] < ns ? site[u] : 0;
        for (int r = 0; r < 2 * km1; ++r) xyrow[r * NS + u * FT + threadIdx.x] = ph[(size_t)r * ns + ii];
#pragma unroll
        for (int az = 1; az <= ZM; ++az) {
            z[u][az - 1] = make_float2(0.f, 0.f);
            if (site[u] < ns && az < km1) z[u][az - 1] = ph[(size_t)(2 * km1 + az) * ns + site[u]];
        }
    }
    const float bz = S.kbf[2];
    // the phase rows above come from the force evaluation's prep, complete before
    // the structure factors started; the weights below from k_sk_reduce
    pdl_wait();
    float Fx[SPT], Fy[SPT], Fz[SPT], Cx[SPT], Cy[SPT], Cz[SPT];
#pragma unroll
    for (int u = 0; u < SPT; ++u) Fx[u] = Fy[u] = Fz[u] = Cx[u] = Cy[u] = Cz[u] = 0.f;
    // the batch's columns (static) and +-kz weights (packed by k_sk_reduce), copied as they are
    const float4 *wpk = a.wpk + 2 * (size_t)J.sk_off;
    for (int bt = bt0; bt < bt1; ++bt) {
        const KBatch B = a.kbatch[S.batch_off + bt];
        const int ncol = B.c1 - B.c0;
        __syncthreads();
        for (int idx = threadIdx.x; idx < ncol; idx += FT) {
            cs[idx] = a.kfc[S.col_off + B.c0 + idx];
            cb[idx] = a.kfb[S.col_off + B.c0 + idx];
        }
        for (int idx = threadIdx.x; idx < B.k1 - B.k0; idx += FT) {
            P1[idx] = wpk[2 * (B.k0 + idx)];
            P2[idx] = wpk[2 * (B.k0 + idx) + 1];
        }
        __syncthreads();
        float fx[SPT], fy[SPT], fz[SPT];
#pragma unroll
        for (int u = 0; u < SPT; ++u) fx[u] = fy[u] = fz[u] = 0.f;
        for (int cc = 0; cc < ncol; ++cc) {
            const int4 C = cs[cc];
            const float4 w0 = P1[C.w];
            float pr[SPT], pi[SPT], u1[SPT], u2[SPT], u3[SPT], u4[SPT];
#pragma unroll
            for (int u = 0; u < SPT; ++u) {
                const float2 x = xyrow[C.x * NS + u * FT + threadIdx.x];
                const float2 y = xyrow[(km1 + abs(C.y)) * NS + u * FT + threadIdx.x];
                const float yi = C.y < 0 ? -y.y : y.y;
                pr[u] = x.x * y.x - x.y * yi;
                pi[u] = x.x * yi + x.y * y.x;
                u1[u] = w0.x;
                u2[u] = -w0.y;
                u3[u] = 0.f;
                u4[u] = 0.f;
            }
#pragma unroll
            for (int az = 1; az <= ZM; ++az) {
                if (az > C.z) break;
                const float4 p1 = P1[C.w + az], p2 = P2[C.w + az];
#pragma unroll
                for (int u = 0; u < SPT; ++u) {
                    const float zx = z[u][az - 1].x, zy = z[u][az - 1].y;
                    u1[u] = fmaf(zx, p1.x, fmaf(zy, p1.y, u1[u]));
                    u2[u] = fmaf(zy, p1.z, fmaf(-zx, p1.w, u2[u]));
                    u3[u] = fmaf(zx, p2.x, fmaf(zy, p2.y, u3[u]));
                    u4[u] = fmaf(zy, p2.z, fmaf(-zx, p2.w, u4[u]));
                }
            }
            const float2 b = cb[cc];
#pragma unroll
            for (int u = 0; u < SPT; ++u) {
                const float v = fmaf(pi[u], u1[u], pr[u] * u2[u]), vz = fmaf(pi[u], u3[u], pr[u] * u4[u]);
                fx[u] = fmaf(b.x, v, fx[u]);
                fy[u] = fmaf(b.y, v, fy[u]);
                fz[u] = fmaf(bz, vz, fz[u]);
            }
        }
#pragma unroll
        for (int u = 0; u < SPT; ++u) {
            kahan_add(Fx[u], Cx[u], fx[u]);
            kahan_add(Fy[u], Cy[u], fy[u]);
            kahan_add(Fz[u], Cz[u], fz[u]);
        }
    }
#pragma unroll
    for (int u = 0; u < SPT; ++u)
        if (site[u] < ns)
            store_plane<float>(a.part, 3 * ((size_t)(a.n_rj + kc) * a.total_sites + J.site_off + site[u]),
                               Fx[u] - Cx[u], Fy[u] - Cy[u], Fz[u] - Cz[u]);
}

template <typename R>
size_t kforce_smem(int kmax);
template <typename R>
size_t ksk_smem(int kmax);

// k_ksk for the context's structure-factor group width
template <typename R, int MODE>
void launch_ksk(const EvalArgs &a, dim3 grid, cudaStream_t s) {
    if (a.kz == 3) k_ksk<R, MODE, 3><<<grid, KT, ksk_smem<R>(a.max_kmax), s>>>(a);
    else k_ksk<R, MODE, 4><<<grid, KT, ksk_smem<R>(a.max_kmax), s>>>(a);
}

// the FP32 k-force kernel for the largest |kz| of the batch (the general form beyond 32)
void launch_kforce_f32(const EvalArgs &a, dim3 grid, cudaStream_t s) {
    // two sites a thread (the block covers 2 FT sites: grid.x halves)
    const size_t sm = (size_t)2 * (a.max_kmax + 1) * 2 * FT * sizeof(float2);
    dim3 g2 = grid;
    g2.x = (grid.x + 1) / 2;
    if (a.kpk && a.max_kmax <= 8) launch_pdl(k_kforce_f32<8, 2>, g2, dim3(FT), sm, s, a);
    else if (a.kpk && a.max_kmax <= 12) launch_pdl(k_kforce_f32<12, 2>, g2, dim3(FT), sm, s, a);
    else if (a.kpk && a.max_kmax <= 16) launch_pdl(k_kforce_f32<16, 2>, g2, dim3(FT), sm, s, a);
    else if (a.kpk && a.max_kmax <= 24) launch_pdl(k_kforce_f32<24, 2>, g2, dim3(FT), sm, s, a);
    else if (a.kpk && a.max_kmax <= 32) launch_pdl(k_kforce_f32<32, 2>, g2, dim3(FT), sm, s, a);
    else k_kforce<float, 0><<<grid, FT, kforce_smem<float>(a.max_kmax), s>>>(a);
}

// ---- k_combine: partial sums, short-range terms and the M-site chain rule ---------

// Minimum image of an intramolecular vector. |r / L| is far below 1/2, where
// round(r * (1/L)) and the reference's round(r / L) agree (both 0, or the same
// integer for a molecule split by wrapping), so no FP64 division is needed.
__device__ __forceinline__ void min_image3(double *r, const SysDev &S) {
    for (int d = 0; d < 3; ++d) r[d] -= S.box[d] * round(r[d] * S.inv_box[d]);
}

// same-molecule real-space pair with erfc - 1 (forces.cpp:141-177); the
// difference vector is formed in FP64, the pair term in R
template <typename R>
__device__ __forceinline__ double ewald_same_mol(const double *ri, const double *rj, double qiqj, const SysDev &S,
                                                 double *fi, double *fj) {
    double rd[3];
    for (int d = 0; d < 3; ++d) rd[d] = ri[d] - rj[d];
    min_image3(rd, S);
    const double r2d = rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2];
    if (!(r2d < S.rc_sq)) return 0.0;
    const R r2 = (R)r2d, rl = f_sqrt(r2), inv = (R)1 / rl, kap = (R)S.kappa;
    const R ec = f_erfc(kap * rl) - (R)1;
    const R e = (R)qiqj * inv * ec;
    const R ff = (e + (R)qiqj * (R)S.ewald_pref * f_exp(-(kap * kap) * r2)) * inv * inv;
    for (int d = 0; d < 3; ++d) {
        fi[d] += (double)(ff * (R)rd[d]);
        fj[d] -= (double)(ff * (R)rd[d]);
    }
    return (double)e;
}

template <typename R>
__global__ void __launch_bounds__(128) k_combine(EvalArgs a) {
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int N = S.n_mols;
    if (blockIdx.x * blockDim.x >= N) return;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    __shared__ double red[4];
    double e = 0.0;
    if (m < N) {
        const double *q = a.pos + J.pos_off + 9 * m;
        double *f = a.out + J.out_off + 9 * m;
        double fs[9];
        for (int k = 0; k < 9; ++k) fs[k] = 0.0;
        if (!a.sr_only) {
            const int np = a.n_rj + a.n_kc;
            for (int p = 0; p < np; ++p) {
                const double *sf = a.part + 3 * ((size_t)p * a.total_sites + J.site_off + 3 * m);
                for (int k = 0; k < 9; ++k) fs[k] += sf[k];
            }
        }
        double fa[9];
        for (int k = 0; k < 9; ++k) fa[k] = 0.0;
        if (J.mode == 0) {
            const Consts &C = a.c;
            const double g = C.gamma_vs;
            const double *chg = a.charge + S.chg_off + 3 * m;
            double site[9];
            for (int d = 0; d < 3; ++d) {
                site[d] = g * q[d] + 0.5 * (1.0 - g) * (q[3 + d] + q[6 + d]);
                site[3 + d] = q[3 + d];
                site[6 + d] = q[6 + d];
            }
            e += ewald_same_mol<R>(site, site + 3, chg[0] * chg[1], S, fs, fs + 3);
            e += ewald_same_mol<R>(site, site + 6, chg[0] * chg[2], S, fs, fs + 6);
            e += ewald_same_mol<R>(site + 3, site + 6, chg[1] * chg[2], S, fs + 3, fs + 6);
            // quartic Morse bonds (forces.cpp:65-93, :519-551); FP64 bond vectors
            double rad[3], rbd[3];
            for (int d = 0; d < 3; ++d) {
                rad[d] = q[d] - q[3 + d];
                rbd[d] = q[d] - q[6 + d];
            }
            min_image3(rad, S);
            min_image3(rbd, S);
            R ra[3], rb[3];
            for (int d = 0; d < 3; ++d) {
                ra[d] = (R)rad[d];
                rb[d] = (R)rbd[d];
            }
            const double lad = sqrt(rad[0] * rad[0] + rad[1] * rad[1] + rad[2] * rad[2]);
            const double lbd = sqrt(rbd[0] * rbd[0] + rbd[1] * rbd[1] + rbd[2] * rbd[2]);
            const R la = (R)lad, lb = (R)lbd;
            const R ar2 = (R)C.ar2, ar3 = (R)C.ar3, ar4 = (R)C.ar4fac, Dr = (R)C.Dr;
            for (int bnd = 0; bnd < 2; ++bnd) {
                const R *r = bnd ? rb : ra;
                const R rl = bnd ? lb : la;
                const R x = (R)((bnd ? lbd : lad) - C.roheq), x2 = x * x, x3 = x2 * x, x4 = x2 * x2;
                e += (double)(Dr * (ar2 * x2 - ar3 * x3 + ar4 * x4));
                const R gg = ((R)2 * ar2 * x - (R)3 * ar3 * x2 + (R)4 * ar4 * x3) * Dr / rl;
                for (int d = 0; d < 3; ++d) {
                    fa[d] -= (double)(gg * r[d]);
                    fa[3 + 3 * bnd + d] += (double)(gg * r[d]);
                }
            }
            // harmonic HOH angle (forces.cpp:96-138)
            {
                const R dot = ra[0] * rb[0] + ra[1] * rb[1] + ra[2] * rb[2];
                const R ia = (R)1 / la, ib = (R)1 / lb, iab = ia * ib;
                const R c = dot * iab;
                const R dacos = (R)1 / f_sqrt((R)1 - c * c);
                const R ca = dot * ia * ia * iab, cb = dot * ib * ib * iab;
                const R dth = f_acos(c) - (R)C.theta_eq;
                e += 0.5 * C.ktheta * (double)dth * (double)dth;
                const R gp = (R)C.ktheta * dth * dacos;
                for (int d = 0; d < 3; ++d) {
                    fa[d] += (double)(gp * (iab * (ra[d] + rb[d]) - ca * ra[d] - cb * rb[d]));
                    fa[3 + d] -= (double)(gp * (iab * rb[d] - ca * ra[d]));
                    fa[6 + d] -= (double)(gp * (iab * ra[d] - cb * rb[d]));
                }
            }
        }
        // M-site chain rule (forces.cpp:613-619)
        const double g = a.c.gamma_vs, h = 0.5 * (1.0 - g);
        for (int d = 0; d < 3; ++d) {
            f[d] = fa[d] + g * fs[d];
            f[3 + d] = fa[3 + d] + fs[3 + d] + h * fs[d];
            f[6 + d] = fa[6 + d] + fs[6 + d] + h * fs[d];
        }
    }
    if (J.mode == 0) {
        if (m == 0 && !a.sr_only) e -= S.self_energy;
        const double t = block_sum(e, red);
        if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
    }
}

// Mixed form of k_combine: the FP32 planes are added with Kahan compensation;
// the atom differences are formed in FP64 and rounded to FP32 (intramolecular
// vectors are ~1-3 bohr, so FP32 keeps them to ~1e-7 relative); the bond
// lengths, whose offsets from r_eq set the stiff Morse force, are taken to FP64
// accuracy as l = l0 + (s - l0^2) / (2 l0), with s = |r|^2 in FP64 and l0 its
// FP32 square root; everything else (same-molecule Ewald, Morse, angle, chain
// rule) is FP32, and the energy is accumulated in FP64.
__device__ __forceinline__ void min_image3f(float *r, const SysDev &S) {
    for (int d = 0; d < 3; ++d) r[d] = fmaf(-S.boxf[d], rintf(r[d] * S.inv_boxf[d]), r[d]);
}

// same-molecule real-space pair with erfc - 1 (forces.cpp:141-177), FP32
__device__ __forceinline__ float ewald_same_mol_f32(const float *rd, float qiqj, const SysDev &S, float *fi, float *fj) {
    const float r2 = rd[0] * rd[0] + rd[1] * rd[1] + rd[2] * rd[2];
    if (!(r2 < (float)S.rc_sq)) return 0.f;
    const float rl = sqrtf(r2), inv = 1.0f / rl, kap = (float)S.kappa;
    const float e = qiqj * inv * (erfcf(kap * rl) - 1.0f);
    const float ff = (e + qiqj * (float)S.ewald_pref * expf(-(kap * kap) * r2)) * inv * inv;
    for (int d = 0; d < 3; ++d) {
        fi[d] += ff * rd[d];
        fj[d] -= ff * rd[d];
    }
    return e;
}

// Intramolecular terms of molecule m of job J (mixed): the same-molecule Ewald
// pairs (erfc - 1) as site-force increments fs[9] (M, H1, H2), the quartic Morse
// bonds and the HOH angle as atom forces fa[9] (O, H1, H2); returns their energy.
__device__ double intra_f32(const EvalArgs &a, const Job &J, const SysDev &S, int m, float *fs, float *fa) {
    const double *q = a.pos + J.pos_off + 9 * m;
    const Consts &C = a.c;
    const double g = C.gamma_vs, h = 0.5 * (1.0 - g);
    const double *cq = a.charge + S.chg_off + 3 * m;
    double e = 0.0;
    // charge sites M, H1, H2 (forces.cpp:558-564) and their differences
    double site[9];
    for (int d = 0; d < 3; ++d) {
        site[d] = g * q[d] + h * (q[3 + d] + q[6 + d]);
        site[3 + d] = q[3 + d];
        site[6 + d] = q[6 + d];
    }
    float dm1[3], dm2[3], d12[3];
    for (int d = 0; d < 3; ++d) {
        dm1[d] = (float)(site[d] - site[3 + d]);
        dm2[d] = (float)(site[d] - site[6 + d]);
        d12[d] = (float)(site[3 + d] - site[6 + d]);
    }
    min_image3f(dm1, S);
    min_image3f(dm2, S);
    min_image3f(d12, S);
    float ef = ewald_same_mol_f32(dm1, (float)(cq[0] * cq[1]), S, fs, fs + 3);
    ef += ewald_same_mol_f32(dm2, (float)(cq[0] * cq[2]), S, fs, fs + 6);
    ef += ewald_same_mol_f32(d12, (float)(cq[1] * cq[2]), S, fs + 3, fs + 6);
    e += (double)ef;
    // quartic Morse bonds (forces.cpp:65-93, :519-551)
    double rad[3], rbd[3];
    for (int d = 0; d < 3; ++d) {
        rad[d] = q[d] - q[3 + d];
        rbd[d] = q[d] - q[6 + d];
    }
    min_image3(rad, S);
    min_image3(rbd, S);
    float ra[3], rb[3], xs[2], ls[2];
    for (int d = 0; d < 3; ++d) {
        ra[d] = (float)rad[d];
        rb[d] = (float)rbd[d];
    }
    for (int bnd = 0; bnd < 2; ++bnd) {
        const double *r = bnd ? rbd : rad;
        const double s2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
        const float l0 = sqrtf((float)s2);
        const float corr = (float)(s2 - (double)l0 * (double)l0) * (0.5f / l0);
        xs[bnd] = (float)((double)l0 - C.roheq) + corr;
        ls[bnd] = l0 + corr;
    }
    const float ar2 = (float)C.ar2, ar3 = (float)C.ar3, ar4 = (float)C.ar4fac, Dr = (float)C.Dr;
    float eb = 0.f;
    for (int bnd = 0; bnd < 2; ++bnd) {
        const float *r = bnd ? rb : ra;
        const float x = xs[bnd], x2 = x * x, x3 = x2 * x, x4 = x2 * x2;
        eb += Dr * (ar2 * x2 - ar3 * x3 + ar4 * x4);
        const float gg = (2.f * ar2 * x - 3.f * ar3 * x2 + 4.f * ar4 * x3) * Dr / ls[bnd];
        for (int d = 0; d < 3; ++d) {
            fa[d] -= gg * r[d];
            fa[3 + 3 * bnd + d] += gg * r[d];
        }
    }
    e += (double)eb;
    // harmonic HOH angle (forces.cpp:96-138)
    const float la = ls[0], lb = ls[1];
    const float dot = ra[0] * rb[0] + ra[1] * rb[1] + ra[2] * rb[2];
    const float ia = 1.f / la, ib = 1.f / lb, iab = ia * ib;
    const float c = dot * iab;
    const float dacos = 1.f / sqrtf(1.f - c * c);
    const float ca = dot * ia * ia * iab, cb = dot * ib * ib * iab;
    const float dth = acosf(c) - (float)C.theta_eq;
    e += 0.5 * C.ktheta * (double)dth * (double)dth;
    const float gp = (float)C.ktheta * dth * dacos;
    for (int d = 0; d < 3; ++d) {
        fa[d] += gp * (iab * (ra[d] + rb[d]) - ca * ra[d] - cb * rb[d]);
        fa[3 + d] -= gp * (iab * rb[d] - ca * ra[d]);
        fa[6 + d] -= gp * (iab * ra[d] - cb * rb[d]);
    }
    return e;
}

// The intramolecular terms of a forked mixed evaluation, on a branch beside the
// pair kernels (they need positions only): per molecule 18 floats (fs, fa) for
// k_combine_f32, the energy (with the Ewald self term) into the job's slot.
__global__ void __launch_bounds__(128) k_intra_f32(EvalArgs a) {
    const Job J = a.jobs[blockIdx.y];
    const SysDev &S = a.sys[J.sys];
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (blockIdx.x * blockDim.x >= S.n_mols) return;
    __shared__ double red[4];
    double e = 0.0;
    if (m < S.n_mols) {
        float fs[9], fa[9];
        for (int k = 0; k < 9; ++k) fs[k] = fa[k] = 0.f;
        e = intra_f32(a, J, S, m, fs, fa);
        if (m == 0) e -= S.self_energy;
        float *o = a.intra + 18 * ((size_t)J.site_off / 3 + m);
        for (int k = 0; k < 9; ++k) {
            o[k] = fs[k];
            o[9 + k] = fa[k];
        }
    }
    const double t = block_sum(e, red);
    if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
}

// CMB molecules per 128-thread block: first every thread sums site-force
// components over the partial planes (one component a thread, plane order,
// Kahan-compensated: the same sums as one thread per molecule would form, spread
// over the block), then one thread per molecule adds the intramolecular and
// Lennard-Jones terms and applies the M-site chain rule.
constexpr int CMB = 32;
__global__ void __launch_bounds__(128) k_combine_f32(EvalArgs a) {
    pdl_launch_dependents();  // the end step may load positions and masses meanwhile
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int N = S.n_mols;
    const int m0 = blockIdx.x * CMB;
    if (m0 >= N) return;
    const int nm = min(CMB, N - m0);
    const int m = m0 + threadIdx.x;
    __shared__ double red[4];
    __shared__ float fsum[CMB * 9];
    {
        const int np = a.n_rj + a.n_kc;
        const size_t stride = 3 * (size_t)a.total_sites;
        const float *pl = reinterpret_cast<const float *>(a.part) + 3 * ((size_t)J.site_off + 3 * m0);
        const long long *rf = a.real_fix ? a.rfix + 3 * ((size_t)J.site_off + 3 * m0) : nullptr;
        for (int o = threadIdx.x; o < 9 * nm; o += blockDim.x) {
            float sum = 0.f, comp = 0.f;
            // the half-interaction real space's fixed-point sums (2^-40 units), loaded
            // beside the planes
            const long long rv = rf ? rf[o] : 0ll;
            for (int p = 0; p < np; p += 16) {  // up to sixteen planes' loads in flight, then their sums in order
                float v[16];
#pragma unroll
                for (int u = 0; u < 16; ++u) v[u] = p + u < np ? pl[(p + u) * stride + o] : 0.f;
#pragma unroll
                for (int u = 0; u < 16; ++u)
                    if (p + u < np) kahan_add(sum, comp, v[u]);
            }
            if (rf) kahan_add(sum, comp, (float)((double)rv * 9.094947017729282e-13));
            fsum[o] = sum - comp;
        }
    }
    __syncthreads();
    double e = 0.0;
    if ((int)threadIdx.x < nm) {
        double *f = a.out + J.out_off + 9 * m;
        float fs[9];
        for (int k = 0; k < 9; ++k) fs[k] = fsum[9 * threadIdx.x + k];
        float fa[9];
        for (int k = 0; k < 9; ++k) fa[k] = 0.f;
        if (J.mode == 0 && a.intra_plane) {  // computed beside the pair kernels (k_intra_f32)
            const float *o = a.intra + 18 * ((size_t)J.site_off / 3 + m);
            for (int k = 0; k < 9; ++k) {
                fs[k] += o[k];
                fa[k] = o[9 + k];
            }
        } else if (J.mode == 0) {  // the same sums in the same order as k_intra_f32's
            float fi[9];
            for (int k = 0; k < 9; ++k) fi[k] = 0.f;
            e += intra_f32(a, J, S, m, fi, fa);
            if (m == 0) e -= S.self_energy;
            for (int k = 0; k < 9; ++k) fs[k] += fi[k];
        }
        // M-site chain rule (forces.cpp:613-619); the dense Lennard-Jones force of a
        // forked evaluation joins the oxygen here
        const float g = (float)a.c.gamma_vs, h = 0.5f * (1.0f - g);
        float lj[3] = {0.f, 0.f, 0.f};
        if (a.lj_plane && J.mode == 0) {
            const float4 l = a.ljf[J.site_off / 3 + m];
            lj[0] = l.x;
            lj[1] = l.y;
            lj[2] = l.z;
        }
        double *f2 = a.out_prop ? a.out_prop + J.out_off + 9 * m : nullptr;
        for (int d = 0; d < 3; ++d) {
            const double fo = (double)(fa[d] + g * fs[d]) + (double)lj[d];
            const double f1 = (double)(fa[3 + d] + fs[3 + d] + h * fs[d]);
            const double f2v = (double)(fa[6 + d] + fs[6 + d] + h * fs[d]);
            f[d] = fo;
            f[3 + d] = f1;
            f[6 + d] = f2v;
            if (f2) {
                f2[d] = fo;
                f2[3 + d] = f1;
                f2[6 + d] = f2v;
            }
        }
    }
    if (J.mode == 0 && !a.intra_plane) {
        const double t = block_sum(e, red);
        if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
    }
}

// ---- k_lj: O-O Lennard-Jones over the Verlet list (forces.cpp:489-515) -----------
// One warp per CSR row; lanes over the row's entries. The pair's displacement
// and the cutoff decision r^2 < r_cut^2 must be the reference's (FP64,
// x - L*round(x/L) with a true division and round-half-away-from-zero, each
// operation rounded): a pair whose working-precision r^2 lies within a
// relative band around r_cut^2, or whose separation is within rounding of
// half a box in some dimension (where the two images tie and the rounding rule
// picks the sign), is recomputed with exactly that arithmetic.
__device__ __forceinline__ double lj_exact_disp(const double *qi, const double *qj, const SysDev &S, double *r) {
    double r2 = 0.0;
    for (int d = 0; d < 3; ++d) {
        double x = __dsub_rn(qi[d], qj[d]);
        x = __dsub_rn(x, __dmul_rn(S.box[d], round(__ddiv_rn(x, S.box[d]))));
        r[d] = x;
        r2 = (d == 0) ? __dmul_rn(x, x) : __dadd_rn(r2, __dmul_rn(x, x));
    }
    return r2;
}

template <typename R, int FULL>
__global__ void __launch_bounds__(128) k_lj(EvalArgs a) {
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int N = S.n_mols;
    if (blockIdx.x * 4 >= N) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.x * 4 + w;
    __shared__ double red[4];
    double e = 0.0;
    const Consts &C = a.c;
    const double rc2 = C.r_cut_sq;
    const R rc2r = (R)rc2;
    const R bandr = sizeof(R) == 4 ? (R)1e-5 : (R)1e-12;
    const R tie = sizeof(R) == 4 ? (R)1e-5 : (R)1e-12;
    // half list: rows 0..N-2, entries j > i, forces on j by atomics; symmetric
    // list (FULL): rows 0..N-1, entries j != i, each pair seen from both ends, so
    // a row's force needs no atomics and the energy is halved
    if (i < (FULL ? N : N - 1)) {
        const double *q = a.pos + J.pos_off;
        double *f = a.out + J.out_off;
        const int cap = FULL ? 2 * S.list_size : S.list_size;
        const int *pt = FULL ? a.point_full + S.pf_off + (size_t)J.bead * (N + 1)
                             : a.point + S.pt_off + (size_t)J.bead * N;
        const int *ls = FULL ? a.list_full + S.lf_off + (size_t)J.bead * cap
                             : a.list + S.ls_off + (size_t)J.bead * S.list_size;
        // a row outside [0, capacity] (overflowed or caller-corrupted list) or an index
        // outside the row's range is skipped and flagged instead of being read out of bounds
        int n0 = pt[i], n1 = pt[i + 1];
        if (n0 < 0 || n1 > cap || n0 > n1) {
            if (lane == 0) atomicOr(a.status, (unsigned)ST_LIST_OVERFLOW);
            n0 = max(0, min(n0, cap));
            n1 = max(n0, min(n1, cap));
        }
        R xi[3];
        const V4<R> *opos = reinterpret_cast<const V4<R> *>(a.opos) + J.site_off / 3;
        if (sizeof(R) == 4) {
            const V4<R> o = opos[i];
            xi[0] = o.x;
            xi[1] = o.y;
            xi[2] = o.z;
        } else {
            for (int d = 0; d < 3; ++d) xi[d] = (R)q[9 * i + d];
        }
        const R s6c = (R)C.sigmalj6, s12c = (R)C.sigmalj12, eps4 = (R)(4.0 * C.epslj), eps24 = (R)(24.0 * C.epslj);
        R fi0 = 0, fi1 = 0, fi2 = 0, el = 0;
        for (int n = n0 + lane; n < n1; n += 32) {
            const int j = ls[n];
            if ((FULL ? j == i : j <= i) || j < 0 || j >= N) {
                atomicOr(a.status, (unsigned)ST_LIST_OVERFLOW);
                continue;
            }
            R r[3];
            if (sizeof(R) == 4) {
                const V4<R> o = opos[j];
                r[0] = xi[0] - o.x;
                r[1] = xi[1] - o.y;
                r[2] = xi[2] - o.z;
            } else {
                for (int d = 0; d < 3; ++d) r[d] = xi[d] - (R)q[9 * j + d];
            }
            bool exact = false;
            for (int d = 0; d < 3; ++d) {
                const R t = r[d] * sys_ibox<R>(S, d);
                const R fr = fabs(t - trunc(t));
                if (fabs(fr - (R)0.5) < tie) exact = true;
                r[d] -= sys_box<R>(S, d) * f_rint(t);
            }
            R r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            if (exact || fabs(r2 - rc2r) <= bandr * rc2r) {
                double rd[3];
                const double r2d = lj_exact_disp(q + 9 * i, q + 9 * j, S, rd);
                for (int d = 0; d < 3; ++d) r[d] = (R)rd[d];
                r2 = (R)r2d;
                exact = r2d < rc2;
            } else {
                exact = r2 < (R)rc2;
            }
            if (exact) {
                const R i2 = (R)1 / r2, i6 = i2 * i2 * i2;
                const R s6 = i6 * s6c, s12 = i6 * i6 * s12c;
                const R en = s12 - s6;
                el += en * eps4 - (R)C.e_cut;
                const R ff = (en + s12) * eps24 * i2;
                fi0 += ff * r[0];
                fi1 += ff * r[1];
                fi2 += ff * r[2];
                if (!FULL) {
                    atomicAdd(&f[9 * j], -(double)(ff * r[0]));
                    atomicAdd(&f[9 * j + 1], -(double)(ff * r[1]));
                    atomicAdd(&f[9 * j + 2], -(double)(ff * r[2]));
                }
            }
        }
        const double d0 = warp_sum((double)fi0), d1 = warp_sum((double)fi1), d2 = warp_sum((double)fi2);
        e = warp_sum((double)el) * (FULL ? 0.5 : 1.0);
        if (lane == 0) {
            if (FULL && a.lj_plane) {  // the mixed combine adds the oxygen force
                a.ljf[J.site_off / 3 + i] = make_float4((float)d0, (float)d1, (float)d2, 0.f);
            } else if (FULL) {
                f[9 * i] += d0;
                f[9 * i + 1] += d1;
                f[9 * i + 2] += d2;
            } else {
                atomicAdd(&f[9 * i], d0);
                atomicAdd(&f[9 * i + 1], d1);
                atomicAdd(&f[9 * i + 2], d2);
            }
        } else {
            e = 0.0;
        }
    }
    const double t = block_sum(e, red);
    if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
}

// ---- k_lj_dense: O-O Lennard-Jones of the device stepper, mixed precision -------
// The stepper rebuilds its Verlet list whenever the skin test (update.cpp:356-385)
// fires, before the forces are evaluated, so the list holds every pair that can
// be inside r_cut: the sum over all pairs with r^2 < r_cut^2 has the pair set of
// the list loop of forces.cpp:489-515. This kernel forms that sum without going
// through the list: the bead's wrapped oxygen positions are staged through
// shared memory, LJD_SUB lanes share a row and split its j's (each warp reads
// LJD_SUB consecutive positions per step: at most one shared-memory wavefront
// for eight lanes a row), and the
// row's sums are reduced over those lanes in FP32 with shuffles. Each pair is
// seen from both ends; the energy is halved.
//
// Pairs whose FP32 r^2 lies in a narrow band around r_cut^2, or that sit at a
// half-box tie where half a box is inside r_cut, must take the reference's FP64
// arithmetic (as in k_lj). They are rare, and that FP64 code is kept out of the
// main loop: the loop skips them and raises a block flag, and only blocks that
// saw one run a second pass that evaluates exactly those pairs.
constexpr int LJD_CH = 1024;                // oxygens per shared-memory chunk

struct LjdConst {
    float L[3], I[3], rc2, band, tie, s6, s12, eps4, eps24, ecut;
    int tie_mask;  // bit d: half of box side d is inside r_cut
};

// 0: outside r_cut; 1: inside, displacement in r; 2: needs the FP64 decision
__device__ __forceinline__ int ljd_classify(const float4 &oi, const float4 &o, const LjdConst &K, float *r,
                                            float *rr) {
    const float dx = oi.x - o.x, dy = oi.y - o.y, dz = oi.z - o.z;
    const float tx = dx * K.I[0], ty = dy * K.I[1], tz = dz * K.I[2];
    // wrapped positions lie in [0, L]: |t| <= 1, and two images tie at |t| = 1/2
    const bool tie = ((K.tie_mask & 1) && fabsf(fabsf(tx) - 0.5f) < K.tie) ||
                     ((K.tie_mask & 2) && fabsf(fabsf(ty) - 0.5f) < K.tie) ||
                     ((K.tie_mask & 4) && fabsf(fabsf(tz) - 0.5f) < K.tie);
    r[0] = fmaf(-K.L[0], rintf(tx), dx);
    r[1] = fmaf(-K.L[1], rintf(ty), dy);
    r[2] = fmaf(-K.L[2], rintf(tz), dz);
    *rr = fmaf(r[0], r[0], fmaf(r[1], r[1], r[2] * r[2]));
    if (tie || fabsf(*rr - K.rc2) <= K.band) return 2;
    return *rr < K.rc2 ? 1 : 0;
}

__device__ __forceinline__ void ljd_pair(const float *r, float rr, const LjdConst &K, float &fx, float &fy, float &fz,
                                         float &el) {
    const float i2 = rcp_approx(rr), i6 = i2 * i2 * i2;
    const float s6 = i6 * K.s6, s12 = i6 * i6 * K.s12;
    const float en = s12 - s6;
    el += en * K.eps4 - K.ecut;
    const float ff = (en + s12) * K.eps24 * i2;
    fx = fmaf(ff, r[0], fx);
    fy = fmaf(ff, r[1], fy);
    fz = fmaf(ff, r[2], fz);
}

template <int LJD_SUB>  // lanes per row: 8, or 32 when there are too few rows to fill the GPU
__global__ void __launch_bounds__(128) k_lj_dense(EvalArgs a) {
    constexpr int LJD_ROWS = 128 / LJD_SUB;  // rows per 128-thread block
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int N = S.n_mols;
    if (blockIdx.x * LJD_ROWS >= N) return;
    __shared__ float4 sj[LJD_CH];
    const int sub = threadIdx.x & (LJD_SUB - 1);
    const int i = blockIdx.x * LJD_ROWS + threadIdx.x / LJD_SUB;
    const bool act = i < N;
    const Consts &C = a.c;
    const double rc2 = C.r_cut_sq;
    LjdConst K;
    for (int d = 0; d < 3; ++d) {
        K.L[d] = S.boxf[d];
        K.I[d] = S.inv_boxf[d];
    }
    // FP32 constants and the tie mask come prepared from the host (no FP64 work per thread)
    K.rc2 = C.ljf[5];
    K.band = 1e-5f * K.rc2;
    K.tie = 1e-5f;
    K.s6 = C.ljf[0];
    K.s12 = C.ljf[1];
    K.eps4 = C.ljf[2];
    K.eps24 = C.ljf[3];
    K.ecut = C.ljf[4];
    K.tie_mask = S.lj_tie_mask;
    const float4 *opos = reinterpret_cast<const float4 *>(a.opos) + J.site_off / 3;
    float4 oi = make_float4(0.f, 0.f, 0.f, 0.f);
    if (act) oi = opos[i];
    float fx = 0.f, fy = 0.f, fz = 0.f, el = 0.f;
    int flagged = 0;
    for (int t0 = 0; t0 < N; t0 += LJD_CH) {
        const int nj = min(LJD_CH, N - t0);
        __syncthreads();
        for (int k = threadIdx.x; k < nj; k += 128) sj[k] = opos[t0 + k];
        __syncthreads();
        if (!act) continue;
#pragma unroll 4
        for (int jj = sub; jj < nj; jj += LJD_SUB) {
            float r[3], rr;
            const int c = ljd_classify(oi, sj[jj], K, r, &rr);
            if (c == 1 && t0 + jj != i) ljd_pair(r, rr, K, fx, fy, fz, el);
            flagged |= (c == 2);
        }
    }
    // second pass, only in blocks that saw a pair needing the FP64 decision
    if (__syncthreads_or(flagged)) {
        const double *q = a.pos + J.pos_off;
        for (int t0 = 0; t0 < N; t0 += LJD_CH) {
            const int nj = min(LJD_CH, N - t0);
            __syncthreads();
            for (int k = threadIdx.x; k < nj; k += 128) sj[k] = opos[t0 + k];
            __syncthreads();
            if (!act || !flagged) continue;
            for (int jj = sub; jj < nj; jj += LJD_SUB) {
                const int j = t0 + jj;
                float r[3], rr;
                if (j == i || ljd_classify(oi, sj[jj], K, r, &rr) != 2) continue;
                double rd[3];
                const double r2d = lj_exact_disp(q + 9 * i, q + 9 * j, S, rd);
                if (r2d < rc2) {
                    r[0] = (float)rd[0];
                    r[1] = (float)rd[1];
                    r[2] = (float)rd[2];
                    ljd_pair(r, (float)r2d, K, fx, fy, fz, el);
                }
            }
        }
    }
#pragma unroll
    for (int m = 1; m < LJD_SUB; m <<= 1) {
        fx += __shfl_xor_sync(0xffffffffu, fx, m);
        fy += __shfl_xor_sync(0xffffffffu, fy, m);
        fz += __shfl_xor_sync(0xffffffffu, fz, m);
        el += __shfl_xor_sync(0xffffffffu, el, m);
    }
    float e = 0.f;
    if (act && sub == 0) {
        if (a.lj_plane) {
            a.ljf[J.site_off / 3 + i] = make_float4(fx, fy, fz, 0.f);
        } else {
            double *f = a.out + J.out_off;
            f[9 * i] += (double)fx;
            f[9 * i + 1] += (double)fy;
            f[9 * i + 2] += (double)fz;
        }
        e = 0.5f * el;
    }
    // the block's FP32 partial (as the real-space warp partials), added to the FP64 energy
    __shared__ float redf[4];
    e = warp_sum(e);
    if ((threadIdx.x & 31) == 0) redf[threadIdx.x >> 5] = e;
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], (double)(((redf[0] + redf[1]) + redf[2]) + redf[3]));
}

// O-O Lennard-Jones of large beads in the mixed stepper: a warp per row of the
// stepper's symmetric Verlet list (every j != i with r < r_skin at the list's
// build, which holds every pair inside r_cut while the skin test holds), the
// pair classification and term of k_lj_dense in FP32 and, for the rare pairs in
// the band around r_cut^2 or at a half-box tie, the reference's FP64 decision
// inline. The row's force goes to the oxygen-force plane the combine adds; each
// pair is seen from both ends and the energy halved.
constexpr int LJL_U = 8;  // list entries a lane loads at a time in k_lj_list_f32
__global__ void __launch_bounds__(128) k_lj_list_f32(EvalArgs a) {
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int N = S.n_mols;
    if (blockIdx.x * 4 >= N) return;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int i = blockIdx.x * 4 + w;
    const Consts &C = a.c;
    LjdConst K;
    for (int d = 0; d < 3; ++d) {
        K.L[d] = S.boxf[d];
        K.I[d] = S.inv_boxf[d];
    }
    K.rc2 = C.ljf[5];
    K.band = 1e-5f * K.rc2;
    K.tie = 1e-5f;
    K.s6 = C.ljf[0];
    K.s12 = C.ljf[1];
    K.eps4 = C.ljf[2];
    K.eps24 = C.ljf[3];
    K.ecut = C.ljf[4];
    K.tie_mask = S.lj_tie_mask;
    float fx = 0.f, fy = 0.f, fz = 0.f, el = 0.f;
    if (i < N) {
        const int cap = 2 * S.list_size;
        const int *pt = a.point_full + S.pf_off + (size_t)J.bead * (N + 1);
        const int *ls = a.list_full + S.lf_off + (size_t)J.bead * cap;
        // a row outside [0, capacity] or an index outside the bead is skipped and flagged
        int n0 = pt[i], n1 = pt[i + 1];
        if (n0 < 0 || n1 > cap || n0 > n1) {
            if (lane == 0) atomicOr(a.status, (unsigned)ST_LIST_OVERFLOW);
            n0 = max(0, min(n0, cap));
            n1 = max(n0, min(n1, cap));
        }
        const float4 *opos = reinterpret_cast<const float4 *>(a.opos) + J.site_off / 3;
        const float4 oi = opos[i];
        // LJL_U entries a lane at a time: their indices, then their positions, then
        // the pairs (the gathers of one batch in flight together)
        bool flagged = false;
        for (int base = n0; base < n1; base += 32 * LJL_U) {
            int jv[LJL_U];
            float4 ov[LJL_U];
#pragma unroll
            for (int u = 0; u < LJL_U; ++u) {
                const int n = base + u * 32 + lane;
                jv[u] = n < n1 ? ls[n] : -1;
            }
#pragma unroll
            for (int u = 0; u < LJL_U; ++u) {
                const bool ok = jv[u] >= 0 && jv[u] < N && jv[u] != i;
                ov[u] = ok ? opos[jv[u]] : oi;
            }
#pragma unroll
            for (int u = 0; u < LJL_U; ++u) {
                const int j = jv[u];
                if (base + u * 32 + lane >= n1) continue;
                if (j == i || j < 0 || j >= N) {
                    atomicOr(a.status, (unsigned)ST_LIST_OVERFLOW);
                    continue;
                }
                float r[3], rr;
                const int c = ljd_classify(oi, ov[u], K, r, &rr);
                if (c == 1) ljd_pair(r, rr, K, fx, fy, fz, el);
                flagged |= (c == 2);
            }
        }
        // the pairs in the band around r_cut^2 or at a half-box tie, with the
        // reference's FP64 decision, only in warps that met one
        if (__any_sync(0xffffffffu, flagged) && flagged) {
            const double *q = a.pos + J.pos_off;
            for (int n = n0 + lane; n < n1; n += 32) {
                const int j = ls[n];
                float r[3], rr;
                if (j == i || j < 0 || j >= N || ljd_classify(oi, opos[j], K, r, &rr) != 2) continue;
                double rd[3];
                const double r2d = lj_exact_disp(q + 9 * i, q + 9 * j, S, rd);
                if (r2d < C.r_cut_sq) {
                    r[0] = (float)rd[0];
                    r[1] = (float)rd[1];
                    r[2] = (float)rd[2];
                    ljd_pair(r, (float)r2d, K, fx, fy, fz, el);
                }
            }
        }
        fx = warp_sum(fx);
        fy = warp_sum(fy);
        fz = warp_sum(fz);
        el = warp_sum(el);
        if (lane == 0) a.ljf[J.site_off / 3 + i] = make_float4(fx, fy, fz, 0.f);
    }
    // the block's FP32 partial (as k_lj_dense), added to the FP64 energy
    __shared__ float redf[4];
    if (lane == 0) redf[w] = i < N ? 0.5f * el : 0.f;
    __syncthreads();
    if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], (double)(((redf[0] + redf[1]) + redf[2]) + redf[3]));
}

// site-force output of the reciprocal-space-only path: out += sum of the k-chunk planes
template <typename R>
__global__ void k_sum_parts(EvalArgs a) {
    const Job J = a.jobs[blockIdx.y];
    const SysDev &S = a.sys[J.sys];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= 3 * S.n_sites) return;
    const R *part = reinterpret_cast<const R *>(a.part);
    double v = 0.0;
    for (int p = 0; p < a.n_rj + a.n_kc; ++p) v += (double)part[3 * ((size_t)p * a.total_sites + J.site_off) + t];
    a.out[J.out_off + t] += v;
}

// FP32 FMA throughput probe: 8 independent dependent chains per thread.
__global__ void __launch_bounds__(256) k_fp32_probe(float *out, int iters) {
    float v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = 1.0f + 1e-7f * (threadIdx.x + k);
    const float b = 0.9999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = fmaf(v[k], b, c);
    }
    float t = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) t += v[k];
    if (t == 12345.f) out[0] = t;  // keeps the chains live
}

// FP64 counterpart: eight independent dependent chains of double FMAs a thread.
__global__ void __launch_bounds__(256) k_fp64_probe(double *out, int iters) {
    double v[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) v[k] = 1.0 + 1e-15 * (threadIdx.x + k);
    const double b = 0.9999999999999, c = 1e-15;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) v[k] = fma(v[k], b, c);
    }
    double t = 0.0;
#pragma unroll
    for (int k = 0; k < 8; ++k) t += v[k];
    if (t == 12345.0) out[0] = t;  // keeps the chains live
}

template <typename R>
size_t ksk_smem(int kmax) {
    return 2 * (CH * sizeof(V4<R>) + (size_t)3 * (kmax + 1) * (CH + 1) * sizeof(V2<R>));
}
template <typename R>
size_t kforce_smem(int kmax) {
    return (size_t)KB * (sizeof(KCol) + 2 * sizeof(V2<R>)) + (size_t)(kmax + 1) * FT * sizeof(V2<R>);
}

template <typename R>
void set_attrs() {
    const int big = 200 * 1024;
    cudaFuncSetAttribute(k_kforce_f32<8, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_kforce_f32<12, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_kforce_f32<16, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_kforce_f32<24, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_kforce_f32<32, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_ksk<R, 0, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_ksk<R, 1, 3>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_ksk<R, 0, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_ksk<R, 1, 4>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_kforce<R, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_kforce<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
}

// Chunk counts so that each force kernel launches enough 4-warp blocks to keep
// per_sm blocks (12: 48 warps) resident on each of the 152 SMs.
int chunks_for(long long base_blocks, int maxc, int per_sm = 12) {
    const long long want = (long long)per_sm * 152;
    const int c = (int)((want + base_blocks - 1) / std::max(1LL, base_blocks));
    return std::max(1, std::min(c, maxc));
}
// a tuned count when the autotuner fixed one, else the heuristic
int chunks_or(int tuned, long long base_blocks, int maxc, int per_sm = 12) {
    return tuned > 0 ? std::min(tuned, maxc) : chunks_for(base_blocks, maxc, per_sm);
}

void launch_lj_dense(const EvalArgs &a, cudaStream_t s) {
    if (a.lj_list && a.lj_plane) {  // large beads: the symmetric Verlet list instead of every pair
        k_lj_list_f32<<<dim3((a.max_mols + 3) / 4, a.n_jobs), 128, 0, s>>>(a);
        return;
    }
    if (a.lj_list) {
        k_lj<float, 1><<<dim3((a.max_mols + 3) / 4, a.n_jobs), 128, 0, s>>>(a);
        return;
    }
    const long long blocks8 = (long long)((a.max_mols + 15) / 16) * a.n_jobs;
    if (blocks8 >= 2LL * 152) k_lj_dense<8><<<dim3((a.max_mols + 15) / 16, a.n_jobs), 128, 0, s>>>(a);
    else k_lj_dense<32><<<dim3((a.max_mols + 3) / 4, a.n_jobs), 128, 0, s>>>(a);
}

// The half-interaction real-space kernel applies to beads of at most
// HALF_MAX_TILES tiles; its plane count is n_ch + T / 2 (n_ch from the
// autotuner's real-space count, else sized for ~12 warps' blocks per SM).
bool half_ok(const EvalArgs &a) { return (3 * a.max_mols + 31) / 32 <= HALF_MAX_TILES; }
int half_chunks(const EvalArgs &a) {
    const int T = (3 * a.max_mols + 31) / 32;
    const long long blocks = (long long)((T + HW - 1) / HW) * a.n_jobs;
    // the autotuner's picks on the 512-water P = 32 step: the most chunks (20 blocks an SM)
    return chunks_or(a.tune_rj, blocks, HALF_MAX_CH, 20);
}
void launch_real_half(EvalArgs &a, cudaStream_t s) {
    const int T = (3 * a.max_mols + 31) / 32, n_ch = half_chunks(a);
    a.n_rj = 0;  // no real-space planes: the combine reads the fixed-point sums
    a.real_fix = 1;
    k_real_half<<<dim3((T + HW - 1) / HW, n_ch, a.n_jobs), 32 * HW, 0, s>>>(a, n_ch);
}

// The pair-list real space (mixed, forces, beads beyond the half-interaction
// kernel, when the context enabled it): its chunk count (planes) per row, sized
// like the other force kernels' grids; three launches (test, rows, forces).
bool list_ok(const EvalArgs &a) { return a.rl_on && a.mode == 0 && !half_ok(a); }
int list_chunks(const EvalArgs &a) {
    return chunks_or(a.tune_rj, (long long)((a.max_mols + RLW - 1) / RLW) * a.n_jobs, MAX_RJ);
}
void launch_real_list(EvalArgs &a, cudaStream_t s) {
    a.n_rj = list_chunks(a);
    cudaMemsetAsync(a.rl_count, 0, sizeof(int), s);
    k_rlist_test<<<dim3((3 * a.max_mols + RLT_SITES - 1) / RLT_SITES, a.n_jobs), 256, 0, s>>>(a);
    const int row_blocks = (a.max_mols + RL_ROWS - 1) / RL_ROWS;
    // one block an SM, or one per 16 items of a rebuild of every configuration when
    // that is more (at most eight an SM): a launch without rebuilds costs each block one load of the count,
    // and a wide grid holds thread slots the force kernels beside it need
    const long long items = (long long)row_blocks * a.n_jobs;
    const int grid = (int)std::min<long long>(items, std::max<long long>(152LL, std::min<long long>(items / 16, 152LL * 8)));
    k_rlist_rows<<<grid, 32 * RL_ROWS, 0, s>>>(a, row_blocks);
    k_real_list<<<dim3((a.max_mols + RLW - 1) / RLW, a.n_rj, a.n_jobs), 32 * RLW, 0, s>>>(a);
}

template <typename R>
void launch_ewald(EvalArgs a, cudaStream_t s, unsigned long long *n, const Forks *forks = nullptr) {
    const int ns = 3 * a.max_mols;
    const int tiles = (ns + RT - 1) / RT, ktiles = (a.max_grp + KT - 1) / KT;
    a.n_rj = chunks_or(a.tune_rj, (long long)tiles * a.n_jobs, MAX_RJ);
    a.n_sc = chunks_or(a.tune_sc, (long long)ktiles * a.n_jobs, MAX_SC);
    a.n_kc = chunks_or(a.tune_kc, (long long)tiles * a.n_jobs, MAX_KC);
    if (sizeof(R) == 4 && forks && a.mode == 0 && a.lj_full && a.ljf) {
        // forked: prep; then real space | reciprocal chain | dense LJ; then combine.
        // The reciprocal chain runs beside the real-space kernel: its grids aim for
        // a third (structure factors) and half (k-force) of the blocks a kernel alone
        // would (the autotuner's picks on the 512-water P = 32 step)
        a.n_sc = chunks_or(a.tune_sc, (long long)ktiles * a.n_jobs, MAX_SC, 4);
        a.n_kc = chunks_or(a.tune_kc, (long long)tiles * a.n_jobs, MAX_KC, 6);
        if (half_ok(a)) {  // k_kforce_f32's planes follow the real-space ones: none here
            a.n_rj = 0;
            a.real_fix = 1;
        }
        else if (list_ok(a)) a.n_rj = list_chunks(a);  // k_kforce_f32's planes follow the real-space ones
        a.lj_plane = 1;
        launch_prep_f32(a, s);
        // capture order: the reciprocal chain (the critical path: three dependent
        // kernels) first, then the Lennard-Jones branch, the real-space kernel last
        // (it fills the SMs the others leave; captured first, the step took 11-14 %
        // longer)
        cudaEventRecord(forks->fork, s);
        cudaStreamWaitEvent(forks->side[0], forks->fork, 0);
        cudaStreamWaitEvent(forks->side[1], forks->fork, 0);
        launch_ksk<R, 0>(a, dim3(ktiles, a.n_sc, a.n_jobs), forks->side[0]);
        launch_sk_reduce<R, 0>(a, forks->side[0]);
        launch_kforce_f32(a, dim3(tiles, a.n_kc, a.n_jobs), forks->side[0]);
        cudaEventRecord(forks->join[0], forks->side[0]);
        if (a.lj_list && forks->lists_ready) cudaStreamWaitEvent(forks->side[1], forks->lists_ready, 0);
        launch_lj_dense(a, forks->side[1]);
        if (a.intra) {
            a.intra_plane = 1;
            k_intra_f32<<<dim3((a.max_mols + 127) / 128, a.n_jobs), 128, 0, forks->side[1]>>>(a);
        }
        cudaEventRecord(forks->join[1], forks->side[1]);
        if (half_ok(a)) launch_real_half(a, s);
        else if (list_ok(a)) launch_real_list(a, s);
        else k_real_f32<<<dim3(tiles, a.n_rj, a.n_jobs), RT, 0, s>>>(a);
        cudaStreamWaitEvent(s, forks->join[0], 0);
        cudaStreamWaitEvent(s, forks->join[1], 0);
        k_combine_f32<<<dim3((a.max_mols + CMB - 1) / CMB, a.n_jobs), 128, 0, s>>>(a);
        if (n) *n += (a.intra_plane ? 8 : 7) + (list_ok(a) ? 2 : 0);
        return;
    }
    if constexpr (sizeof(R) == 4) launch_prep_f32(a, s);
    else k_prep<R><<<dim3((ns + 127) / 128, a.n_jobs), 128, 0, s>>>(a);
    if (a.mode == 0) {
        if (sizeof(R) == 4 && half_ok(a)) launch_real_half(a, s);
        else if (sizeof(R) == 4 && list_ok(a)) {
            launch_real_list(a, s);
            if (n) *n += 2;
        } else if (sizeof(R) == 4) k_real_f32<<<dim3(tiles, a.n_rj, a.n_jobs), RT, 0, s>>>(a);
        else k_real<R, 0><<<dim3(tiles, a.n_rj, a.n_jobs), RT, 0, s>>>(a);
        launch_ksk<R, 0>(a, dim3(ktiles, a.n_sc, a.n_jobs), s);
        launch_sk_reduce<R, 0>(a, s);
        if (sizeof(R) == 4) launch_kforce_f32(a, dim3(tiles, a.n_kc, a.n_jobs), s);
        else k_kforce<R, 0><<<dim3(tiles, a.n_kc, a.n_jobs), FT, kforce_smem<R>(a.max_kmax), s>>>(a);
    } else {
        k_real<R, 1><<<dim3(tiles, a.n_rj, a.n_jobs), RT, 0, s>>>(a);
        launch_ksk<R, 1>(a, dim3(ktiles, a.n_sc, a.n_jobs), s);
        launch_sk_reduce<R, 1>(a, s);
        k_kforce<R, 1><<<dim3(tiles, a.n_kc, a.n_jobs), FT, kforce_smem<R>(a.max_kmax), s>>>(a);
    }
    const dim3 gm((a.max_mols + 127) / 128, a.n_jobs);
    // mixed with the dense Lennard-Jones: its oxygen forces go to their plane first,
    // so the combine writes the complete force
    const bool plane = sizeof(R) == 4 && a.mode == 0 && a.lj_full && a.ljf;
    if (plane) {
        a.lj_plane = 1;
        launch_lj_dense(a, s);
    }
    if (sizeof(R) == 4) k_combine_f32<<<dim3((a.max_mols + CMB - 1) / CMB, a.n_jobs), 128, 0, s>>>(a);
    else k_combine<double><<<gm, 128, 0, s>>>(a);
    if (n) *n += plane ? 7 : 6;
    if (a.mode == 0 && !plane) {
        if (sizeof(R) == 4 && a.lj_full)
            launch_lj_dense(a, s);
        else if (a.lj_full) k_lj<R, 1><<<dim3((a.max_mols + 3) / 4, a.n_jobs), 128, 0, s>>>(a);
        else k_lj<R, 0><<<dim3((a.max_mols + 3) / 4, a.n_jobs), 128, 0, s>>>(a);
        if (n) *n += 1;
    }
}

}  // namespace

void launch_fp32_probe(float *out, int blocks, int iters, cudaStream_t s) {
    k_fp32_probe<<<blocks, 256, 0, s>>>(out, iters);
}

void launch_fp64_probe(double *out, int blocks, int iters, cudaStream_t s) {
    k_fp64_probe<<<blocks, 256, 0, s>>>(out, iters);
}

void launch_ewald_kernel(const EvalArgs &a0, bool mixed, const char *name, cudaStream_t s) {
    EvalArgs a = a0;
    const int ns = 3 * a.max_mols;
    const int tiles = (ns + RT - 1) / RT, ktiles = (a.max_grp + KT - 1) / KT;
    // the shapes of the stepper's evaluation (forked in the mixed form; the
    // half-interaction real space leaves fixed-point sums instead of planes)
    a.n_rj = chunks_or(a.tune_rj, (long long)tiles * a.n_jobs, MAX_RJ);
    if (mixed && half_ok(a)) {
        a.n_rj = 0;
        a.real_fix = 1;
    }
    a.n_sc = chunks_or(a.tune_sc, (long long)ktiles * a.n_jobs, MAX_SC, mixed ? 4 : 12);
    a.n_kc = chunks_or(a.tune_kc, (long long)tiles * a.n_jobs, MAX_KC, mixed ? 6 : 12);
    const dim3 gs((ns + 127) / 128, a.n_jobs), gr(tiles, a.n_rj, a.n_jobs);
    const dim3 gk(ktiles, a.n_sc, a.n_jobs), gf(tiles, a.n_kc, a.n_jobs);
    const dim3 gm((a.max_mols + 127) / 128, a.n_jobs), gl((a.max_mols + 3) / 4, a.n_jobs);
    const std::string n(name);
    if (n == "prep") {
        if (mixed) launch_prep_f32(a, s);
        else k_prep<double><<<gs, 128, 0, s>>>(a);
    } else if (n == "real") {
        if (mixed && half_ok(a)) launch_real_half(a, s);
        else if (mixed && list_ok(a)) launch_real_list(a, s);
        else if (mixed) k_real_f32<<<gr, RT, 0, s>>>(a);
        else k_real<double, 0><<<gr, RT, 0, s>>>(a);
    } else if (n == "ksk") {
        if (mixed) launch_ksk<float, 0>(a, gk, s);
        else launch_ksk<double, 0>(a, gk, s);
    } else if (n == "sk_reduce") {
        if (mixed) launch_sk_reduce<float, 0>(a, s);
        else launch_sk_reduce<double, 0>(a, s);
    } else if (n == "kforce") {
        if (mixed) launch_kforce_f32(a, gf, s);
        else k_kforce<double, 0><<<gf, FT, kforce_smem<double>(a.max_kmax), s>>>(a);
    } else if (n == "combine") {
        if (mixed) k_combine_f32<<<dim3((a.max_mols + CMB - 1) / CMB, a.n_jobs), 128, 0, s>>>(a);
        else k_combine<double><<<gm, 128, 0, s>>>(a);
    } else if (n == "lj") {
        if (mixed) {
            if (a.lj_full && a.ljf) a.lj_plane = 1;  // as the stepper's forked evaluation
            if (a.lj_full) launch_lj_dense(a, s);
            else k_lj<float, 0><<<gl, 128, 0, s>>>(a);
        } else {
            if (a.lj_full) k_lj<double, 1><<<gl, 128, 0, s>>>(a);
            else k_lj<double, 0><<<gl, 128, 0, s>>>(a);
        }
    }
}

void init_force_kernel_attributes() {
    set_attrs<float>();
    set_attrs<double>();
}

void launch_eval_fp64(const EvalArgs &a, cudaStream_t s, unsigned long long *n) {
    if (a.n_jobs <= 0) return;
    if (!a.sr_only) {
        launch_ewald<double>(a, s, n);
        return;
    }
    // short-range terms only (FP64): LJ reads the raw positions, no preparation pass
    const dim3 gm((a.max_mols + 127) / 128, a.n_jobs);
    k_combine<double><<<gm, 128, 0, s>>>(a);
    if (a.lj_full) k_lj<double, 1><<<dim3((a.max_mols + 3) / 4, a.n_jobs), 128, 0, s>>>(a);
    else k_lj<double, 0><<<dim3((a.max_mols + 3) / 4, a.n_jobs), 128, 0, s>>>(a);
    if (n) *n += 2;
}

void launch_eval_mixed(const EvalArgs &a, cudaStream_t s, unsigned long long *n, const Forks *forks) {
    if (a.n_jobs <= 0) return;
    if (a.sr_only) {
        launch_eval_fp64(a, s, n);  // the finite-difference short-range terms stay FP64
        return;
    }
    launch_ewald<float>(a, s, n, forks);
}

// Reciprocal space only, on caller-supplied charge sites: out (site forces,
// 9N per job) += k-space forces.
void launch_kwald_only(const EvalArgs &a0, bool mixed, cudaStream_t s, unsigned long long *n) {
    if (a0.n_jobs <= 0) return;
    EvalArgs a = a0;
    const int ns = 3 * a.max_mols;
    const int tiles = (ns + FT - 1) / FT, ktiles = (a.max_grp + KT - 1) / KT;
    a.n_rj = 0;
    a.n_sc = chunks_or(a.tune_sc, (long long)ktiles * a.n_jobs, MAX_SC);
    a.n_kc = chunks_or(a.tune_kc, (long long)tiles * a.n_jobs, MAX_KC);
    const dim3 gs((ns + 127) / 128, a.n_jobs), gk(ktiles, a.n_sc, a.n_jobs), gf(tiles, a.n_kc, a.n_jobs);
    if (mixed) {
        launch_prep_f32(a, s);
        launch_ksk<float, 0>(a, gk, s);
        launch_sk_reduce<float, 0>(a, s);
        launch_kforce_f32(a, gf, s);
    } else {
        k_prep<double><<<gs, 128, 0, s>>>(a);
        launch_ksk<double, 0>(a, gk, s);
        launch_sk_reduce<double, 0>(a, s);
        k_kforce<double, 0><<<gf, FT, kforce_smem<double>(a.max_kmax), s>>>(a);
    }
    if (mixed) k_sum_parts<float><<<dim3((3 * ns + 127) / 128, a.n_jobs), 128, 0, s>>>(a);
    else k_sum_parts<double><<<dim3((3 * ns + 127) / 128, a.n_jobs), 128, 0, s>>>(a);
    if (n) *n += 5;
}

}  // namespace qtg
