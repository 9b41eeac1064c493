// qTIP4P/F force evaluation on GB300 (replaces forces.cpp:25-630).
//
// A launch evaluates a batch of "jobs" (one configuration of one system each;
// all beads of all replicas at once). Per job:
//   k_prep     charge sites (M, H1, H2) wrapped into the box, charges, and the
//              per-site phase tables exp(i 2 pi m s_d), m = 0..k_max, d = x,y,z
//              (charge folded into the x factor);
//   k_real     real-space Ewald between sites of different molecules, j-sites
//              tiled through shared memory, every i-site owned by one thread
//              (no atomics, deterministic);
//   k_ksk      structure factors S(k) = sum_i q_i exp(i k.r_i), one thread per
//              k-vector, site chunks staged in shared memory; chunk partial sums
//              are promoted to FP64 (compensated accumulation);
//   k_kforce   reciprocal-space site forces, one thread per site, k-vector
//              chunks (k, 2 c_k k, S(k)) broadcast from shared memory;
//   k_combine  FP64 per molecule: same-molecule real-space pairs (erfc - 1),
//              quartic-Morse bonds, HOH angle, M-site chain rule;
//   k_lj       FP64 O-O Lennard-Jones over the CSR Verlet list.
// The Ewald kernels are templated on the arithmetic type: double for the
// parity mode, float (FP64 accumulation across tiles/chunks) for the mixed mode.
// Mode-1 jobs compute the directional derivative of the intermolecular Ewald
// forces along a per-dof direction (used by the Suzuki-Chin force gradient).
#include <math.h>

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

__device__ __forceinline__ float f_erfc(float x) { return erfcf(x); }
__device__ __forceinline__ double f_erfc(double x) { return erfc(x); }
__device__ __forceinline__ float f_exp(float x) { return expf(x); }
__device__ __forceinline__ double f_exp(double x) { return exp(x); }
__device__ __forceinline__ float f_rint(float x) { return rintf(x); }
__device__ __forceinline__ double f_rint(double x) { return rint(x); }
__device__ __forceinline__ float f_sqrt(float x) { return sqrtf(x); }
__device__ __forceinline__ double f_sqrt(double x) { return sqrt(x); }
__device__ __forceinline__ void f_sincospi(float t, float *s, float *c) { sincospif(t, s, c); }
__device__ __forceinline__ void f_sincospi(double t, double *s, double *c) { sincospi(t, s, c); }

template <typename R> __device__ __forceinline__ R sys_box(const SysDev &S, int d);
template <> __device__ __forceinline__ float sys_box<float>(const SysDev &S, int d) { return S.boxf[d]; }
template <> __device__ __forceinline__ double sys_box<double>(const SysDev &S, int d) { return S.box[d]; }
template <typename R> __device__ __forceinline__ R sys_ibox(const SysDev &S, int d);
template <> __device__ __forceinline__ float sys_ibox<float>(const SysDev &S, int d) { return S.inv_boxf[d]; }
template <> __device__ __forceinline__ double sys_ibox<double>(const SysDev &S, int d) { return S.inv_box[d]; }

// ---- k_prep -------------------------------------------------------------------
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
    }
    const double chg = a.charge[S.chg_off + s];
    double frac[3];
    for (int d = 0; d < 3; ++d) {
        double t = x[d] * S.inv_box[d];
        frac[d] = t - floor(t);
    }
    V4<R> *sites = reinterpret_cast<V4<R> *>(a.sites) + J.site_off;
    V4<R> sv;
    sv.x = (R)(frac[0] * S.box[0]);
    sv.y = (R)(frac[1] * S.box[1]);
    sv.z = (R)(frac[2] * S.box[2]);
    sv.w = (R)chg;
    sites[s] = sv;
    if (J.mode == 1) {
        V4<R> *tan = reinterpret_cast<V4<R> *>(a.tan_sites) + J.site_off;
        V4<R> tv;
        tv.x = (R)u[0];
        tv.y = (R)u[1];
        tv.z = (R)u[2];
        tv.w = (R)0;
        tan[s] = tv;
    }
    // phase table exp(i 2 pi m frac_d), layout [(d * (kmax+1) + m) * ns + s]
    const int km1 = S.k_max + 1;
    V2<R> *ph = reinterpret_cast<V2<R> *>(a.phase) + J.phase_off;
    for (int d = 0; d < 3; ++d) {
        for (int m = 0; m < km1; ++m) {
            double t = 2.0 * m * frac[d];
            t -= 2.0 * floor(0.5 * t + 0.5);  // in [-1, 1)
            R sn, cs;
            f_sincospi((R)t, &sn, &cs);
            if (d == 0) {
                cs = (R)(cs * chg);
                sn = (R)(sn * chg);
            }
            V2<R> e;
            e.x = cs;
            e.y = sn;
            ph[(size_t)(d * km1 + m) * ns + s] = e;
        }
    }
}

// ---- k_real: intermolecular real-space Ewald ----------------------------------
constexpr int RT = 128;

template <typename R, int MODE>
__global__ void __launch_bounds__(RT) k_real(EvalArgs a) {
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int ns = S.n_sites;
    if (blockIdx.x * RT >= ns) return;
    const int i = blockIdx.x * RT + threadIdx.x;
    const bool act = i < ns;
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
    const int mi = i / 3;
    double Fx = 0.0, Fy = 0.0, Fz = 0.0, E = 0.0;
    for (int t0 = 0; t0 < ns; t0 += RT) {
        __syncthreads();
        if (t0 + threadIdx.x < ns) {
            sj[threadIdx.x] = sites[t0 + threadIdx.x];
            if (MODE == 1) uj[threadIdx.x] = tans[t0 + threadIdx.x];
        }
        __syncthreads();
        const int nj = min(RT, ns - t0);
        R fx = 0, fy = 0, fz = 0, e = 0;
        if (act) {
            for (int jj = 0; jj < nj; ++jj) {
                const int j = t0 + jj;
                if (j / 3 == mi) continue;
                const V4<R> b = sj[jj];
                R dx = si.x - b.x, dy = si.y - b.y, dz = si.z - b.z;
                dx -= L0 * f_rint(dx * I0);
                dy -= L1 * f_rint(dy * I1);
                dz -= L2 * f_rint(dz * I2);
                const R r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rc2) {
                    const R r = f_sqrt(r2);
                    const R inv = (R)1 / r;
                    const R qq = si.w * b.w;
                    const R ex = f_exp(-kap2 * r2);
                    const R en = qq * inv * f_erfc(kap * r);
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
    if (act) {
        double *fs = a.site_force + 3 * (J.site_off + i);
        fs[0] = Fx;
        fs[1] = Fy;
        fs[2] = Fz;
    }
    if (MODE == 0) {
        double t = block_sum(0.5 * E, red);
        if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
    }
}

// ---- k_ksk: structure factors ---------------------------------------------------
constexpr int KT = 128;  // threads (k-vectors) per block
constexpr int CH = 32;   // sites per shared-memory chunk

template <typename R, int MODE>
__global__ void __launch_bounds__(KT) k_ksk(EvalArgs a) {
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int nk = S.n_kvec, ns = S.n_sites, km1 = S.k_max + 1;
    if (blockIdx.x * KT >= nk) return;
    const int t = blockIdx.x * KT + threadIdx.x;
    const bool act = t < nk;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // 16-byte elements first so every array stays aligned for vector access
    V4<R> *ush = reinterpret_cast<V4<R> *>(smem_raw);                 // [CH] (mode 1)
    V2<R> *tab = reinterpret_cast<V2<R> *>(ush + CH);                 // [3*km1][CH+1]
    __shared__ double red[KT / 32];
    KVec kv;
    kv.kx = kv.ky = kv.kz = 0;
    kv.coef = 0.0;
    if (act) kv = a.kvec[S.kvec_off + t];
    const int ax = kv.kx, ay = abs(kv.ky), az = abs(kv.kz);
    const R sy = kv.ky < 0 ? (R)-1 : (R)1, sz = kv.kz < 0 ? (R)-1 : (R)1;
    const R kx = (R)(2.0 * PI_REF * kv.kx * S.inv_box[0]);
    const R ky = (R)(2.0 * PI_REF * kv.ky * S.inv_box[1]);
    const R kz = (R)(2.0 * PI_REF * kv.kz * S.inv_box[2]);
    const V2<R> *ph = reinterpret_cast<const V2<R> *>(a.phase) + J.phase_off;
    const V4<R> *tans = reinterpret_cast<const V4<R> *>(a.tan_sites) + J.site_off;
    double Sr = 0.0, Si = 0.0, dSr = 0.0, dSi = 0.0;
    const int rows = 3 * km1;
    for (int c0 = 0; c0 < ns; c0 += CH) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < rows * CH; idx += KT) {
            const int row = idx / CH, c = idx - row * CH, s = c0 + c;
            V2<R> v;
            v.x = v.y = (R)0;
            if (s < ns) v = ph[(size_t)row * ns + s];
            tab[row * (CH + 1) + c] = v;
        }
        if (MODE == 1 && threadIdx.x < CH) {
            V4<R> z;
            z.x = z.y = z.z = z.w = (R)0;
            ush[threadIdx.x] = (c0 + threadIdx.x < ns) ? tans[c0 + threadIdx.x] : z;
        }
        __syncthreads();
        const int nc = min(CH, ns - c0);
        R sr = 0, si = 0, dsr = 0, dsi = 0;
        const V2<R> *X = tab + ax * (CH + 1);
        const V2<R> *Y = tab + (km1 + ay) * (CH + 1);
        const V2<R> *Z = tab + (2 * km1 + az) * (CH + 1);
        for (int c = 0; c < nc; ++c) {
            const V2<R> x = X[c], y = Y[c], z = Z[c];
            const R yi = sy * y.y, zi = sz * z.y;
            const R pr = x.x * y.x - x.y * yi, pi = x.x * yi + x.y * y.x;
            const R er = pr * z.x - pi * zi, ei = pr * zi + pi * z.x;
            sr += er;
            si += ei;
            if (MODE == 1) {
                const V4<R> u = ush[c];
                const R ku = kx * u.x + ky * u.y + kz * u.z;
                dsr -= ku * ei;
                dsi += ku * er;
            }
        }
        Sr += (double)sr;
        Si += (double)si;
        if (MODE == 1) {
            dSr += (double)dsr;
            dSi += (double)dsi;
        }
    }
    if (act) {
        a.sk[J.sk_off + t] = make_double2(Sr, Si);
        if (MODE == 1) a.dsk[J.sk_off + t] = make_double2(dSr, dSi);
    }
    if (MODE == 0) {
        double e = act ? kv.coef * (Sr * Sr + Si * Si) : 0.0;
        double tot = block_sum(e, red);
        if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], tot);
    }
}

// ---- k_kforce: reciprocal-space site forces -------------------------------------
constexpr int FT = 128;  // threads (sites) per block
constexpr int KC = 128;  // k-vectors per shared-memory chunk

template <typename R, int MODE>
__global__ void __launch_bounds__(FT) k_kforce(EvalArgs a) {
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int nk = S.n_kvec, ns = S.n_sites, km1 = S.k_max + 1;
    if (blockIdx.x * FT >= ns) return;
    const int i = blockIdx.x * FT + threadIdx.x;
    const bool act = i < ns;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    // 16-byte elements first so every array stays aligned for vector access
    int4 *kk = reinterpret_cast<int4 *>(smem_raw);      // [KC]
    V4<R> *gg = reinterpret_cast<V4<R> *>(kk + KC);     // [KC]
    V2<R> *ss = reinterpret_cast<V2<R> *>(gg + KC);     // [KC]
    V2<R> *ds = ss + KC;                                // [KC]
    V2<R> *myph = ds + KC;                              // [3*km1][FT]
    const V2<R> *ph = reinterpret_cast<const V2<R> *>(a.phase) + J.phase_off;
    for (int row = 0; row < 3 * km1; ++row) {
        V2<R> v;
        v.x = v.y = (R)0;
        if (act) v = ph[(size_t)row * ns + i];
        myph[row * FT + threadIdx.x] = v;
    }
    V4<R> ui;
    ui.x = ui.y = ui.z = ui.w = (R)0;
    if (MODE == 1 && act) ui = reinterpret_cast<const V4<R> *>(a.tan_sites)[J.site_off + i];
    const R b0 = (R)(2.0 * PI_REF * S.inv_box[0]), b1 = (R)(2.0 * PI_REF * S.inv_box[1]),
            b2 = (R)(2.0 * PI_REF * S.inv_box[2]);
    double Fx = 0.0, Fy = 0.0, Fz = 0.0;
    for (int k0 = 0; k0 < nk; k0 += KC) {
        __syncthreads();
        for (int idx = threadIdx.x; idx < KC; idx += FT) {
            const int k = k0 + idx;
            if (k < nk) {
                const KVec v = a.kvec[S.kvec_off + k];
                kk[idx] = make_int4(v.kx, abs(v.ky), abs(v.kz), (v.ky < 0 ? 1 : 0) | (v.kz < 0 ? 2 : 0));
                V4<R> g;
                g.x = (R)v.gx;
                g.y = (R)v.gy;
                g.z = (R)v.gz;
                g.w = (R)0;
                gg[idx] = g;
                const double2 sk = a.sk[J.sk_off + k];
                V2<R> s2;
                s2.x = (R)sk.x;
                s2.y = (R)sk.y;
                ss[idx] = s2;
                if (MODE == 1) {
                    const double2 d = a.dsk[J.sk_off + k];
                    V2<R> d2;
                    d2.x = (R)d.x;
                    d2.y = (R)d.y;
                    ds[idx] = d2;
                }
            }
        }
        __syncthreads();
        const int nc = min(KC, nk - k0);
        R fx = 0, fy = 0, fz = 0;
        for (int c = 0; c < nc; ++c) {
            const int4 k = kk[c];
            const V2<R> x = myph[k.x * FT + threadIdx.x];
            const V2<R> y = myph[(km1 + k.y) * FT + threadIdx.x];
            const V2<R> z = myph[(2 * km1 + k.z) * FT + threadIdx.x];
            const R yi = (k.w & 1) ? -y.y : y.y, zi = (k.w & 2) ? -z.y : z.y;
            const R pr = x.x * y.x - x.y * yi, pi = x.x * yi + x.y * y.x;
            const R er = pr * z.x - pi * zi, ei = pr * zi + pi * z.x;
            const V2<R> sk = ss[c];
            R val = sk.x * ei - sk.y * er;  // q_i Im(conj(S) e_i)
            if (MODE == 1) {
                const V2<R> d = ds[c];
                const R sgy = (k.w & 1) ? (R)-1 : (R)1, sgz = (k.w & 2) ? (R)-1 : (R)1;
                const R ku = b0 * (R)k.x * ui.x + b1 * sgy * (R)k.y * ui.y + b2 * sgz * (R)k.z * ui.z;
                val = (d.x * ei - d.y * er) + ku * (sk.x * er + sk.y * ei);
            }
            const V4<R> g = gg[c];
            fx += val * g.x;
            fy += val * g.y;
            fz += val * g.z;
        }
        Fx += (double)fx;
        Fy += (double)fy;
        Fz += (double)fz;
    }
    if (act) {
        double *fs = a.site_force + 3 * (J.site_off + i);
        fs[0] += Fx;
        fs[1] += Fy;
        fs[2] += Fz;
    }
}

// ---- k_combine: FP64 short-range terms and the M-site chain rule ------------------

__device__ __forceinline__ void min_image3(double *r, const SysDev &S) {
    for (int d = 0; d < 3; ++d) r[d] -= S.box[d] * round(r[d] / S.box[d]);
}

// same-molecule real-space pair with erfc - 1 (forces.cpp:141-177)
__device__ __forceinline__ double ewald_same_mol(const double *ri, const double *rj, double qiqj,
                                                 const SysDev &S, double *fi, double *fj) {
    double r[3];
    for (int d = 0; d < 3; ++d) r[d] = ri[d] - rj[d];
    min_image3(r, S);
    const double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
    if (!(r2 < S.rc_sq)) return 0.0;
    const double rl = sqrt(r2), inv = 1.0 / rl;
    const double ec = erfc(S.kappa * rl) - 1.0;
    const double e = qiqj * inv * ec;
    const double ff = (e + qiqj * S.ewald_pref * exp(-(S.kappa * S.kappa) * r2)) * inv * inv;
    for (int d = 0; d < 3; ++d) {
        fi[d] += ff * r[d];
        fj[d] -= ff * r[d];
    }
    return e;
}

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
        if (a.sr_only) {
            for (int k = 0; k < 9; ++k) fs[k] = 0.0;
        } else {
            const double *sf = a.site_force + 3 * (J.site_off + 3 * m);
            for (int k = 0; k < 9; ++k) fs[k] = sf[k];
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
            e += ewald_same_mol(site, site + 3, chg[0] * chg[1], S, fs, fs + 3);
            e += ewald_same_mol(site, site + 6, chg[0] * chg[2], S, fs, fs + 6);
            e += ewald_same_mol(site + 3, site + 6, chg[1] * chg[2], S, fs + 3, fs + 6);
            // quartic Morse bonds (forces.cpp:65-93, :519-551)
            double ra[3], rb[3];
            for (int d = 0; d < 3; ++d) {
                ra[d] = q[d] - q[3 + d];
                rb[d] = q[d] - q[6 + d];
            }
            min_image3(ra, S);
            min_image3(rb, S);
            const double la = sqrt(ra[0] * ra[0] + ra[1] * ra[1] + ra[2] * ra[2]);
            const double lb = sqrt(rb[0] * rb[0] + rb[1] * rb[1] + rb[2] * rb[2]);
            for (int bnd = 0; bnd < 2; ++bnd) {
                const double *r = bnd ? rb : ra;
                const double rl = bnd ? lb : la;
                const double x = rl - C.roheq, x2 = x * x, x3 = x2 * x, x4 = x2 * x2;
                e += C.Dr * (C.ar2 * x2 - C.ar3 * x3 + C.ar4fac * x4);
                const double gg = (2.0 * C.ar2 * x - 3.0 * C.ar3 * x2 + 4.0 * C.ar4fac * x3) * C.Dr / rl;
                for (int d = 0; d < 3; ++d) {
                    fa[d] -= gg * r[d];
                    fa[3 + 3 * bnd + d] += gg * r[d];
                }
            }
            // harmonic HOH angle (forces.cpp:96-138)
            {
                const double dot = ra[0] * rb[0] + ra[1] * rb[1] + ra[2] * rb[2];
                const double ia = 1.0 / la, ib = 1.0 / lb, iab = ia * ib;
                const double c = dot * iab;
                const double dacos = 1.0 / sqrt(1.0 - c * c);
                const double ca = dot * ia * ia * iab, cb = dot * ib * ib * iab;
                const double dth = acos(c) - C.theta_eq;
                e += 0.5 * C.ktheta * dth * dth;
                const double gp = C.ktheta * dth * dacos;
                for (int d = 0; d < 3; ++d) {
                    fa[d] += gp * (iab * (ra[d] + rb[d]) - ca * ra[d] - cb * rb[d]);
                    fa[3 + d] -= gp * (iab * rb[d] - ca * ra[d]);
                    fa[6 + d] -= gp * (iab * ra[d] - cb * rb[d]);
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
        double t = block_sum(e, red);
        if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
    }
}

// ---- k_lj: O-O Lennard-Jones over the Verlet list (forces.cpp:489-515) -----------
__global__ void __launch_bounds__(128) k_lj(EvalArgs a) {
    const int jb = blockIdx.y;
    const Job J = a.jobs[jb];
    const SysDev &S = a.sys[J.sys];
    const int N = S.n_mols;
    if (blockIdx.x * blockDim.x >= N) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    __shared__ double red[4];
    double e = 0.0;
    if (i < N - 1) {
        const double *q = a.pos + J.pos_off;
        double *f = a.out + J.out_off;
        const int *pt = a.point + S.pt_off + (size_t)J.bead * N;
        const int *ls = a.list + S.ls_off + (size_t)J.bead * S.list_size;
        const Consts &C = a.c;
        double fi[3] = {0.0, 0.0, 0.0};
        // a row outside [0, list_size] (overflowed or caller-corrupted list) or an index
        // outside [0, N) is skipped and flagged instead of being read out of bounds
        int n0 = pt[i], n1 = pt[i + 1];
        if (n0 < 0 || n1 > S.list_size || n0 > n1) {
            atomicOr(a.status, (unsigned)ST_LIST_OVERFLOW);
            n0 = max(0, min(n0, S.list_size));
            n1 = max(n0, min(n1, S.list_size));
        }
        for (int n = n0; n < n1; ++n) {
            const int j = ls[n];
            if (j <= i || j >= N) {
                atomicOr(a.status, (unsigned)ST_LIST_OVERFLOW);
                continue;
            }
            double r[3];
            for (int d = 0; d < 3; ++d) {
                double x = __dsub_rn(q[9 * i + d], q[9 * j + d]);
                r[d] = __dsub_rn(x, __dmul_rn(S.box[d], round(__ddiv_rn(x, S.box[d]))));
            }
            const double r2 = __dadd_rn(__dadd_rn(__dmul_rn(r[0], r[0]), __dmul_rn(r[1], r[1])),
                                        __dmul_rn(r[2], r[2]));
            if (r2 < C.r_cut_sq) {
                const double i2 = 1.0 / r2, i6 = i2 * i2 * i2;
                const double s6 = i6 * C.sigmalj6, s12 = i6 * i6 * C.sigmalj12;
                const double en = s12 - s6;
                e += en * 4.0 * C.epslj - C.e_cut;
                const double ff = (en + s12) * 24.0 * C.epslj * i2;
                for (int d = 0; d < 3; ++d) {
                    fi[d] += ff * r[d];
                    atomicAdd(&f[9 * j + d], -ff * r[d]);
                }
            }
        }
        for (int d = 0; d < 3; ++d) atomicAdd(&f[9 * i + d], fi[d]);
    }
    double t = block_sum(e, red);
    if (threadIdx.x == 0) atomicAdd(&a.energy[J.slot], t);
}

template <typename R>
size_t ksk_smem(int kmax) {
    return (size_t)3 * (kmax + 1) * (CH + 1) * sizeof(V2<R>) + CH * sizeof(V4<R>);
}
template <typename R>
size_t kforce_smem(int kmax) {
    return (size_t)3 * (kmax + 1) * FT * sizeof(V2<R>) + KC * (sizeof(int4) + sizeof(V4<R>) + 2 * sizeof(V2<R>));
}

template <typename R>
void set_attrs() {
    const int big = 200 * 1024;
    cudaFuncSetAttribute(k_ksk<R, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_ksk<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_kforce<R, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
    cudaFuncSetAttribute(k_kforce<R, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, big);
}

template <typename R>
void launch_ewald(const EvalArgs &a, cudaStream_t s, unsigned long long *n) {
    const int ns = 3 * a.max_mols;
    dim3 gs((ns + 127) / 128, a.n_jobs);
    dim3 gk((a.max_kvec + KT - 1) / KT, a.n_jobs);
    k_prep<R><<<gs, 128, 0, s>>>(a);
    if (a.mode == 0) {
        k_real<R, 0><<<dim3((ns + RT - 1) / RT, a.n_jobs), RT, 0, s>>>(a);
        k_ksk<R, 0><<<gk, KT, ksk_smem<R>(a.max_kmax), s>>>(a);
        k_kforce<R, 0><<<dim3((ns + FT - 1) / FT, a.n_jobs), FT, kforce_smem<R>(a.max_kmax), s>>>(a);
    } else {
        k_real<R, 1><<<dim3((ns + RT - 1) / RT, a.n_jobs), RT, 0, s>>>(a);
        k_ksk<R, 1><<<gk, KT, ksk_smem<R>(a.max_kmax), s>>>(a);
        k_kforce<R, 1><<<dim3((ns + FT - 1) / FT, a.n_jobs), FT, kforce_smem<R>(a.max_kmax), s>>>(a);
    }
    if (n) *n += 4;
}

void launch_short_range(const EvalArgs &a, cudaStream_t s, unsigned long long *n) {
    dim3 gm((a.max_mols + 127) / 128, a.n_jobs);
    k_combine<<<gm, 128, 0, s>>>(a);
    if (n) *n += 1;
    if (a.mode == 0) {
        k_lj<<<gm, 128, 0, s>>>(a);
        if (n) *n += 1;
    }
}

// FP32 FMA throughput probe: 8 independent dependent chains per thread.
__global__ void __launch_bounds__(256) k_fp32_probe(float *out, int iters) {
    float a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = 1.0f + 1e-7f * (threadIdx.x + k);
    const float b = 0.9999999f, c = 1e-7f;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int k = 0; k < 8; ++k) a[k] = fmaf(a[k], b, c);
    }
    float t = 0.f;
#pragma unroll
    for (int k = 0; k < 8; ++k) t += a[k];
    if (t == 12345.f) out[0] = t;  // keeps the chains live
}

}  // namespace

void launch_fp32_probe(float *out, int blocks, int iters, cudaStream_t s) {
    k_fp32_probe<<<blocks, 256, 0, s>>>(out, iters);
}

void launch_ewald_kernel(const EvalArgs &a, bool mixed, const char *name, cudaStream_t s) {
    const int ns = 3 * a.max_mols;
    const dim3 gs((ns + 127) / 128, a.n_jobs), gr((ns + RT - 1) / RT, a.n_jobs);
    const dim3 gk((a.max_kvec + KT - 1) / KT, a.n_jobs), gf((ns + FT - 1) / FT, a.n_jobs);
    const dim3 gm((a.max_mols + 127) / 128, a.n_jobs);
    const std::string n(name);
    if (n == "prep") {
        if (mixed) k_prep<float><<<gs, 128, 0, s>>>(a);
        else k_prep<double><<<gs, 128, 0, s>>>(a);
    } else if (n == "real") {
        if (mixed) k_real<float, 0><<<gr, RT, 0, s>>>(a);
        else k_real<double, 0><<<gr, RT, 0, s>>>(a);
    } else if (n == "ksk") {
        if (mixed) k_ksk<float, 0><<<gk, KT, ksk_smem<float>(a.max_kmax), s>>>(a);
        else k_ksk<double, 0><<<gk, KT, ksk_smem<double>(a.max_kmax), s>>>(a);
    } else if (n == "kforce") {
        if (mixed) k_kforce<float, 0><<<gf, FT, kforce_smem<float>(a.max_kmax), s>>>(a);
        else k_kforce<double, 0><<<gf, FT, kforce_smem<double>(a.max_kmax), s>>>(a);
    } else if (n == "combine") {
        k_combine<<<gm, 128, 0, s>>>(a);
    } else if (n == "lj") {
        k_lj<<<gm, 128, 0, s>>>(a);
    }
}

void init_force_kernel_attributes() {
    set_attrs<float>();
    set_attrs<double>();
}

void launch_eval_fp64(const EvalArgs &a, cudaStream_t s, unsigned long long *n) {
    if (a.n_jobs <= 0) return;
    if (!a.sr_only) launch_ewald<double>(a, s, n);
    launch_short_range(a, s, n);
}

void launch_eval_mixed(const EvalArgs &a, cudaStream_t s, unsigned long long *n) {
    if (a.n_jobs <= 0) return;
    if (!a.sr_only) launch_ewald<float>(a, s, n);
    launch_short_range(a, s, n);
}

// Reciprocal space only, on caller-supplied charge sites; site forces are
// accumulated into a.site_force (which the caller pre-loads).
void launch_kwald_only(const EvalArgs &a, bool mixed, cudaStream_t s, unsigned long long *n) {
    if (a.n_jobs <= 0) return;
    const int ns = 3 * a.max_mols;
    dim3 gs((ns + 127) / 128, a.n_jobs);
    dim3 gk((a.max_kvec + KT - 1) / KT, a.n_jobs);
    dim3 gf((ns + FT - 1) / FT, a.n_jobs);
    if (mixed) {
        k_prep<float><<<gs, 128, 0, s>>>(a);
        k_ksk<float, 0><<<gk, KT, ksk_smem<float>(a.max_kmax), s>>>(a);
        k_kforce<float, 0><<<gf, FT, kforce_smem<float>(a.max_kmax), s>>>(a);
    } else {
        k_prep<double><<<gs, 128, 0, s>>>(a);
        k_ksk<double, 0><<<gk, KT, ksk_smem<double>(a.max_kmax), s>>>(a);
        k_kforce<double, 0><<<gf, FT, kforce_smem<double>(a.max_kmax), s>>>(a);
    }
    if (n) *n += 3;
}

}  // namespace qtg
