/* CPU oracle for the qTIP4P/F force and ring-polymer propagation path.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C FP64 restatement of the reference's
 * algorithms (rayseashyn/qtip4pf_water), used as the checker in tests/ and as
 * the timed CPU baseline in bench.py. The product never links or calls it.
 * Parity with the reference's own compiled sources is pinned by the fixtures
 * in tests/golden. Compile with -ffp-contract=off (see oracle/Makefile).
 */
#include "qtip_oracle.h"

#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* ---- qTIP4P/F constants, restated from qtip4pfparams.h:41-133 -------------
 * The value of pi is the reference's truncated 3.14159265359
 * (qtip4pfparams.h:45); it enters theta_eq, sqrt(pi), 2pi/L and sin(k pi/P). */
#define QO_PI 3.14159265359

typedef struct {
    double angs2bohr, fs2au, K2au, mo, mh;
    double r_cut, r_cut_sq, r_skin, r_skin_sq;
    double gamma_vs, epslj, sigmalj, sigmalj6, sigmalj12, e_cut;
    double roheq, ar, ar2, ar3, ar4fac, Dr, theta_eq, ktheta, qo, qh;
} qo_consts;

static qo_consts K;
static int K_ready = 0;

static void consts_init(void) {
    if (K_ready) return;
    const double me = 9.10938356e-31, kb = 1.38064852e-23, Na = 6.0221409e23;
    const double eh = 4.3597447222071e-18, kcal2au = 1.5936e-3;
    const double mhgmol = 1.0080, mogmol = 15.9994, hbar_SI = 1.054571817e-34;
    K.angs2bohr = 1.0 / 0.529177210903;
    K.mo = 0.001 * mogmol / (Na * me);
    K.mh = 0.001 * mhgmol / (Na * me);
    K.K2au = kb / eh;
    double au2fs = hbar_SI * 1e15 / eh;
    K.fs2au = 1.0 / au2fs;
    K.r_cut = 9.0 * K.angs2bohr;
    K.r_cut_sq = K.r_cut * K.r_cut;
    K.r_skin = 1.30 * K.r_cut;
    K.r_skin_sq = K.r_skin * K.r_skin;
    K.gamma_vs = 0.73612;
    K.epslj = 0.1852 * kcal2au;
    K.sigmalj = 3.1589 * K.angs2bohr;
    K.sigmalj6 = pow(K.sigmalj, 6.0);
    K.sigmalj12 = K.sigmalj6 * K.sigmalj6;
    K.e_cut = 4.0 * K.epslj * (pow((K.sigmalj / K.r_cut), 12.0) - pow((K.sigmalj / K.r_cut), 6.0));
    K.roheq = 0.9419 * K.angs2bohr;
    K.ar = 2.287 / K.angs2bohr;
    K.ar2 = K.ar * K.ar;
    K.ar3 = K.ar2 * K.ar;
    K.ar4fac = 7.0 * K.ar3 * K.ar / 12.0;
    K.Dr = 116.09 * kcal2au;
    K.theta_eq = 107.4 * QO_PI / 180.0;
    K.ktheta = 87.85 * kcal2au;
    K.qo = -1.1128;
    K.qh = -0.5 * K.qo;
    K_ready = 1;
}

void qo_constants(double *out) {
    consts_init();
    double v[] = {K.angs2bohr, K.fs2au, K.K2au,   K.mo,       K.mh,     K.qo,   K.qh,
                  K.gamma_vs,  K.epslj, K.sigmalj, K.e_cut,   K.roheq,  K.ar,   K.Dr,
                  K.theta_eq,  K.ktheta, K.r_cut, K.r_skin,   QO_PI};
    memcpy(out, v, sizeof(v));
}

/* water.cpp:76-157 (box given directly) and forces.cpp:574-584 */
void qo_init(qo_sys *s, int n_mols, int n_beads, const double box_bohr[3], double temp_K,
             double dt_fs, double eps_ewald, double eps_sc) {
    consts_init();
    memset(s, 0, sizeof(*s));
    s->n_mols = n_mols;
    s->n_atoms = 3 * n_mols;
    s->n_dof = 9 * n_mols;
    s->n_beads = n_beads;
    for (int d = 0; d < 3; ++d) s->box[d] = box_bohr[d];
    s->vol = s->box[0] * s->box[1] * s->box[2];
    s->min_box = fmin(fmin(s->box[0], s->box[1]), s->box[2]);
    s->max_box = fmax(fmax(s->box[0], s->box[1]), s->box[2]);
    s->temp_K = temp_K;
    s->beta = 1.0 / (K.K2au * temp_K);
    s->beta_n = s->beta / n_beads;
    double omega_p = 1.0 / s->beta_n; /* hbar = 1 */
    s->omega_psq = omega_p * omega_p;
    s->pi_over_p = QO_PI / n_beads;
    s->dt = dt_fs * K.fs2au;
    s->halfdt = 0.5 * s->dt;
    s->eps_sc = eps_sc;
    double rho_ox = n_mols / s->vol;
    s->list_size = (int)round(4.0 * K.r_skin * K.r_skin * K.r_skin * n_mols * rho_ox);
    s->acc = sqrt(-log(eps_ewald));
    double rho = s->n_atoms / s->vol;
    s->k_pref = 2.0 * QO_PI / s->vol;
    double kappa = 2.6 * pow(rho / s->vol, 1.0 / 6.0);
    double rc = s->acc / kappa;
    if (rc > 0.5 * s->min_box) {
        rc = 0.5 * s->min_box;
        kappa = s->acc / rc;
    }
    s->kappa = kappa;
    s->rc_sq = rc * rc;
    double kc = 2.0 * s->acc * kappa;
    s->kc_sq = kc * kc;
    s->k_max = (int)(kc * s->max_box / (2.0 * QO_PI));
    s->ewald_pref = 2.0 * kappa / sqrt(QO_PI);
    s->r_cut = K.r_cut;
    s->r_cut_sq = K.r_cut_sq;
    s->r_skin = K.r_skin;
    s->r_skin_sq = K.r_skin_sq;
    s->mo = K.mo;
    s->mh = K.mh;
    s->qo = K.qo;
    s->qh = K.qh;
    s->gamma_m = K.gamma_vs;
}

void qo_default_charges(const qo_sys *s, double *charge) {
    for (int m = 0; m < s->n_mols; ++m) {
        charge[3 * m] = K.qo;
        charge[3 * m + 1] = K.qh;
        charge[3 * m + 2] = K.qh;
    }
}

void qo_default_masses(const qo_sys *s, double *mass) {
    for (int m = 0; m < s->n_mols; ++m)
        for (int d = 0; d < 3; ++d) {
            mass[9 * m + d] = K.mo;
            mass[9 * m + 3 + d] = K.mh;
            mass[9 * m + 6 + d] = K.mh;
        }
}

/* minimum image of one component, as neighbour.cpp:46 / forces.cpp:503 */
static inline double min_image(double x, double L) { return x - L * round(x / L); }

/* ---- Verlet list: neighbour.cpp:12-62 ------------------------------------ */
int qo_neighbour_list(const qo_sys *s, const double *pos, int *point, int *list, double *disp,
                      int bead) {
    const int N = s->n_mols;
    const double *q = pos + (size_t)bead * s->n_dof;
    int *row = point + (size_t)bead * N;
    int *lst = list + (size_t)bead * s->list_size;
    for (int k = 0; k < s->list_size; ++k) lst[k] = 0;
    for (int k = 0; k < 3 * N; ++k) disp[(size_t)bead * 3 * N + k] = 0.0;
    int n = 0, overflow = 0;
    for (int i = 0; i < N; ++i) {
        row[i] = n;
        for (int j = i + 1; j < N; ++j) {
            double dx = min_image(q[9 * i] - q[9 * j], s->box[0]);
            double dy = min_image(q[9 * i + 1] - q[9 * j + 1], s->box[1]);
            double dz = min_image(q[9 * i + 2] - q[9 * j + 2], s->box[2]);
            double r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < s->r_skin_sq) {
                if (n < s->list_size) lst[n] = j;
                else overflow = 1;
                ++n;
            }
        }
    }
    return overflow ? -1 : n;
}

/* ---- pair and intramolecular terms: forces.cpp:25-177 --------------------- */

/* Lennard-Jones O-O (forces.cpp:25-59): shifted energy, unshifted force. */
static double lj_pair(const double r[3], double r2, double *fi, double *fj) {
    double inv2 = 1.0 / r2;
    double s6 = inv2 * inv2 * inv2;
    double s12 = s6 * s6;
    s6 *= K.sigmalj6;
    s12 *= K.sigmalj12;
    double e = s12 - s6;
    double ff = e + s12;
    e *= 4.0 * K.epslj;
    e -= K.e_cut;
    ff *= 24.0 * K.epslj * inv2;
    for (int d = 0; d < 3; ++d) {
        fi[d] += ff * r[d];
        fj[d] -= ff * r[d];
    }
    return e;
}

/* quartic Morse O-H bond (forces.cpp:65-93); r = r_O - r_H. */
static double morse_bond(const double r[3], double rlen, double *fo, double *fh) {
    double inv = 1.0 / rlen;
    double x = rlen - K.roheq;
    double x2 = x * x, x3 = x2 * x, x4 = x2 * x2;
    double e = K.ar2 * x2 - K.ar3 * x3 + K.ar4fac * x4;
    e *= K.Dr;
    double g = 2.0 * K.ar2 * x - 3.0 * K.ar3 * x2 + 4.0 * K.ar4fac * x3;
    g *= K.Dr * inv;
    for (int d = 0; d < 3; ++d) {
        fo[d] -= g * r[d];
        fh[d] += g * r[d];
    }
    return e;
}

/* harmonic H-O-H angle (forces.cpp:96-138); a = r_O - r_H1, b = r_O - r_H2. */
static double hoh_angle(const double a[3], const double b[3], double la, double lb, double *fo,
                        double *f1, double *f2) {
    double dot = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
    double ia = 1.0 / la, ib = 1.0 / lb;
    double ia2 = ia * ia, ib2 = ib * ib, iab = ia * ib;
    double c = dot * iab;
    double dacos = 1.0 / sqrt(1.0 - c * c);
    double ca = dot * ia2 * iab;
    double cb = dot * ib2 * iab;
    double dth = acos(c) - K.theta_eq;
    double e = 0.5 * K.ktheta * dth * dth;
    double g = K.ktheta * dth * dacos;
    for (int d = 0; d < 3; ++d) {
        fo[d] += g * (iab * (a[d] + b[d]) - ca * a[d] - cb * b[d]);
        f1[d] -= g * (iab * b[d] - ca * a[d]);
        f2[d] -= g * (iab * a[d] - cb * b[d]);
    }
    return e;
}

/* real-space Ewald pair (forces.cpp:141-177); same-molecule pairs use erfc-1. */
static double ewald_real_pair(const double r[3], double r2, double qiqj, int same_mol,
                              double kappa, double *fi, double *fj) {
    double pref = 2.0 * kappa / sqrt(QO_PI);
    double rl = sqrt(r2);
    double inv = 1.0 / rl;
    double inv2 = inv * inv;
    double ec = erfc(kappa * rl);
    if (same_mol) ec -= 1.0;
    double e = qiqj * inv * ec;
    double ff = e + qiqj * pref * exp(-(kappa * kappa) * r2);
    ff *= inv2;
    for (int d = 0; d < 3; ++d) {
        fi[d] += ff * r[d];
        fj[d] -= ff * r[d];
    }
    return e;
}

/* ---- reciprocal-space Ewald: forces.cpp:180-448 ----------------------------
 * The k-vectors are those the reference visits: kx = 0..k_max (weight 2 for
 * kx > 0); (kx,0,0) only when 0 < |k|^2 < kc^2; every other combination
 * (kx, +-ky, +-kz) while |k|^2 <= kc^2, with the partial sums' early exits of
 * forces.cpp:286/333/380. S(k) = sum_i q_i exp(i k.r_i) is built from
 * per-dimension phase powers obtained by complex recursion (forces.cpp:233-240),
 * with the charge folded into the x factor (forces.cpp:241-244). */
typedef struct { int kx, ky, kz; double ksq, coef; } qo_kvec;

static int enumerate_k(const qo_sys *s, qo_kvec *out) {
    double bk[3];
    for (int d = 0; d < 3; ++d) bk[d] = 2.0 * QO_PI / s->box[d];
    double quart = 0.25 / (s->kappa * s->kappa);
    int n = 0, km = s->k_max;
#define QO_PUSH(a, b, c, KSQ)                                                        \
    do {                                                                             \
        if (out) {                                                                   \
            out[n].kx = (a); out[n].ky = (b); out[n].kz = (c); out[n].ksq = (KSQ);   \
            out[n].coef = s->k_pref * exp(-(KSQ) * quart) / (KSQ) * ((a) ? 2.0 : 1.0); \
        }                                                                            \
        ++n;                                                                         \
    } while (0)
    for (int kx = 0; kx <= km; ++kx) {
        double rx = bk[0] * kx;
        double ksq = rx * rx;
        if (ksq > 0.0 && ksq < s->kc_sq) QO_PUSH(kx, 0, 0, ksq);
        for (int kz = 1; kz <= km; ++kz) {
            double rz = bk[2] * kz;
            ksq = rx * rx + rz * rz;
            if (ksq > s->kc_sq) break;
            QO_PUSH(kx, 0, kz, ksq);
            QO_PUSH(kx, 0, -kz, ksq);
        }
        for (int ky = 1; ky <= km; ++ky) {
            double ry = bk[1] * ky;
            ksq = rx * rx + ry * ry;
            if (ksq > s->kc_sq) break;
            QO_PUSH(kx, ky, 0, ksq);
            QO_PUSH(kx, -ky, 0, ksq);
            for (int kz = 1; kz <= km; ++kz) {
                double rz = bk[2] * kz;
                ksq = rx * rx + ry * ry + rz * rz;
                if (ksq > s->kc_sq) break;
                QO_PUSH(kx, ky, kz, ksq);
                QO_PUSH(kx, ky, -kz, ksq);
                QO_PUSH(kx, -ky, kz, ksq);
                QO_PUSH(kx, -ky, -kz, ksq);
            }
        }
    }
#undef QO_PUSH
    return n;
}

int qo_count_kvectors(const qo_sys *s) { return enumerate_k(s, NULL); }

double qo_kwald(const qo_sys *s, const double *sites_all, double *f_all, const double *charge,
                int bead) {
    const int ns = s->n_atoms, km = s->k_max, w = km + 1;
    const double *r = sites_all + (size_t)bead * s->n_dof;
    double *f = f_all + (size_t)bead * s->n_dof;
    double bk[3];
    for (int d = 0; d < 3; ++d) bk[d] = 2.0 * QO_PI / s->box[d];
    /* phase powers: ph[(site*3 + d)*w + m] = exp(i m bk_d r_d), x scaled by q */
    double *pc = (double *)malloc(sizeof(double) * (size_t)ns * 3 * w);
    double *ps = (double *)malloc(sizeof(double) * (size_t)ns * 3 * w);
    for (int i = 0; i < ns; ++i) {
        for (int d = 0; d < 3; ++d) {
            double *c = pc + ((size_t)i * 3 + d) * w, *sn = ps + ((size_t)i * 3 + d) * w;
            double th = bk[d] * r[3 * i + d];
            double c1 = cos(th), s1 = sin(th);
            c[0] = 1.0;
            sn[0] = 0.0;
            for (int m = 1; m <= km; ++m) {
                c[m] = c1 * c[m - 1] - s1 * sn[m - 1];
                sn[m] = s1 * c[m - 1] + c1 * sn[m - 1];
            }
        }
        for (int m = 0; m <= km; ++m) {
            pc[((size_t)i * 3) * w + m] *= charge[i];
            ps[((size_t)i * 3) * w + m] *= charge[i];
        }
    }
    int nk = enumerate_k(s, NULL);
    qo_kvec *kv = (qo_kvec *)malloc(sizeof(qo_kvec) * (size_t)(nk > 0 ? nk : 1));
    enumerate_k(s, kv);
    double *er = (double *)malloc(sizeof(double) * (size_t)ns);
    double *ei = (double *)malloc(sizeof(double) * (size_t)ns);
    double energy = 0.0;
    for (int t = 0; t < nk; ++t) {
        int ky = kv[t].ky, kz = kv[t].kz;
        int ay = ky < 0 ? -ky : ky, az = kz < 0 ? -kz : kz;
        double sy = ky < 0 ? -1.0 : 1.0, sz = kz < 0 ? -1.0 : 1.0;
        double sr = 0.0, si = 0.0;
        for (int i = 0; i < ns; ++i) {
            double xr = pc[((size_t)i * 3) * w + kv[t].kx], xi = ps[((size_t)i * 3) * w + kv[t].kx];
            double yr = pc[((size_t)i * 3 + 1) * w + ay], yi = sy * ps[((size_t)i * 3 + 1) * w + ay];
            double zr = pc[((size_t)i * 3 + 2) * w + az], zi = sz * ps[((size_t)i * 3 + 2) * w + az];
            double ar = xr * yr - xi * yi, ai = xr * yi + xi * yr;
            er[i] = ar * zr - ai * zi;
            ei[i] = ar * zi + ai * zr;
            sr += er[i];
            si += ei[i];
        }
        double c = kv[t].coef;
        energy += c * (sr * sr + si * si);
        double gx = 2.0 * c * bk[0] * kv[t].kx, gy = 2.0 * c * bk[1] * ky, gz = 2.0 * c * bk[2] * kz;
        for (int i = 0; i < ns; ++i) {
            /* q_i (Sr sin - Si cos); the charge is already inside er/ei */
            double tq = ei[i] * sr - er[i] * si;
            f[3 * i] += gx * tq;
            f[3 * i + 1] += gy * tq;
            f[3 * i + 2] += gz * tq;
        }
    }
    free(kv);
    free(er);
    free(ei);
    free(pc);
    free(ps);
    return energy;
}

/* ---- one configuration: forces.cpp:468-630 -------------------------------- */
/* ---- tabulated pair corrections: forces.cpp:452-466, :634-691 ---------------
 * The reference's spline is boost::math::cubic_b_spline (not installed here):
 * restated as the clamped uniform cubic B-spline interpolant that type
 * documents. s(x) = sum_{j=-1}^{n} c_j B(t - j), t = (x - start)/step, B the
 * centred cubic B-spline; (c_{i-1} + 4 c_i + c_{i+1})/6 = y_i at the knots and
 * (c_1 - c_{-1})/(2 step), (c_n - c_{n-2})/(2 step) the end slopes. */
int qo_spline_build(const double *y, int n, double step, double dl, double dr, double *c) {
    if (n < 5 || !(step > 0)) return 0;
    if (isnan(dl)) dl = (-25.0 * y[0] + 48.0 * y[1] - 36.0 * y[2] + 16.0 * y[3] - 3.0 * y[4]) / (12.0 * step);
    if (isnan(dr))
        dr = (25.0 * y[n - 1] - 48.0 * y[n - 2] + 36.0 * y[n - 3] - 16.0 * y[n - 4] + 3.0 * y[n - 5]) / (12.0 * step);
    /* tridiagonal system for x_i = c_i, i = 0..n-1: rows 1..n-2 are (1, 4, 1) = 6 y_i,
     * row 0 is 4 x_0 + 2 x_1 = 6 y_0 + 2 step dl, row n-1 is 2 x_{n-2} + 4 x_{n-1} =
     * 6 y_{n-1} - 2 step dr; forward elimination into (d, r), back substitution */
    double *d = (double *)malloc(sizeof(double) * (size_t)n);
    double *r = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        const double lo = i == 0 ? 0.0 : (i == n - 1 ? 2.0 : 1.0);
        const double up_prev = i == 1 ? 2.0 : 1.0;
        double rhs = 6.0 * y[i];
        if (i == 0) rhs += 2.0 * step * dl;
        if (i == n - 1) rhs -= 2.0 * step * dr;
        if (i == 0) {
            d[0] = 4.0;
            r[0] = rhs;
        } else {
            const double w = lo / d[i - 1];
            d[i] = 4.0 - w * up_prev;
            r[i] = rhs - w * r[i - 1];
        }
    }
    double *x = c + 1;
    x[n - 1] = r[n - 1] / d[n - 1];
    for (int i = n - 2; i >= 0; --i) x[i] = (r[i] - (i == 0 ? 2.0 : 1.0) * x[i + 1]) / d[i];
    c[0] = x[1] - 2.0 * step * dl;
    c[n + 1] = x[n - 2] + 2.0 * step * dr;
    free(d);
    free(r);
    return 1;
}

/* the centred cubic B-spline */
static double bspl3(double t) {
    t = fabs(t);
    if (t >= 2.0) return 0.0;
    if (t >= 1.0) return (2.0 - t) * (2.0 - t) * (2.0 - t) / 6.0;
    return (4.0 - 6.0 * t * t + 3.0 * t * t * t) / 6.0;
}
static double bspl3_prime(double t) {
    const double a = fabs(t), sg = t < 0.0 ? -1.0 : 1.0;
    if (a >= 2.0) return 0.0;
    if (a >= 1.0) return -0.5 * sg * (2.0 - a) * (2.0 - a);
    return sg * (-2.0 * a + 1.5 * a * a);
}

double qo_spline_eval(const double *c, int n, double start, double step, double x, double *deriv) {
    const double t = (x - start) / step;
    int i0 = (int)floor(t);
    if (i0 < 0) i0 = 0;
    if (i0 > n - 2) i0 = n - 2;
    double v = 0.0, dv = 0.0;
    for (int j = i0 - 1; j <= i0 + 2; ++j) {
        v += c[j + 1] * bspl3(t - j);
        dv += c[j + 1] * bspl3_prime(t - j);
    }
    if (deriv) *deriv = dv / step;
    return v;
}

void qo_set_splines(qo_sys *s, const qo_splines *spl) { s->spl = spl; }

/* get_forces_wspline's pair loop (forces.cpp:644-688): every atom pair i < j,
 * minimum image, the type's spline inside its cutoff, get_spline's force
 * (forces.cpp:454-463: F_i -= s'(r)/r r_ij, F_j += s'(r)/r r_ij) */
static double spline_pairs(const qo_sys *s, const double *q, double *f) {
    const int na = s->n_atoms;
    double energy = 0.0;
    for (int i = 0; i < na; ++i)
        for (int j = i + 1; j < na; ++j) {
            double r[3];
            for (int d = 0; d < 3; ++d) {
                r[d] = q[3 * i + d] - q[3 * j + d];
                r[d] -= s->box[d] * round(r[d] / s->box[d]);
            }
            const double rsq = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            const int t = (i % 3 == 0 ? 0 : 1) + (j % 3 == 0 ? 0 : 1);
            const qo_spline *sp = &s->spl->t[t];
            if (!sp->c || !(rsq < sp->cut_sq)) continue;
            const double rij = sqrt(rsq);
            double dv;
            energy += qo_spline_eval(sp->c, sp->n, sp->start, sp->step, rij, &dv);
            const double fp = dv / rij;
            for (int d = 0; d < 3; ++d) {
                f[3 * i + d] -= fp * r[d];
                f[3 * j + d] += fp * r[d];
            }
        }
    return energy;
}

double qo_get_forces(const qo_sys *s, const double *pos, double *f_all, const double *charge,
                     const int *point, const int *list, int bead) {
    const int N = s->n_mols, ns = s->n_atoms, nd = s->n_dof;
    const double *q = pos + (size_t)bead * nd;
    double *f = f_all + (size_t)bead * nd;
    const int *row = point + (size_t)bead * N;
    const int *lst = list + (size_t)bead * s->list_size;
    double energy = 0.0;
    for (int k = 0; k < nd; ++k) f[k] = 0.0;
    /* LJ over the Verlet list (forces.cpp:489-515) */
    for (int i = 0; i < N - 1; ++i) {
        for (int n = row[i]; n < row[i + 1]; ++n) {
            int j = lst[n];
            double r[3];
            for (int d = 0; d < 3; ++d) r[d] = min_image(q[9 * i + d] - q[9 * j + d], s->box[d]);
            double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            if (r2 < s->r_cut_sq) energy += lj_pair(r, r2, f + 9 * i, f + 9 * j);
        }
    }
    /* intramolecular (forces.cpp:519-554) */
    for (int i = 0; i < N; ++i) {
        double a[3], b[3];
        for (int d = 0; d < 3; ++d) a[d] = min_image(q[9 * i + d] - q[9 * i + 3 + d], s->box[d]);
        double la = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
        energy += morse_bond(a, la, f + 9 * i, f + 9 * i + 3);
        for (int d = 0; d < 3; ++d) b[d] = min_image(q[9 * i + d] - q[9 * i + 6 + d], s->box[d]);
        double lb = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        energy += morse_bond(b, lb, f + 9 * i, f + 9 * i + 6);
        energy += hoh_angle(a, b, la, lb, f + 9 * i, f + 9 * i + 3, f + 9 * i + 6);
    }
    /* charge sites: M replaces O (forces.cpp:558-564) */
    double *site = (double *)malloc(sizeof(double) * (size_t)nd);
    double *fs = (double *)calloc((size_t)nd, sizeof(double));
    const double g = K.gamma_vs;
    for (int i = 0; i < N; ++i)
        for (int d = 0; d < 3; ++d) {
            site[9 * i + d] = g * q[9 * i + d] + 0.5 * (1.0 - g) * (q[9 * i + 3 + d] + q[9 * i + 6 + d]);
            site[9 * i + 3 + d] = q[9 * i + 3 + d];
            site[9 * i + 6 + d] = q[9 * i + 6 + d];
        }
    /* real-space Ewald over all site pairs (forces.cpp:589-608) */
    for (int i = 0; i < ns - 1; ++i)
        for (int j = i + 1; j < ns; ++j) {
            double r[3];
            for (int d = 0; d < 3; ++d) r[d] = min_image(site[3 * i + d] - site[3 * j + d], s->box[d]);
            double r2 = r[0] * r[0] + r[1] * r[1] + r[2] * r[2];
            if (r2 < s->rc_sq)
                energy += ewald_real_pair(r, r2, charge[i] * charge[j], i / 3 == j / 3, s->kappa,
                                          fs + 3 * i, fs + 3 * j);
        }
    /* reciprocal space (forces.cpp:611) */
    energy += qo_kwald(s, site, fs, charge, 0);
    /* M-site chain rule (forces.cpp:613-619) */
    for (int i = 0; i < N; ++i)
        for (int d = 0; d < 3; ++d) {
            f[9 * i + d] += g * fs[9 * i + d];
            f[9 * i + 3 + d] += fs[9 * i + 3 + d] + 0.5 * (1.0 - g) * fs[9 * i + d];
            f[9 * i + 6 + d] += fs[9 * i + 6 + d] + 0.5 * (1.0 - g) * fs[9 * i + d];
        }
    /* self term (forces.cpp:622-624) */
    for (int i = 0; i < ns; ++i) energy -= 0.5 * s->ewald_pref * charge[i] * charge[i];
    free(site);
    free(fs);
    if (s->spl) energy += spline_pairs(s, q, f);
    return energy;
}

/* ---- Suzuki-Chin assembly: forces.cpp:698-789 ------------------------------ */
double qo_force_eval_sc(const qo_sys *s, const double *pos, double *f, const double *charge,
                        const double *mass, const int *point, const int *list, double *sc_pot,
                        double *fphys) {
    const int P = s->n_beads, nd = s->n_dof;
    double tot = 0.0, vop = 0.0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : tot, vop)
    for (int b = 0; b < P; ++b) {
        double e = qo_get_forces(s, pos, fphys, charge, point, list, b);
        const double *fp = fphys + (size_t)b * nd;
        double *fo = f + (size_t)b * nd;
        if (b % 2 == 0) {
            tot += 2.0 * e;
            for (int i = 0; i < nd; ++i) fo[i] = 2.0 * fp[i] / 3.0;
            vop += e;
        } else {
            tot += 4.0 * e;
            double fsq = 0.0;
            for (int i = 0; i < nd; ++i) fsq += fp[i] * fp[i] / mass[i];
            fsq /= 3.0 * s->omega_psq;
            tot += fsq;
            double dl = 0.0;
            for (int i = 0; i < nd; ++i) {
                double t = fp[i] / mass[i];
                dl += t * t;
            }
            dl /= s->n_atoms * P;
            dl = 1.0 / sqrt(dl);
            double scl = s->eps_sc * dl;
            double fscale = 1.0 / (9.0 * s->omega_psq * scl);
            /* displaced copies of this bead only, stored as bead 0 of a scratch
             * system so that qo_get_forces indexes them at offset 0 */
            double *qp = (double *)malloc(sizeof(double) * (size_t)nd * 4);
            double *qm = qp + nd, *fpl = qp + 2 * nd, *fmi = qp + 3 * nd;
            const double *qb = pos + (size_t)b * nd;
            for (int i = 0; i < nd; ++i) {
                double dq = scl * fp[i] / mass[i];
                qp[i] = qb[i] + dq;
                qm[i] = qb[i] - dq;
            }
            const int *pt = point + (size_t)b * s->n_mols;
            const int *ls = list + (size_t)b * s->list_size;
            /* rebase the CSR pointers: qo_get_forces reads bead 0 of the arrays it gets */
            qo_get_forces(s, qp, fpl, charge, pt, ls, 0);
            qo_get_forces(s, qm, fmi, charge, pt, ls, 0);
            for (int i = 0; i < nd; ++i) {
                fo[i] = 4.0 * fp[i] / 3.0;
                fo[i] -= fscale * (fpl[i] - fmi[i]);
            }
            free(qp);
        }
    }
    *sc_pot = 2.0 * vop / P;
    return tot / 3.0;
}

double qo_force_eval_trotter(const qo_sys *s, const double *pos, double *f, const double *charge,
                             const int *point, const int *list, double *pot_est) {
    const int P = s->n_beads;
    double tot = 0.0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : tot)
    for (int b = 0; b < P; ++b) tot += qo_get_forces(s, pos, f, charge, point, list, b);
    *pot_est = tot / P;
    return tot;
}

/* ---- normal-mode transform: fourier.cpp:12-69 ------------------------------
 * Forward: y_0 = sqrt(1/P) sum_b x_b; y_k = sqrt(2/P) Re X_k (1 <= k < P/2);
 * y_{P-k} = sqrt(2/P) Im X_k with X_k = sum_b x_b exp(-2 pi i b k / P);
 * y_{P/2} = sqrt(1/P) X_{P/2} for even P. Backward is the transpose. */
static void dft_twiddle(int a, int b, int n, double *c, double *sn) {
    const double two_pi = 6.283185307179586476925286766559;
    long m = ((long)a * (long)b) % n;
    double ang = two_pi * (double)m / (double)n;
    *c = cos(ang);
    *sn = sin(ang);
}

void qo_ftransform(const qo_sys *s, double *a, int length, int forwards) {
    const int P = s->n_beads;
    double sc = sqrt(1.0 / P), sc2 = sqrt(2.0 / P), r2 = sqrt(2.0);
    double *x = (double *)malloc(sizeof(double) * (size_t)P);
    double *y = (double *)malloc(sizeof(double) * (size_t)P);
    for (int col = 0; col < length; ++col) {
        for (int b = 0; b < P; ++b) x[b] = a[(size_t)b * length + col];
        if (forwards) {
            for (int k = 0; k <= P / 2; ++k) {
                double re = 0.0, im = 0.0;
                for (int b = 0; b < P; ++b) {
                    double c, sn;
                    dft_twiddle(b, k, P, &c, &sn);
                    re += x[b] * c;
                    im -= x[b] * sn;
                }
                y[k] = re;
                if (k > 0 && 2 * k != P) y[P - k] = im;
            }
            a[col] = sc * y[0];
            for (int k = 1; k < P; ++k) a[(size_t)k * length + col] = sc2 * y[k];
            if (P % 2 == 0) a[(size_t)(P / 2) * length + col] /= r2;
        } else {
            for (int k = 1; k < P; ++k) x[k] /= r2;
            if (P % 2 == 0) x[P / 2] *= r2;
            for (int b = 0; b < P; ++b) {
                double acc = x[0];
                for (int k = 1; 2 * k < P; ++k) {
                    double c, sn;
                    dft_twiddle(b, k, P, &c, &sn);
                    acc += 2.0 * (x[k] * c - x[P - k] * sn);
                }
                if (P % 2 == 0) acc += x[P / 2] * ((b % 2 == 0) ? 1.0 : -1.0);
                y[b] = acc;
            }
            for (int b = 0; b < P; ++b) a[(size_t)b * length + col] = sc * y[b];
        }
    }
    free(x);
    free(y);
}

/* ---- PILE-G: thermostat.cpp:64-133 ----------------------------------------- */
double qo_pile_g(const qo_sys *s, double *p, const double *mass, const double *noise) {
    const int P = s->n_beads, nd = s->n_dof;
    double heat = 0.0, ke0 = 0.0;
    for (int i = 0; i < nd; ++i) ke0 += 0.5 * p[i] * p[i] / mass[i];
    heat += ke0;
    double R = noise[0], g2 = noise[1];
    double alpha = sqrt((R * R + g2) / (2.0 * s->beta_n * ke0));
    for (int i = 0; i < nd; ++i) p[i] *= alpha;
    for (int i = 0; i < nd; ++i) heat -= 0.5 * p[i] * p[i] / mass[i];
    const double *xi = noise + 2;
    double pref = 4.0 / s->beta_n;
    for (int k = 1; k < P; ++k) {
        double *pk = p + (size_t)k * nd;
        for (int i = 0; i < nd; ++i) heat += 0.5 * pk[i] * pk[i] / mass[i];
        double gk = pref * sin(k * QO_PI / P);
        double c1 = exp(-s->dt * gk);
        double c2 = sqrt(1.0 - c1 * c1);
        for (int i = 0; i < nd; ++i)
            pk[i] = c1 * pk[i] + sqrt(mass[i] / s->beta_n) * c2 * xi[(size_t)(k - 1) * nd + i];
        for (int i = 0; i < nd; ++i) heat -= 0.5 * pk[i] * pk[i] / mass[i];
    }
    return heat;
}

/* ---- Bussi global rescale: thermostat.cpp:12-60 ----------------------------
 * The first n_dof momenta (the reference's classical system) are rescaled by
 * alpha = sqrt((R^2 + g2) / (beta sum p^2 / m)), m the atom's mass; returns the
 * heat (kinetic energy before minus after). noise = [R, g2]. */
double qo_bussi(const qo_sys *s, double *p, const double *mass, const double *noise) {
    const int nd = s->n_dof;
    double heat = 0.0, p2 = 0.0;
    for (int i = 0; i < nd; ++i) heat += 0.5 * p[i] * p[i] / mass[3 * (i / 3)];
    for (int i = 0; i < nd; ++i) p2 += p[i] * p[i] / mass[3 * (i / 3)];
    const double R = noise[0], g2 = noise[1];
    const double alpha = sqrt((R * R + g2) / (s->beta * p2));
    for (int i = 0; i < nd; ++i) p[i] *= alpha;
    for (int i = 0; i < nd; ++i) heat -= 0.5 * p[i] * p[i] / mass[3 * (i / 3)];
    return heat;
}

/* ---- estimators: path_integrals.cpp:10-81 ---------------------------------- */
double qo_get_kcv(const qo_sys *s, const double *q, const double *f) {
    const int P = s->n_beads, nd = s->n_dof;
    double *qc = (double *)malloc(sizeof(double) * (size_t)nd);
    for (int j = 0; j < nd; ++j) {
        double acc = 0.0;
        for (int b = 0; b < P; ++b) acc += q[(size_t)b * nd + j];
        qc[j] = acc / (double)(float)P;
    }
    double tq = 0.0;
    for (int b = 0; b < P; b += 2)
        for (int j = 0; j < nd; ++j) tq -= (q[(size_t)b * nd + j] - qc[j]) * f[(size_t)b * nd + j];
    tq /= P;
    free(qc);
    return 0.5 * nd / s->beta + tq;
}

double qo_get_conserved(const qo_sys *s, double *q, double *p, const double *mass, double energy) {
    const int P = s->n_beads, nd = s->n_dof;
    qo_ftransform(s, q, nd, 1);
    qo_ftransform(s, p, nd, 1);
    double kin = 0.0, spring = 0.0;
    double pref = 2.0 / s->beta_n;
    for (int k = 0; k < P; ++k) {
        double sn = sin(k * (QO_PI / P));
        double w2 = pref * pref * sn * sn;
        double q2 = 0.0;
        for (int j = 0; j < nd; ++j) {
            double pj = p[(size_t)k * nd + j], qj = q[(size_t)k * nd + j];
            kin += 0.5 * pj * pj / mass[j];
            q2 += mass[j] * qj * qj;
        }
        spring += q2 * (0.5 * w2);
    }
    qo_ftransform(s, q, nd, 0);
    qo_ftransform(s, p, nd, 0);
    return energy + kin + spring;
}

/* ---- the Verlet-list skin test of update.cpp:95-123 / :356-385 ------------- */
static int needs_rebuild(const qo_sys *s, const double *disp, int bead) {
    const int N = s->n_mols;
    const double *dsp = disp + (size_t)bead * 3 * N;
    double m1 = 0.0, m2 = 0.0;
    for (int i = 0; i < N; ++i) {
        double d2 = dsp[3 * i] * dsp[3 * i] + dsp[3 * i + 1] * dsp[3 * i + 1] + dsp[3 * i + 2] * dsp[3 * i + 2];
        if (d2 > m1) {
            m2 = m1;
            m1 = d2;
        } else if (d2 > m2) {
            m2 = d2;
        }
    }
    return sqrt(m1) + sqrt(m2) > s->r_skin - s->r_cut;
}

/* ---- classical velocity Verlet: update.cpp:78-137 --------------------------- */
double qo_update_class(const qo_sys *s, double *q, double *p, const double *mass, double *f,
                       const double *charge, int *point, int *list, double *disp) {
    const int na = s->n_atoms;
    for (int i = 0; i < na; ++i)
        for (int d = 0; d < 3; ++d) {
            p[3 * i + d] += s->halfdt * f[3 * i + d];
            q[3 * i + d] += p[3 * i + d] * s->dt / mass[3 * i + d];
            if (i % 3 == 0) disp[i + d] += p[3 * i + d] * s->dt / mass[3 * i + d];
        }
    if (needs_rebuild(s, disp, 0)) qo_neighbour_list(s, q, point, list, disp, 0);
    double e = qo_get_forces(s, q, f, charge, point, list, 0);
    for (int i = 0; i < 3 * na; ++i) p[i] += s->halfdt * f[i];
    return e;
}

/* ---- ring-polymer step: update.cpp:271-401 ----------------------------------
 * B(dt/2) -> NM forward (q, p, disp) -> sqrt-Cayley A(dt/2) -> O -> A(dt/2)
 * -> NM back -> per-bead list check -> forces -> B(dt/2). */
static void cayley_half(const qo_sys *s, double *q, double *p, const double *mass, double *disp) {
    const int P = s->n_beads, na = s->n_atoms, nd = s->n_dof, N = s->n_mols;
    double pref = 2.0 / s->beta_n, pref2 = pref * pref;
    for (int k = 0; k < P; ++k) {
        double sn = sin(k * s->pi_over_p);
        double w2 = pref2 * sn * sn;
        double sc = 1.0 / sqrt(1.0 + 0.25 * w2 * s->dt * s->dt);
        for (int i = 0; i < na; ++i)
            for (int d = 0; d < 3; ++d) {
                size_t at = (size_t)k * nd + 3 * i + d;
                double m = mass[3 * i];
                double qn = s->halfdt * p[at] / m + q[at];
                qn *= sc;
                p[at] = p[at] - s->halfdt * w2 * q[at] * m;
                p[at] *= sc;
                if (i % 3 == 0) disp[(size_t)k * 3 * N + i + d] += qn - q[at];
                q[at] = qn;
            }
    }
}

double qo_update_pimd(const qo_sys *s, double *q, double *p, const double *mass, double *f,
                      double *fphys, const double *charge, int *point, int *list, double *disp,
                      int is_nvt, const double *noise, double *heat, double *pot_est, int trotter) {
    const int P = s->n_beads, nd = s->n_dof, N = s->n_mols;
    for (size_t i = 0; i < (size_t)P * nd; ++i) p[i] += s->halfdt * f[i];
    qo_ftransform(s, q, nd, 1);
    qo_ftransform(s, p, nd, 1);
    qo_ftransform(s, disp, 3 * N, 1);
    cayley_half(s, q, p, mass, disp);
    if (is_nvt) *heat -= qo_pile_g(s, p, mass, noise);
    cayley_half(s, q, p, mass, disp);
    qo_ftransform(s, q, nd, 0);
    qo_ftransform(s, p, nd, 0);
    qo_ftransform(s, disp, 3 * N, 0);
    for (int b = 0; b < P; ++b)
        if (needs_rebuild(s, disp, b)) qo_neighbour_list(s, q, point, list, disp, b);
    double e;
    if (trotter) {
        e = qo_force_eval_trotter(s, q, f, charge, point, list, pot_est);
        memcpy(fphys, f, sizeof(double) * (size_t)P * nd);
    } else {
        e = qo_force_eval_sc(s, q, f, charge, mass, point, list, pot_est, fphys);
    }
    for (size_t i = 0; i < (size_t)P * nd; ++i) p[i] += s->halfdt * f[i];
    return e;
}

/* ==== the device stepper's propagation (new paths, no reference counterpart) ====
 * The library's device-resident stepper follows update.cpp:271-401 (B, NM
 * forward, sqrt-Cayley A, O, A, NM back, list check, forces, B) but draws its
 * thermostat noise from a counter-based generator keyed by (seed, system, step,
 * mode, dof) instead of std::mt19937, and adds two thermostat variants and a
 * centroid constraint. This section restates that propagation on the CPU so
 * that a thermostatted device trajectory can be followed step for step.
 *
 * Generator: Philox4x32-10 (Salmon, Moraes, Dror & Shaw, "Parallel random
 * numbers: as easy as 1, 2, 3", SC'11): ten rounds of
 *   (c0, c1, c2, c3) <- (hi(M1 c2) ^ c1 ^ k0, lo(M1 c2), hi(M0 c0) ^ c3 ^ k1, lo(M0 c0))
 * with M0 = 0xD2511F53, M1 = 0xCD9E8D57 and the key bumped by the Weyl
 * constants (0x9E3779B9, 0xBB67AE85) after every round. */
void qo_philox4x32_10(const uint32_t ctr[4], uint32_t k0, uint32_t k1, uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    for (int r = 0; r < 10; ++r) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c0, p1 = (uint64_t)0xCD9E8D57u * c2;
        const uint32_t n0 = (uint32_t)(p1 >> 32) ^ c1 ^ k0, n2 = (uint32_t)(p0 >> 32) ^ c3 ^ k1;
        c0 = n0;
        c1 = (uint32_t)p1;
        c2 = n2;
        c3 = (uint32_t)p0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0;
    out[1] = c1;
    out[2] = c2;
    out[3] = c3;
}

/* stream keys: the low and high seed words mixed with the system index and the
 * stream tag (1 normal-mode noise, 2 centroid normal, 3 centroid gamma) */
static void stepper_key(uint64_t seed, int sys, uint32_t tag, uint32_t *k0, uint32_t *k1) {
    *k0 = (uint32_t)seed ^ ((uint32_t)sys * 0x85EBCA6Bu);
    *k1 = (uint32_t)(seed >> 32) ^ (tag * 0xC2B2AE35u);
}

static void stepper_block(uint32_t c0, uint32_t c1, uint64_t st, uint32_t k0, uint32_t k1, uint32_t out[4]) {
    const uint32_t ctr[4] = {c0, c1, (uint32_t)st, (uint32_t)(st >> 32)};
    qo_philox4x32_10(ctr, k0, k1, out);
}

/* uniform in (0, 1) from two words, 53 significant bits */
static double u01_from(uint32_t a, uint32_t b) {
    uint64_t x = ((uint64_t)a << 21) ^ (uint64_t)(b >> 11);
    x &= ((1ull << 53) - 1ull);
    return ((double)x + 0.5) * (1.0 / 9007199254740992.0);
}

/* thermostat noise of the normal modes: Box-Muller in single precision from the
 * block's first two words (24-bit uniforms at cell centres); each operation is
 * rounded to float here as on the device (libm in double, then rounded: the
 * device's single-precision functions differ from this by an ulp or two) */
double qo_stepper_normal_f32(uint32_t v0, uint32_t v1) {
    const float u1 = ((float)(v0 >> 8) + 0.5f) * (1.0f / 16777216.0f);
    const float u2 = ((float)(v1 >> 8) + 0.5f) * (1.0f / 16777216.0f);
    const float c = (float)cos(2.0 * 3.14159265358979323846 * (double)u2);
    const float l = (float)log((double)u1);
    const float r = sqrtf(-2.0f * l);
    return (double)(r * c);
}

/* Box-Muller in double precision: the first of the pair */
static double normal2_x(const uint32_t v[4]) {
    const double u1 = u01_from(v[0], v[1]), u2 = u01_from(v[2], v[3]);
    return sqrt(-2.0 * log(u1)) * cos(2.0 * 3.14159265358979323846 * u2);
}

/* Gamma(shape), shape >= 1, by Marsaglia & Tsang ("A simple method for
 * generating gamma variables", ACM TOMS 26, 2000): candidate `it` takes its
 * normal from block (2 it, 0) and its uniform from block (2 it + 1, 0); the
 * first accepted of at most 64 candidates is returned (*ok = 0 if none is). */
static double stepper_gamma(double shape, uint64_t seed, int sys, uint64_t st, int *ok) {
    const double d = shape - 1.0 / 3.0, cc = 1.0 / sqrt(9.0 * d);
    uint32_t k0, k1, v[4];
    stepper_key(seed, sys, 3u, &k0, &k1);
    for (uint32_t it = 0; it < 64; ++it) {
        stepper_block(2 * it, 0u, st, k0, k1, v);
        const double x = normal2_x(v);
        double w = 1.0 + cc * x;
        if (w <= 0.0) continue;
        w = w * w * w;
        stepper_block(2 * it + 1, 0u, st, k0, k1, v);
        const double u = u01_from(v[0], v[1]);
        if (u < 1.0 - 0.0331 * x * x * x * x || log(u) < 0.5 * x * x + d * (1.0 - w + log(w))) return d * w;
    }
    *ok = 0;
    return shape;
}

int qo_stepper_centroid_draw(unsigned long long seed, int sys, int n_dof, unsigned long long st, double *R,
                             double *g2) {
    uint32_t k0, k1, v[4];
    stepper_key(seed, sys, 2u, &k0, &k1);
    stepper_block(0u, 0u, st, k0, k1, v);
    *R = normal2_x(v);
    int ok = 1;
    *g2 = 2.0 * stepper_gamma(0.5 * (n_dof - 1), seed, sys, st, &ok);
    return ok;
}

/* One device-stepper step (update.cpp:271-401 with the changes above):
 *  - PILE-G (thermostat 1): centroid p *= alpha, alpha^2 = (R^2 + g2) /
 *    (2 beta_n K0), K0 the centroid normal-mode kinetic energy at the O step and
 *    (R, g2) drawn at counter step - 1; modes k >= 1 as thermostat.cpp:119-133
 *    with xi from block (dof, k) at counter step;
 *  - PILE-L (thermostat 2): as PILE-G for k >= 1; the centroid is a Langevin
 *    mode too, c1 = exp(-dt / tau0), xi from block (dof, 0);
 *  - centroid_fixed: the centroid normal-mode momentum is zeroed before the
 *    free ring-polymer step and not thermostatted, so the centroid stays put;
 *    cf_acc (per dof, may be NULL) accumulates (1/P) sum_b fphys_b after the
 *    forces, st->cf_samples counts the steps.
 * The counter advances by one per step (the device's starts at 1 after its
 * first force evaluation). Returns the force assembly's total energy. */
double qo_stepper_step(const qo_sys *s, qo_stepper *st, double *q, double *p, const double *mass, double *f,
                       double *fphys, const double *charge, int *point, int *list, double *disp, int is_nvt,
                       double *cf_acc, double *pot_est) {
    const int P = s->n_beads, nd = s->n_dof, N = s->n_mols;
    for (size_t i = 0; i < (size_t)P * nd; ++i) p[i] += s->halfdt * f[i];
    qo_ftransform(s, q, nd, 1);
    qo_ftransform(s, p, nd, 1);
    qo_ftransform(s, disp, 3 * N, 1);
    if (st->centroid_fixed)
        for (int i = 0; i < nd; ++i) p[i] = 0.0;
    cayley_half(s, q, p, mass, disp);
    if (is_nvt && st->thermostat != 0) {
        uint32_t k0, k1, v[4];
        stepper_key(st->seed, st->sys, 1u, &k0, &k1);
        const double pref = 4.0 / s->beta_n;
        for (int k = 0; k < P; ++k) {
            double *pk = p + (size_t)k * nd;
            if (k == 0 && st->centroid_fixed) continue;
            if (k == 0 && st->thermostat == 1) {
                double ke0 = 0.0, R, g2;
                for (int i = 0; i < nd; ++i) ke0 += 0.5 * pk[i] * pk[i] / mass[i];
                qo_stepper_centroid_draw(st->seed, st->sys, nd, st->step - 1, &R, &g2);
                const double alpha = sqrt((R * R + g2) / (2.0 * s->beta_n * ke0));
                for (int i = 0; i < nd; ++i) pk[i] *= alpha;
                continue;
            }
            const double c1 = k == 0 ? exp(-s->dt / (st->tau0_fs * K.fs2au)) : exp(-s->dt * pref * sin(k * QO_PI / P));
            const double c2 = sqrt(1.0 - c1 * c1);
            for (int i = 0; i < nd; ++i) {
                stepper_block((uint32_t)i, (uint32_t)k, st->step, k0, k1, v);
                const double xi = qo_stepper_normal_f32(v[0], v[1]);
                pk[i] = c1 * pk[i] + sqrt(mass[i] / s->beta_n) * c2 * xi;
            }
        }
    }
    cayley_half(s, q, p, mass, disp);
    qo_ftransform(s, q, nd, 0);
    qo_ftransform(s, p, nd, 0);
    qo_ftransform(s, disp, 3 * N, 0);
    for (int b = 0; b < P; ++b)
        if (needs_rebuild(s, disp, b)) qo_neighbour_list(s, q, point, list, disp, b);
    double e;
    if (st->trotter) {
        e = qo_force_eval_trotter(s, q, f, charge, point, list, pot_est);
        memcpy(fphys, f, sizeof(double) * (size_t)P * nd);
    } else {
        e = qo_force_eval_sc(s, q, f, charge, mass, point, list, pot_est, fphys);
    }
    if (cf_acc && st->centroid_fixed) {
        for (int i = 0; i < nd; ++i) {
            double sf = 0.0;
            for (int b = 0; b < P; ++b) sf += fphys[(size_t)b * nd + i];
            cf_acc[i] += sf / (double)P;
        }
        st->cf_samples += 1.0;
    }
    for (size_t i = 0; i < (size_t)P * nd; ++i) p[i] += s->halfdt * f[i];
    st->step += 1;
    return e;
}
