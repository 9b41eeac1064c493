/* CPU oracle for the qTIP4P/F force and ring-polymer propagation path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C, FP64 restatement of the
 * reference's algorithms (rayseashyn/qtip4pf_water), used by the test-suite as
 * the checker for the CUDA library and by bench.py as the timed CPU baseline.
 * The product never links, loads or calls it. Each function cites the
 * reference file:line it restates. Parity of this restatement with the
 * reference's own compiled sources is pinned by tests/golden (fixtures made by
 * tests/golden/make_golden.py from the reference built with oracle/Makefile).
 *
 * Layouts follow the reference (indexing.h:6-24):
 *   positions / momenta / forces  double[P][9N]   ([bead][mol][O,H1,H2][xyz])
 *   neighbour list                point int[P][N], list int[P][list_size]
 *   oxygen displacements          double[P][3N]
 *   charges double[3N], masses double[9N] (per degree of freedom)
 */
#ifndef QTIP_ORACLE_H
#define QTIP_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

typedef struct qo_sys {
    int n_mols, n_atoms, n_dof, n_beads, list_size, k_max;
    double box[3], vol, min_box, max_box;
    double temp_K, beta, beta_n, omega_psq, pi_over_p;
    double dt, halfdt, eps_sc;
    double acc, kappa, rc_sq, kc_sq, k_pref, ewald_pref;
    double r_cut, r_cut_sq, r_skin, r_skin_sq;
    double mo, mh, qo, qh, gamma_m;
    const struct qo_splines *spl; /* tabulated pair corrections, or NULL (qo_set_splines) */
} qo_sys;

/* ---- tabulated pair corrections (forces.cpp:452-466, :634-691) ----------------
 * A clamped uniform cubic B-spline per pair type: c holds c_{-1} .. c_n
 * (n + 2 values) for knots start + i step; pairs with r^2 < cut_sq. */
typedef struct qo_spline {
    int n;
    double start, step, cut_sq;
    const double *c;
} qo_spline;
typedef struct qo_splines {
    qo_spline t[3]; /* O-O, O-H, H-H */
} qo_splines;
/* coefficients of the interpolant of y_0 .. y_{n-1} with end slopes dl, dr (NaN:
 * five-point one-sided estimates); returns 0 on bad input */
int qo_spline_build(const double *y, int n, double step, double dl, double dr, double *c);
/* value at x (and the derivative into *deriv when not NULL) */
double qo_spline_eval(const double *c, int n, double start, double step, double x, double *deriv);
/* attach (NULL: remove) the tables used by every force evaluation of s */
void qo_set_splines(qo_sys *s, const qo_splines *spl);

/* derived parameters: water.cpp:76-157 and forces.cpp:574-584 */
void qo_init(qo_sys *s, int n_mols, int n_beads, const double box_bohr[3], double temp_K,
             double dt_fs, double eps_ewald, double eps_sc);
/* the qTIP4P/F constants in atomic units (qtip4pfparams.h:43-133); out[0..]:
 * angs2bohr, fs2au, K2au, mo, mh, qo, qh, gamma_vs, epslj, sigmalj, e_cut,
 * roheq, ar, Dr, theta_eq, ktheta, r_cut, r_skin, pi */
void qo_constants(double *out);
void qo_default_charges(const qo_sys *s, double *charge);
void qo_default_masses(const qo_sys *s, double *mass);

/* neighbour.cpp:12-62. Returns the number of pairs, or -1 on overflow. */
int qo_neighbour_list(const qo_sys *s, const double *pos, int *point, int *list, double *disp,
                      int bead);
/* forces.cpp:468-630. Returns the bead's potential energy (Hartree). */
double qo_get_forces(const qo_sys *s, const double *pos, double *f, const double *charge,
                     const int *point, const int *list, int bead);
/* forces.cpp:180-448 on an explicit site array (charge sites: M,H1,H2). */
double qo_kwald(const qo_sys *s, const double *sites, double *f_sites, const double *charge,
                int bead);
/* forces.cpp:698-789 (OpenMP over beads). */
double qo_force_eval_sc(const qo_sys *s, const double *pos, double *f, const double *charge,
                        const double *mass, const int *point, const int *list, double *sc_pot,
                        double *fphys);
/* second-order (Trotter) assembly: every bead weight 1, f = fphys; returns sum_b V_b,
 * *pot_est = sum_b V_b / P. No reference counterpart (new path). */
double qo_force_eval_trotter(const qo_sys *s, const double *pos, double *f, const double *charge,
                             const int *point, const int *list, double *pot_est);
/* fourier.cpp:12-69 (orthonormal real DFT along beads, halfcomplex storage). */
void qo_ftransform(const qo_sys *s, double *a, int length, int forwards);
/* thermostat.cpp:64-133 with the random numbers supplied:
 * noise = [R, g2, xi(bead 1..P-1, dof 0..n_dof-1)]. Returns the heat. */
double qo_pile_g(const qo_sys *s, double *p, const double *mass, const double *noise);
/* thermostat.cpp:12-60; noise = [R, g2] (the combined chi-square draw) */
double qo_bussi(const qo_sys *s, double *p, const double *mass, const double *noise);
/* path_integrals.cpp:29-48 and :55-81 */
double qo_get_kcv(const qo_sys *s, const double *q, const double *f);
double qo_get_conserved(const qo_sys *s, double *q, double *p, const double *mass, double energy);
/* update.cpp:78-137 */
double qo_update_class(const qo_sys *s, double *q, double *p, const double *mass, double *f,
                       const double *charge, int *point, int *list, double *disp);
/* update.cpp:271-401; noise as for qo_pile_g (ignored when is_nvt == 0).
 * trotter != 0 swaps the force assembly for qo_force_eval_trotter. */
double qo_update_pimd(const qo_sys *s, double *q, double *p, const double *mass, double *f,
                      double *fphys, const double *charge, int *point, int *list, double *disp,
                      int is_nvt, const double *noise, double *heat, double *pot_est, int trotter);
/* ---- the device stepper's propagation (new paths; no reference counterpart) ----
 * Counter-based noise (Philox4x32-10), PILE-G / PILE-L thermostats and the
 * centroid constraint as the library's device-resident stepper applies them. */
typedef struct qo_stepper {
    unsigned long long seed; /* the system's seed */
    int sys;                 /* the system's index in its context */
    int thermostat;          /* 0 none, 1 PILE-G, 2 PILE-L */
    int trotter;             /* 1 second-order assembly, 0 Suzuki-Chin */
    int centroid_fixed;      /* 1: centroid-constrained PIMD */
    double tau0_fs;          /* PILE-L centroid time constant */
    unsigned long long step; /* counter while the next step runs (1 after the first force evaluation) */
    double cf_samples;       /* steps accumulated into the mean centroid force */
} qo_stepper;
void qo_philox4x32_10(const unsigned int ctr[4], unsigned int k0, unsigned int k1, unsigned int out[4]);
double qo_stepper_normal_f32(unsigned int v0, unsigned int v1);
int qo_stepper_centroid_draw(unsigned long long seed, int sys, int n_dof, unsigned long long st, double *R,
                             double *g2);
double qo_stepper_step(const qo_sys *s, qo_stepper *st, double *q, double *p, const double *mass, double *f,
                       double *fphys, const double *charge, int *point, int *list, double *disp, int is_nvt,
                       double *cf_acc, double *pot_est);

/* number of k-vectors forces.cpp:251-445 visits (each +/- combination counted once). */
int qo_count_kvectors(const qo_sys *s);

#ifdef __cplusplus
}
#endif
#endif
