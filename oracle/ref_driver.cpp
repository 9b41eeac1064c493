// Driver that turns the reference's own force/propagation sources into a
// loadable library (oracle/_ref/libqtipref.so) for pinning the oracle.
//
// Test infrastructure only: it is compiled in the development container, from
// the reference's unmodified sources (forces.cpp, neighbour.cpp, fourier.cpp,
// update.cpp, thermostat.cpp, path_integrals.cpp) plus the FFTW/Boost shims in
// oracle/shim. It defines the configuration globals that water.cpp:29-38 would
// define (the reference keeps all configuration in mutable globals, see
// qtip4pfparams.h:17-156), derives them the way water.cpp:76-157 does for an
// arbitrary orthorhombic box, and exposes C entry points around the reference
// functions. Nothing under oracle/ is part of the product.
#include <array>
#include <cmath>
#include <cstring>
#include <fstream>
#include <random>
#include <string>
#include <vector>
#include <boost/math/interpolators/cubic_b_spline.hpp>

#include "qtip4pfparams.h"
#include "indexing.h"
#include "forces.h"
#include "neighbour.h"
#include "fourier.h"
#include "update.h"
#include "thermostat.h"
#include "path_integrals.h"
#include "initialise.h"

// ---- the reference's configuration globals (declared extern in qtip4pfparams.h)
double T_K, epsilonsc, rho_inp, dtfs, eps, a_cell_angs, a_cell, b_cell, c_cell, rnn;
int n_beads, n_cell_x, n_cell_y, n_cell_z, n_cells;
int n_mols, n_atoms, n_dof, list_size;
double T_red, beta, piovern, beta_n, omega_p, omega_psq;
double v_cell, vol, rho_ox, sd_ox, sd_h, dt, halfdt;
double acc, rho, min_xy, min_box, kwald_prefactor, max_xy, max_box;
std::array<double, 3> boxl;
int n_equil, n_samp;
bool is_spline;

static std::vector<double> g_charge;
static std::vector<double> g_mass;

extern "C" {

// Set every global for a system of nmol waters in an orthorhombic box (bohr).
// Mirrors the derivations of water.cpp:76-157, with the box given directly
// instead of through fcc/orth unit cells (vol = Lx*Ly*Lz, rho_ox = N/vol).
void ref_setup(int nmol, int nbeads, const double *box_bohr, double temp_K,
               double dt_fs, double eps_ewald, double eps_sc) {
    n_beads = nbeads;
    T_K = temp_K;
    epsilonsc = eps_sc;
    dtfs = dt_fs;
    eps = eps_ewald;
    n_mols = nmol;
    n_cells = 1;
    n_cell_x = n_cell_y = n_cell_z = 1;
    T_red = K2au * T_K;
    beta = 1.0 / T_red;
    piovern = pi / n_beads;
    beta_n = beta / n_beads;
    omega_p = 1.0 / (beta_n * hbar);
    omega_psq = omega_p * omega_p;
    n_atoms = 3 * n_mols;
    n_dof = 3 * n_atoms;
    boxl = {box_bohr[0], box_bohr[1], box_bohr[2]};
    a_cell = boxl[0];
    b_cell = boxl[1];
    c_cell = boxl[2];
    v_cell = boxl[0] * boxl[1] * boxl[2];
    vol = v_cell;
    rho_ox = n_mols / vol;
    list_size = std::round(4.0 * r_skin * r_skin * r_skin * n_mols * rho_ox);
    sd_ox = sqrt(mo / beta_n);
    sd_h = sqrt(mh / beta_n);
    dt = dtfs * fs2au;
    halfdt = 0.5 * dt;
    acc = sqrt(-log(eps));
    rho = n_atoms / vol;
    min_xy = std::min(boxl[0], boxl[1]);
    min_box = std::min(min_xy, boxl[2]);
    kwald_prefactor = 2.0 * pi / vol;
    max_xy = std::max(boxl[0], boxl[1]);
    max_box = std::max(max_xy, boxl[2]);
    g_charge.assign(n_atoms, 0.0);
    g_mass.assign(n_dof, 0.0);
    for (int i = 0; i < n_mols; ++i) {
        g_charge[3 * i] = qo;
        g_charge[3 * i + 1] = qh;
        g_charge[3 * i + 2] = qh;
        for (int d = 0; d < 3; ++d) {
            g_mass[9 * i + d] = mo;
            g_mass[9 * i + d + 3] = mh;
            g_mass[9 * i + d + 6] = mh;
        }
    }
}

int ref_list_size(void) { return list_size; }

// Ewald parameters exactly as forces.cpp:574-584 derives them.
void ref_ewald_params(double *out) {
    double ewald_kappa = 2.6 * std::pow(rho / vol, 1.0 / 6.0);
    double rwald_cut = acc / ewald_kappa;
    if (rwald_cut > 0.5 * min_box) {
        rwald_cut = 0.5 * min_box;
        ewald_kappa = acc / rwald_cut;
    }
    double k_cut = 2.0 * acc * ewald_kappa;
    int k_max = static_cast<int>(k_cut * max_box / (2.0 * pi));
    out[0] = ewald_kappa;
    out[1] = rwald_cut;
    out[2] = k_cut;
    out[3] = (double)k_max;
    out[4] = (double)list_size;
    out[5] = dt;
    out[6] = beta_n;
    out[7] = omega_psq;
}

void ref_neighbour_list(const double *pos, int *point, int *list, double *disp, int bead) {
    neighbour_list(pos, point, list, disp, bead);
}

double ref_get_forces(const double *pos, double *f, const int *point, const int *list, int bead) {
    return get_forces_nospline(pos, f, g_charge.data(), point, list, bead);
}

// kwald alone on a caller-built charge-site array, with the parameters of
// forces.cpp:574-584.
double ref_kwald(const double *charge_pos, double *f, int bead) {
    double p[8];
    ref_ewald_params(p);
    double k_cut_sq = p[2] * p[2];
    return kwald(charge_pos, f, g_charge.data(), (int)p[3], p[0], k_cut_sq, bead);
}

double ref_force_eval_sc(const double *pos, double *f, const int *point, const int *list,
                         double *sc_pot, double *fphys) {
    double scp = 0.0;
    double e = force_eval_sc_nospline(pos, f, g_charge.data(), g_mass.data(), point, list, scp, fphys);
    *sc_pot = scp;
    return e;
}

void ref_ftransform(double *a, int length, int fwd) { ftransform(a, length, fwd != 0); }

double ref_get_kcv(const double *q, const double *f) { return get_kcv(q, f); }

double ref_get_conserved(double *q, double *p, double energy) {
    return get_conserved(q, p, g_mass.data(), energy);
}

double ref_update_class(double *q, double *p, double *f, int *point, int *list, double *disp) {
    return update_trajectory_class_nospline(q, p, g_mass.data(), f, g_charge.data(), point, list, disp);
}

double ref_update_sc(double *q, double *p, double *f, double *fphys, int *point, int *list,
                     double *disp, unsigned seed, int is_nvt, double *heat, double *sc_pot) {
    std::mt19937 rng(seed);
    double h = *heat, scp = 0.0;
    double e = update_sc_nospline(q, p, g_mass.data(), f, fphys, g_charge.data(), point, list,
                                  disp, rng, is_nvt != 0, h, scp);
    *heat = h;
    *sc_pot = scp;
    return e;
}

// pile_g with a generator seeded by `seed`. The random numbers it consumes are
// replayed from an identical generator with identically constructed
// distributions, in the same call order as thermostat.cpp:64-133, and returned
// in `noise` as [R, g2, xi(bead=1..P-1, dof=0..n_dof-1)], where g2 is the
// combined chi-square draw (2*gamma + R_add^2 for even dof, 2*gamma otherwise).
double ref_pile_g(double *p, unsigned seed, double *noise) {
    std::mt19937 rng(seed);
    std::mt19937 replay(seed);
    double heat = pile_g(p, g_mass.data(), rng);
    std::normal_distribution<double> gauss(0.0, 1.0);
    int dof = 3 * n_atoms;
    double R = gauss(replay);
    double g2;
    if (dof % 2 == 0) {
        std::gamma_distribution<double> gam((dof - 2) / 2, 1.0);
        double R_add = gauss(replay);
        g2 = 2.0 * gam(replay) + R_add * R_add;
    } else {
        std::gamma_distribution<double> gam((dof - 1) / 2, 1.0);
        g2 = 2.0 * gam(replay);
    }
    noise[0] = R;
    noise[1] = g2;
    size_t k = 2;
    for (int b = 1; b < n_beads; ++b)
        for (int i = 0; i < n_dof; ++i) noise[k++] = gauss(replay);
    return heat;
}

// bussi (thermostat.cpp:12-60) with a generator seeded by `seed`; its two
// draws are replayed as for ref_pile_g and returned in noise = [R, g2].
double ref_bussi(double *p, unsigned seed, double *noise) {
    std::mt19937 rng(seed);
    std::mt19937 replay(seed);
    double heat = bussi(p, g_mass.data(), rng);
    std::normal_distribution<double> gauss(0.0, 1.0);
    int dof = 3 * n_atoms;
    double R = gauss(replay);
    double g2;
    if (dof % 2 == 0) {
        std::gamma_distribution<double> gam((dof - 2) / 2, 1.0);
        double R_add = gauss(replay);
        g2 = 2.0 * gam(replay) + R_add * R_add;
    } else {
        std::gamma_distribution<double> gam((dof - 1) / 2, 1.0);
        g2 = 2.0 * gam(replay);
    }
    noise[0] = R;
    noise[1] = g2;
    return heat;
}

// ---- starting configurations: initialise.cpp -------------------------------
// The cell globals as water.cpp:76-114 derives them for "fcc" (cell 0) or
// "orth" (cell 1) from nx x ny x nz cells at density rho (g/cm^3).
void ref_setup_cells(int nx, int ny, int nz, double rho_g_cm3, int orth, int nbeads) {
    n_beads = nbeads;
    n_cell_x = nx;
    n_cell_y = ny;
    n_cell_z = nz;
    n_cells = nx * ny * nz;
    rho_inp = rho_g_cm3;
    if (!orth) {
        n_mols = 4 * n_cells;
        a_cell_angs = 1e8 * std::cbrt(4 * mh2o / rho_inp);
        a_cell = a_cell_angs * angs2bohr;
        b_cell = a_cell;
        c_cell = a_cell;
    } else {
        n_mols = 8 * n_cells;
        a_cell_angs = 1e8 * std::cbrt(4 * mh2o / (sqrt(2.0) * rho_inp));
        a_cell = a_cell_angs * angs2bohr;
        b_cell = sqrt3 * a_cell;
        c_cell = 2.0 * sqrt(2.0 / 3.0) * a_cell;
        rnn = (0.5 - 2.0 * zo) * c_cell;
    }
    n_atoms = 3 * n_mols;
    n_dof = 3 * n_atoms;
    boxl = {n_cell_x * a_cell, n_cell_y * b_cell, n_cell_z * c_cell};
}

int ref_n_mols(void) { return n_mols; }
void ref_box(double *out) {
    out[0] = boxl[0];
    out[1] = boxl[1];
    out[2] = boxl[2];
}

void ref_initialise_fcc(double *out) {
    double *p = initialise_fcc();
    std::memcpy(out, p, sizeof(double) * (size_t)n_beads * n_dof);
    delete[] p;
}

// initialise_orth with std::mt19937(seed); its log lines go to `logpath`
void ref_initialise_orth(unsigned seed, const char *logpath, double *out) {
    std::mt19937 rng(seed);
    std::ofstream log(logpath);
    double *p = initialise_orth(rng, log);
    std::memcpy(out, p, sizeof(double) * (size_t)n_beads * n_dof);
    delete[] p;
}

// ---- the spline ("fast-CMD") path: forces.cpp:634-691, :791-882; update.cpp
// :16-75, :139-269. Tables as simulation.cpp:36-116 builds them: values on the
// knots 0, 0.01, ... bohr, cutoff^2 = (0.01 (n - 1))^2, end slopes estimated.
static boost::math::cubic_b_spline<double> g_spl[3];
static double g_spl_cutsq[3];

void ref_set_splines(const double *oo, int n_oo, const double *oh, int n_oh, const double *hh, int n_hh) {
    const double *v[3] = {oo, oh, hh};
    const int n[3] = {n_oo, n_oh, n_hh};
    for (int t = 0; t < 3; ++t) {
        g_spl[t] = boost::math::cubic_b_spline<double>(v[t], v[t] + n[t], 0.0, 0.01);
        const double cut = 0.0 + 0.01 * (n[t] - 1);
        g_spl_cutsq[t] = cut * cut;
    }
}

double ref_get_forces_wspline(const double *pos, double *f, const int *point, const int *list, int bead) {
    return get_forces_wspline(pos, f, g_charge.data(), point, list, g_spl[0], g_spl[1], g_spl[2], g_spl_cutsq[0],
                              g_spl_cutsq[1], g_spl_cutsq[2], bead);
}

double ref_force_eval_sc_wspline(const double *pos, double *f, const int *point, const int *list, double *sc_pot,
                                 double *fphys) {
    double scp = 0.0;
    double e = force_eval_sc_wspline(pos, f, g_charge.data(), g_mass.data(), point, list, g_spl[0], g_spl[1],
                                     g_spl[2], g_spl_cutsq[0], g_spl_cutsq[1], g_spl_cutsq[2], scp, fphys);
    *sc_pot = scp;
    return e;
}

double ref_update_class_wspline(double *q, double *p, double *f, int *point, int *list, double *disp) {
    return update_trajectory_class_wspline(q, p, g_mass.data(), f, g_charge.data(), point, list, disp, g_spl[0],
                                           g_spl[1], g_spl[2], g_spl_cutsq[0], g_spl_cutsq[1], g_spl_cutsq[2]);
}

double ref_update_sc_wspline(double *q, double *p, double *f, double *fphys, int *point, int *list, double *disp,
                             double *sc_pot) {
    std::mt19937 rng(1);
    double h = 0.0, scp = 0.0;
    double e = update_sc_wspline(q, p, g_mass.data(), f, fphys, g_charge.data(), point, list, disp, rng, false, h,
                                 scp, g_spl[0], g_spl[1], g_spl[2], g_spl_cutsq[0], g_spl_cutsq[1], g_spl_cutsq[2]);
    *sc_pot = scp;
    return e;
}

}  // extern "C"
