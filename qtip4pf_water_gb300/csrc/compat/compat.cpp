// Drop-in replacement, with the reference's own C++ signatures, for the force /
// neighbour / fourier / update / thermostat / estimator functions that
// rayseashyn/qtip4pf_water's simulation.cpp calls (forces.h, neighbour.h,
// fourier.h, update.h, thermostat.h, path_integrals.h). Link simulation.cpp,
// water.cpp and initialise.cpp against libqtip_compat.so instead of
// forces.cpp, neighbour.cpp, fourier.cpp, update.cpp, thermostat.cpp and
// path_integrals.cpp; the GPU does the work through the C ABI of libqtipgpu.
//
// The reference keeps its configuration in mutable globals (qtip4pfparams.h
// :17-156, defined in water.cpp:29-38); this file reads the same globals and
// keeps one library context matching them, recreated if they change.
//
// Random numbers: the thermostat draws from the caller's std::mt19937 with the
// same distributions, constructed and called in the same order as
// thermostat.cpp:64-133 (one normal R, then for even dof a normal and a gamma,
// then (P-1) * n_dof normals), and hands them to the GPU. The caller's
// generator therefore advances exactly as it does under the reference.
//
// Errors: the reference prints to std::cerr and continues; so does this shim
// (a failing library call prints the library's message to std::cerr).
//
// Precision: FP64 (the reference's arithmetic) unless the environment sets
// QTG_PRECISION=mixed (FP32 Ewald with FP64 accumulation, integration and
// thermostat; forces within 1e-4 relative of FP64).
//
// Host arrays: the reference allocates its state with new[] (simulation.cpp
// :308-315, :797-805). The first step call registers those five arrays with
// the library (page-locked and mapped), so later calls move them inside the
// step's graph instead of by copy calls. They stay registered until the
// process exits (the reference frees them without telling the shim; freed
// registered pages are still valid heap memory). QTG_COMPAT_REGISTER=0 turns
// this off.
//
// Spline ("fast-CMD") path: the *_wspline functions take the caller's
// boost::math::cubic_b_spline tables. Boost's spline has no accessors for its
// knots, so the shim reads it through its interface on the grid the
// reference's run drivers build it on (knots 0, 0.01, ... bohr up to the
// cutoff, simulation.cpp:38-39, :59-60 and likewise for O-H and H-H): the
// values at the knots and the slopes at both ends determine the clamped cubic
// spline, which the library then evaluates on the GPU for every pair. The
// tables are read once per set of spline objects; a *_nospline call after them
// removes the tables from the library again.
//
// forces.h's per-pair helpers (lj_oxygen, intra_morse_bond, intra_harm_angle,
// rwald, get_spline) and get_q_centroid are exported for link compatibility and
// evaluate on the host, as the reference's do: the library's force
// evaluations never call them (the GPU evaluates every pair inside its force
// kernels). kwald runs on the GPU.
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <random>
#include <set>
#include <vector>

#include <boost/math/interpolators/cubic_b_spline.hpp>

#include "qtip4pf_gb300.h"

// ---- the reference's configuration globals (defined by the host program) ----
extern double T_K, epsilonsc, dtfs, eps;
extern int n_beads, n_mols, n_atoms, n_dof, list_size;
extern std::array<double, 3> boxl;

namespace {

struct Key {
    int n_mols, n_beads;
    double box[3], T_K, dtfs, eps, epsilonsc;
    bool operator==(const Key &o) const {
        return n_mols == o.n_mols && n_beads == o.n_beads && box[0] == o.box[0] && box[1] == o.box[1] &&
               box[2] == o.box[2] && T_K == o.T_K && dtfs == o.dtfs && eps == o.eps && epsilonsc == o.epsilonsc;
    }
};

qtg_ctx *g_ctx = nullptr;
Key g_key;

using spline_t = boost::math::cubic_b_spline<double>;
constexpr double KNOT_STEP = 0.01;  // simulation.cpp:39, :67, :94

struct SplineKey {
    const void *t[3] = {nullptr, nullptr, nullptr};
    double cut_sq[3] = {0, 0, 0};
    bool operator==(const SplineKey &o) const {
        for (int k = 0; k < 3; ++k)
            if (t[k] != o.t[k] || cut_sq[k] != o.cut_sq[k]) return false;
        return true;
    }
};
SplineKey g_spl_key;  // the tables attached to the library context (all null: none)

Key current_key() {
    Key k;
    k.n_mols = n_mols;
    k.n_beads = n_beads;
    for (int d = 0; d < 3; ++d) k.box[d] = boxl[d];
    k.T_K = T_K;
    k.dtfs = dtfs;
    k.eps = eps;
    k.epsilonsc = epsilonsc;
    return k;
}

void report(qtg_status st, const char *what) {
    if (st != QTG_OK)
        std::cerr << what << ": " << qtg_status_string(st) << " (" << qtg_last_error(g_ctx) << ")\n";
}

qtg_ctx *ctx() {
    const Key k = current_key();
    if (g_ctx && k == g_key) return g_ctx;
    if (g_ctx) qtg_destroy(g_ctx);
    g_ctx = nullptr;
    qtg_system_desc d;
    d.n_mols = n_mols;
    d.n_beads = n_beads;
    for (int i = 0; i < 3; ++i) d.box_bohr[i] = boxl[i];
    d.temp_K = T_K;
    d.dt_fs = dtfs;
    d.eps_ewald = eps;
    d.eps_sc = epsilonsc;
    d.propagator = n_beads > 1 ? QTG_SUZUKI_CHIN : QTG_TROTTER;
    d.thermostat = QTG_THERMO_PILE_G;
    d.tau0_fs = 0.0;
    d.seed = 0;
    const char *prec = std::getenv("QTG_PRECISION");
    const int precision = (prec && std::strcmp(prec, "mixed") == 0) ? QTG_MIXED : QTG_FP64;
    qtg_status st = qtg_create(&d, 1, precision, &g_ctx);
    if (st != QTG_OK) {
        std::cerr << "qtg_create: " << qtg_status_string(st) << "\n";
        g_ctx = nullptr;
    }
    g_key = k;
    g_spl_key = SplineKey{};
    return g_ctx;
}

// ---- host arrays: registered once each (see the file comment) ----
std::set<const void *> g_registered;

void register_arrays(double *q, double *p, double *f, double *fphys, double *disp, size_t nt, size_t nd) {
    static const bool on = [] {
        const char *e = std::getenv("QTG_COMPAT_REGISTER");
        return !(e && std::strcmp(e, "0") == 0);
    }();
    if (!on) return;
    double *a[5] = {q, p, f, fphys, disp};
    const size_t n[5] = {nt, nt, nt, nt, nd};
    for (int k = 0; k < 5; ++k) {
        if (!a[k] || g_registered.count(a[k])) continue;
        if (qtg_register_host(a[k], n[k] * sizeof(double)) == QTG_OK) g_registered.insert(a[k]);
    }
}

// ---- spline tables (see the file comment) ----

bool attach_splines(const spline_t &oo, const spline_t &oh, const spline_t &hh, double oo_cutsq, double oh_cutsq,
                    double hh_cutsq) {
    SplineKey k;
    const spline_t *sp[3] = {&oo, &oh, &hh};
    const double cs[3] = {oo_cutsq, oh_cutsq, hh_cutsq};
    for (int t = 0; t < 3; ++t) {
        k.t[t] = sp[t];
        k.cut_sq[t] = cs[t];
    }
    if (k == g_spl_key) return true;
    std::vector<double> vals[3];
    qtg_pair_spline tab[3];
    for (int t = 0; t < 3; ++t) {
        const double r_end = std::sqrt(cs[t]);
        const int n = (int)std::lround(r_end / KNOT_STEP) + 1;
        vals[t].resize(n);
        for (int i = 0; i < n; ++i) vals[t][i] = (*sp[t])(KNOT_STEP * i);
        tab[t].values = vals[t].data();
        tab[t].n = n;
        tab[t].start = 0.0;
        tab[t].step = KNOT_STEP;
        tab[t].left_deriv = sp[t]->prime(0.0);
        tab[t].right_deriv = sp[t]->prime(KNOT_STEP * (n - 1));
        tab[t].cut_sq = cs[t];
    }
    const qtg_status st = qtg_set_pair_splines(g_ctx, 0, &tab[0], &tab[1], &tab[2]);
    report(st, "spline tables");
    if (st != QTG_OK) return false;
    g_spl_key = k;
    return true;
}

void detach_splines() {
    if (g_spl_key == SplineKey{}) return;
    report(qtg_set_pair_splines(g_ctx, 0, nullptr, nullptr, nullptr), "spline tables");
    g_spl_key = SplineKey{};
}

qtg_constants consts() {
    static const qtg_constants K = [] {
        qtg_constants k;
        qtg_get_constants(&k);
        return k;
    }();
    return K;
}

// indexing.h:6-8: element of bead b at index i
inline size_t bidx(int bead, int i) { return (size_t)bead * n_dof + i; }

// The random numbers thermostat.cpp:64-133 consumes, drawn in its order.
void draw_pile_noise(std::mt19937 &gen, std::vector<double> &noise) {
    std::normal_distribution<double> gauss_dev(0.0, 1.0);
    const int dof = 3 * n_atoms;
    noise.assign(2 + (size_t)(n_beads - 1) * n_dof, 0.0);
    const double R = gauss_dev(gen);
    double g2;
    if (dof % 2 == 0) {
        std::gamma_distribution<double> gamma_dev((dof - 2) / 2, 1.0);
        const double R_add = gauss_dev(gen);
        g2 = 2.0 * gamma_dev(gen) + R_add * R_add;
    } else {
        std::gamma_distribution<double> gamma_dev((dof - 1) / 2, 1.0);
        g2 = 2.0 * gamma_dev(gen);
    }
    noise[0] = R;
    noise[1] = g2;
    size_t k = 2;
    for (int bead = 1; bead < n_beads; ++bead)
        for (int i = 0; i < n_dof; ++i) noise[k++] = gauss_dev(gen);
}

}  // namespace

// neighbour.h:4
void neighbour_list(const double position_array[], int point[], int list[], double disp_array[], int bead) {
    if (!ctx()) return;
    report(qtg_neighbour_list(g_ctx, 0, position_array, point, list, disp_array, bead), "neighbour_list");
}

// forces.h:16
double get_forces_nospline(const double position_array[], double force_array[], const double charge_array[],
                           const int point[], const int list[], int bead) {
    double e = 0.0;
    if (!ctx()) return e;
    detach_splines();
    report(qtg_get_forces(g_ctx, 0, position_array, force_array, charge_array, point, list, bead, &e),
           "get_forces_nospline");
    return e;
}

// forces.h:20
double force_eval_sc_nospline(const double position_array[], double force_array[], const double charge_array[],
                              const double mass_array[], const int point[], const int list[], double &sc_pot,
                              double fphys[]) {
    double e = 0.0;
    if (!ctx()) return e;
    detach_splines();
    std::vector<double> tmp;
    if (!fphys) {
        tmp.assign((size_t)n_beads * n_dof, 0.0);
        fphys = tmp.data();
    }
    report(qtg_force_eval_sc(g_ctx, 0, position_array, force_array, charge_array, mass_array, point, list, &sc_pot,
                             fphys, &e),
           "force_eval_sc_nospline");
    return e;
}

// fourier.h:4
void ftransform(double input_array[], const int length, const bool is_forwards) {
    if (!ctx()) return;
    report(qtg_ftransform(g_ctx, 0, input_array, length, is_forwards ? 1 : 0), "ftransform");
}

// thermostat.h:6
double pile_g(double momentum_array[], const double mass_array[], std::mt19937 &gen) {
    double heat = 0.0;
    if (!ctx()) return heat;
    std::vector<double> noise;
    draw_pile_noise(gen, noise);
    report(qtg_pile_g(g_ctx, 0, momentum_array, mass_array, noise.data(), &heat), "pile_g");
    return heat;
}

// thermostat.h:4 (the reference's classical runs have it commented out,
// simulation.cpp:181; the drop-in serves it all the same)
double bussi(double momentum_array[], const double mass_array[], std::mt19937 &gen) {
    double heat = 0.0;
    if (!ctx()) return heat;
    // the two draws of thermostat.cpp:33-44, from the caller's generator in order
    std::normal_distribution<double> gauss_dev(0.0, 1.0);
    const int dof = 3 * n_atoms;
    double noise[2];
    noise[0] = gauss_dev(gen);
    if (dof % 2 == 0) {
        std::gamma_distribution<double> gamma_dev((dof - 2) / 2, 1.0);
        const double R_add = gauss_dev(gen);
        noise[1] = 2.0 * gamma_dev(gen) + R_add * R_add;
    } else {
        std::gamma_distribution<double> gamma_dev((dof - 1) / 2, 1.0);
        noise[1] = 2.0 * gamma_dev(gen);
    }
    report(qtg_bussi(g_ctx, 0, momentum_array, mass_array, noise, &heat), "bussi");
    return heat;
}

// path_integrals.h:5-6
double get_kcv(const double position_array[], const double force_array[]) {
    double v = 0.0;
    if (!ctx()) return v;
    report(qtg_get_kcv(g_ctx, 0, position_array, force_array, &v), "get_kcv");
    return v;
}

double get_conserved(double position_array[], double momentum_array[], const double mass_array[], double energy) {
    double v = 0.0;
    if (!ctx()) return v;
    report(qtg_get_conserved(g_ctx, 0, position_array, momentum_array, mass_array, energy, &v), "get_conserved");
    return v;
}

// update.h:5
double update_trajectory_class_nospline(double position_array[], double momentum_array[], const double mass_array[],
                                        double force_array[], double charge_array[], int point[], int list[],
                                        double disp_array[]) {
    double e = 0.0;
    if (!ctx()) return e;
    detach_splines();
    register_arrays(position_array, momentum_array, force_array, nullptr, disp_array, (size_t)n_dof,
                    (size_t)3 * n_mols);
    report(qtg_update_class(g_ctx, 0, position_array, momentum_array, mass_array, force_array, charge_array, point,
                            list, disp_array, &e),
           "update_trajectory_class_nospline");
    return e;
}

// update.h:7
double update_sc_nospline(double position_array[], double momentum_array[], const double mass_array[],
                          double force_array[], double fphys[], double charge_array[], int point[], int list[],
                          double disp_array[], std::mt19937 &rng, bool is_nvt, double &heat, double &sc_pot) {
    double e = 0.0;
    if (!ctx()) return e;
    detach_splines();
    register_arrays(position_array, momentum_array, force_array, fphys, disp_array, (size_t)n_beads * n_dof,
                    (size_t)n_beads * 3 * n_mols);
    std::vector<double> noise;
    if (is_nvt) draw_pile_noise(rng, noise);
    report(qtg_update_pimd(g_ctx, 0, position_array, momentum_array, mass_array, force_array, fphys, charge_array,
                           point, list, disp_array, is_nvt ? 1 : 0, is_nvt ? noise.data() : nullptr, &heat, &sc_pot,
                           &e),
           "update_sc_nospline");
    return e;
}

// ---- the spline ("fast-CMD") path: forces.h:14-22, update.h:4-6 -------------

// forces.h:18 (forces.cpp:634-691)
double get_forces_wspline(const double position_array[], double force_array[], const double charge_array[],
                          const int point[], const int list[], const spline_t &oo_spline, const spline_t &oh_spline,
                          const spline_t &hh_spline, const double oo_spline_cutsq, const double oh_spline_cutsq,
                          const double hh_spline_cutsq, int bead) {
    double e = 0.0;
    if (!ctx() || !attach_splines(oo_spline, oh_spline, hh_spline, oo_spline_cutsq, oh_spline_cutsq, hh_spline_cutsq))
        return e;
    report(qtg_get_forces(g_ctx, 0, position_array, force_array, charge_array, point, list, bead, &e),
           "get_forces_wspline");
    return e;
}

// forces.h:22 (forces.cpp:791-882)
double force_eval_sc_wspline(const double position_array[], double force_array[], const double charge_array[],
                             const double mass_array[], const int point[], const int list[], const spline_t &oo_spline,
                             const spline_t &oh_spline, const spline_t &hh_spline, const double oo_spline_cutsq,
                             const double oh_spline_cutsq, const double hh_spline_cutsq, double &sc_pot,
                             double fphys[]) {
    double e = 0.0;
    if (!ctx() || !attach_splines(oo_spline, oh_spline, hh_spline, oo_spline_cutsq, oh_spline_cutsq, hh_spline_cutsq))
        return e;
    std::vector<double> tmp;
    if (!fphys) {
        tmp.assign((size_t)n_beads * n_dof, 0.0);
        fphys = tmp.data();
    }
    report(qtg_force_eval_sc(g_ctx, 0, position_array, force_array, charge_array, mass_array, point, list, &sc_pot,
                             fphys, &e),
           "force_eval_sc_wspline");
    return e;
}

// update.h:4 (update.cpp:16-75)
double update_trajectory_class_wspline(double position_array[], double momentum_array[], const double mass_array[],
                                       double force_array[], double charge_array[], int point[], int list[],
                                       double disp_array[], const spline_t &oo_spline, const spline_t &oh_spline,
                                       const spline_t &hh_spline, const double oo_spline_cutsq,
                                       const double oh_spline_cutsq, const double hh_spline_cutsq) {
    double e = 0.0;
    if (!ctx() || !attach_splines(oo_spline, oh_spline, hh_spline, oo_spline_cutsq, oh_spline_cutsq, hh_spline_cutsq))
        return e;
    register_arrays(position_array, momentum_array, force_array, nullptr, disp_array, (size_t)n_dof,
                    (size_t)3 * n_mols);
    report(qtg_update_class(g_ctx, 0, position_array, momentum_array, mass_array, force_array, charge_array, point,
                            list, disp_array, &e),
           "update_trajectory_class_wspline");
    return e;
}

// update.h:6 (update.cpp:139-269)
double update_sc_wspline(double position_array[], double momentum_array[], const double mass_array[],
                         double force_array[], double fphys[], double charge_array[], int point[], int list[],
                         double disp_array[], std::mt19937 &rng, bool is_nvt, double &heat, double &sc_pot,
                         const spline_t &oo_spline, const spline_t &oh_spline, const spline_t &hh_spline,
                         const double oo_spline_cutsq, const double oh_spline_cutsq, const double hh_spline_cutsq) {
    double e = 0.0;
    if (!ctx() || !attach_splines(oo_spline, oh_spline, hh_spline, oo_spline_cutsq, oh_spline_cutsq, hh_spline_cutsq))
        return e;
    register_arrays(position_array, momentum_array, force_array, fphys, disp_array, (size_t)n_beads * n_dof,
                    (size_t)n_beads * 3 * n_mols);
    std::vector<double> noise;
    if (is_nvt) draw_pile_noise(rng, noise);
    report(qtg_update_pimd(g_ctx, 0, position_array, momentum_array, mass_array, force_array, fphys, charge_array,
                           point, list, disp_array, is_nvt ? 1 : 0, is_nvt ? noise.data() : nullptr, &heat, &sc_pot,
                           &e),
           "update_sc_wspline");
    return e;
}

// ---- forces.h:4-14: the per-pair helpers (host; see the file comment) -------

// forces.h:4 (forces.cpp:25-59): shifted LJ between the oxygens of molecules i, j
double lj_oxygen(const std::array<double, 3> &r_ij, double rijsq, double force_array[], int i, int j, int bead) {
    const qtg_constants K = consts();
    const double p2 = 1.0 / rijsq;
    const double p6 = p2 * p2 * p2, p12 = p6 * p6;
    const double s6 = p6 * K.sigmalj6, s12 = p12 * K.sigmalj12;
    const double e4 = s12 - s6;
    const double fr = (e4 + s12) * (24.0 * K.epslj * p2);
    for (int d = 0; d < 3; ++d) {
        force_array[bidx(bead, 9 * i + d)] += fr * r_ij[d];
        force_array[bidx(bead, 9 * j + d)] -= fr * r_ij[d];
    }
    return e4 * (4.0 * K.epslj) - K.e_cut;
}

// forces.h:6 (forces.cpp:65-93): quartic Morse bond O - H(bond_step) of molecule i
double intra_morse_bond(const std::array<double, 3> &r_oh, double roh, double force_array[], int i, int bond_step,
                        int bead) {
    const qtg_constants K = consts();
    const double x = roh - K.roheq, x2 = x * x, x3 = x2 * x, x4 = x2 * x2;
    const double energy = (K.ar2 * x2 - K.ar3 * x3 + K.ar4fac * x4) * K.Dr;
    const double fr = (2.0 * K.ar2 * x - 3.0 * K.ar3 * x2 + 4.0 * K.ar4fac * x3) * (K.Dr * (1.0 / roh));
    for (int d = 0; d < 3; ++d) {
        force_array[bidx(bead, 9 * i + d)] -= fr * r_oh[d];
        force_array[bidx(bead, 9 * i + 3 * bond_step + d)] += fr * r_oh[d];
    }
    return energy;
}

// forces.h:8 (forces.cpp:96-138): harmonic H-O-H angle of molecule i
double intra_harm_angle(const std::array<double, 3> &r_oh1, const std::array<double, 3> &r_oh2, double roh1,
                        double roh2, double force_array[], int i, int bead) {
    const qtg_constants K = consts();
    const double dot = r_oh1[0] * r_oh2[0] + r_oh1[1] * r_oh2[1] + r_oh1[2] * r_oh2[2];
    const double i1 = 1.0 / roh1, i2 = 1.0 / roh2, i12 = i1 * i2;
    const double c = dot * i12;
    const double th = std::acos(c) - K.theta_eq;
    const double g = K.ktheta * th * (1.0 / std::sqrt(1.0 - c * c));
    const double a1 = dot * (i1 * i1) * i12, a2 = dot * (i2 * i2) * i12;
    for (int d = 0; d < 3; ++d) {
        force_array[bidx(bead, 9 * i + d)] += g * (i12 * (r_oh1[d] + r_oh2[d]) - a1 * r_oh1[d] - a2 * r_oh2[d]);
        force_array[bidx(bead, 9 * i + 3 + d)] -= g * (i12 * r_oh2[d] - a1 * r_oh1[d]);
        force_array[bidx(bead, 9 * i + 6 + d)] -= g * (i12 * r_oh1[d] - a2 * r_oh2[d]);
    }
    return 0.5 * K.ktheta * th * th;
}

// forces.h:10 (forces.cpp:141-177): real-space Ewald between sites i, j (erfc - 1
// inside one molecule)
double rwald(const std::array<double, 3> &r_ij, double rijsq, double force_array[], const double charge_array[], int i,
             int j, double ewald_kappa, int bead) {
    const qtg_constants K = consts();
    const double r = std::sqrt(rijsq), ir = 1.0 / r;
    const double qq = charge_array[i] * charge_array[j];
    double ef = std::erfc(ewald_kappa * r);
    if (i / 3 == j / 3) ef -= 1.0;
    const double energy = qq * ir * ef;
    const double kappa_sq = ewald_kappa * ewald_kappa;
    const double fr = (energy + qq * (2.0 * ewald_kappa / std::sqrt(K.pi)) * std::exp(-kappa_sq * rijsq)) * (ir * ir);
    for (int d = 0; d < 3; ++d) {
        force_array[bidx(bead, 3 * i + d)] += fr * r_ij[d];
        force_array[bidx(bead, 3 * j + d)] -= fr * r_ij[d];
    }
    return energy;
}

// forces.h:12 (forces.cpp:180-448), on the GPU. The library derives kappa, k_max and
// the k set from the globals as get_forces_nospline does (forces.cpp:574-584); other
// parameters are reported and nothing is added.
double kwald(const double position_array[], double force_array[], const double charge_array[], int k_max,
             double ewald_kappa, double k_cut_sq, int bead) {
    double e = 0.0;
    if (!ctx()) return e;
    qtg_system_info info;
    report(qtg_system_info_get(g_ctx, 0, &info), "kwald");
    if (k_max != info.k_max || ewald_kappa != info.kappa || k_cut_sq != info.kc * info.kc) {
        std::cerr << "kwald: parameters differ from the ones the globals give (k_max " << info.k_max << ", kappa "
                  << info.kappa << "); nothing added\n";
        return e;
    }
    report(qtg_kwald(g_ctx, 0, position_array, force_array, charge_array, bead, &e), "kwald");
    return e;
}

// forces.h:14 (forces.cpp:452-466): one spline pair
double get_spline(const std::array<double, 3> r_ij, const double rij, double force_array[], const int i, const int j,
                  const spline_t &spline, int bead) {
    const double fp = spline.prime(rij) / rij;
    for (int d = 0; d < 3; ++d) {
        force_array[bidx(bead, 3 * i + d)] -= fp * r_ij[d];
        force_array[bidx(bead, 3 * j + d)] += fp * r_ij[d];
    }
    return spline(rij);
}

// path_integrals.cpp:10-26 (the definition; path_integrals.h:4 declares a
// by-value first argument that nothing defines): the bead average of each of
// `length` coordinates, in a new[] array the caller deletes.
double *get_q_centroid(const double input_array[], const int length) {
    double *qc = new double[length];
    for (int i = 0; i < length; ++i) {
        double s = 0.0;
        for (int b = 0; b < n_beads; ++b) s += input_array[(size_t)b * length + i];
        qc[i] = s / static_cast<float>(n_beads);
    }
    return qc;
}
