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
#include <array>
#include <cstdio>
#include <iostream>
#include <random>
#include <vector>

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
    qtg_status st = qtg_create(&d, 1, QTG_FP64, &g_ctx);
    if (st != QTG_OK) {
        std::cerr << "qtg_create: " << qtg_status_string(st) << "\n";
        g_ctx = nullptr;
    }
    g_key = k;
    return g_ctx;
}

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
    std::vector<double> noise;
    if (is_nvt) draw_pile_noise(rng, noise);
    report(qtg_update_pimd(g_ctx, 0, position_array, momentum_array, mass_array, force_array, fphys, charge_array,
                           point, list, disp_array, is_nvt ? 1 : 0, is_nvt ? noise.data() : nullptr, &heat, &sc_pot,
                           &e),
           "update_sc_nospline");
    return e;
}
