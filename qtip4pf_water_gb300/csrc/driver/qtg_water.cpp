// qtg_water: the reference's run driver (water.cpp + simulation.cpp) on the GB300
// library's device-resident stepper.
//
// It reads the reference's config.txt (water.cpp:45-63: n_beads, T_K,
// epsilon_sc, n_cell_x/y/z, rho_inp, dtfs, eps_ewald, n_equil, n_samp,
// is_spline, cell_type fcc|orth, from_file yes <file>|no), builds the start
// the same way (fcc lattice, proton-disordered ice Ih, or a position file:
// initialise.cpp), draws the momenta from the run's std::mt19937 as
// simulation.cpp:347-372 / :848-873 do, and runs the reference's two phases
// -- classical velocity Verlet NVE, or Suzuki-Chin PIMD with PILE-G -- writing
// the reference's files in its formats:
//   output.txt             "rd output <seed>", the ice-rule search lines, progress
//   initial_positions.txt  "x y z" per atom, bead by bead (water.cpp:195-207)
//   cons.txt               conserved quantity every n_step = 100 steps of both phases
//   pot.txt, kin.txt       classical: mean potential and kinetic energy of sampling
//   pot_sc.txt, kcv.txt    PIMD: mean Suzuki-Chin potential and centroid-virial
//                          kinetic energy of sampling (simulation.cpp:949-987)
//   final_positions.txt    as initial_positions.txt, after the run (water.cpp:233-245)
// With is_spline 1 the pair tables oo/oh/hh_spline.txt (one value a line, knots
// 0, 0.01, ... bohr; simulation.cpp:36-116) are added to every force
// evaluation, and the PIMD phases run the spline driver's ensembles
// (equilibration NVE, sampling NVT; simulation.cpp:676, :732).
//
// What differs from the reference, by design: the steps run device-resident
// (one CUDA-graph replay each, estimators recorded on the device), so the
// thermostat's noise comes from the library's counter-based generator keyed by
// the run's seed, not from the std::mt19937 stream (the drop-in
// libqtip_compat.so keeps that stream when it matters); the conserved quantity
// is evaluated without the normal-mode round trip that perturbs the
// reference's live state every 100 steps (path_integrals.cpp:61-78); a phase
// of fewer than 10 steps prints no progress lines (the reference divides by
// zero there).
//
// usage: qtg_water [--seed N] [--precision mixed|fp64] [--dump-sampling-start FILE]
//   --seed       the run's std::mt19937 seed (default: std::random_device, as water.cpp:153)
//   --precision  mixed (default; forces within 1e-4 of FP64) or fp64
//   --dump-sampling-start  write the state that enters the sampling phase (the
//                start-file layout of the drop-in tests: int32 N, P; double box[3],
//                T, dt_fs, eps_ewald, eps_sc; q, p), for replaying it elsewhere
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <random>
#include <string>
#include <vector>

#include "../../../include/qtip4pf_gb300.h"
#include "../lattice.h"

namespace {

constexpr int N_STEP = 100;  // qtip4pfparams.h:37

struct Config {
    int n_beads = 1, ncx = 1, ncy = 1, ncz = 1, n_equil = 0, n_samp = 0;
    double T_K = 298.0, eps_sc = 1e-5, rho = 0.997, dtfs = 0.5, eps = 1e-6;
    bool is_spline = false;
    std::string cell_type = "fcc", from_file = "no", filename;
};

// water.cpp:45-63: "name value" pairs in a fixed order
bool read_config(const char *path, Config &c) {
    std::ifstream in(path);
    if (!in.is_open()) return false;
    std::string name;
    in >> name >> c.n_beads >> name >> c.T_K >> name >> c.eps_sc >> name >> c.ncx >> name >> c.ncy >> name >> c.ncz;
    in >> name >> c.rho >> name >> c.dtfs >> name >> c.eps >> name >> c.n_equil >> name >> c.n_samp;
    in >> name >> c.is_spline >> name >> c.cell_type >> name >> c.from_file;
    if (c.from_file == "yes") in >> c.filename;
    return !in.fail() || c.from_file != "yes";
}

void check(qtg_status st, qtg_ctx *ctx, const char *what) {
    if (st == QTG_OK) return;
    std::cerr << "qtg_water: " << what << ": " << qtg_status_string(st) << " (" << qtg_last_error(ctx) << ")\n";
    std::exit(1);
}

void write_positions(const char *name, const std::vector<double> &q, int n_beads, int n_atoms) {
    std::ofstream f(name);
    for (int b = 0; b < n_beads; ++b)
        for (int i = 0; i < n_atoms; ++i) {
            const double *x = q.data() + (size_t)b * 3 * n_atoms + 3 * i;
            f << x[0] << " " << x[1] << " " << x[2] << "\n";
        }
}

std::vector<double> read_table(const char *name) {
    std::ifstream in(name);
    std::vector<double> v;
    std::string line;
    if (!in.is_open()) std::cerr << "couldn't read, " << name << " appears to be closed \n";
    while (std::getline(in, line))
        if (!line.empty()) v.push_back(std::stod(line));
    return v;
}

// Maxwell-Boltzmann momenta at the bead temperature from the run's generator in
// the reference's order (bead, molecule, dimension: O, H1, H2), then the mean
// momentum per atom of the whole extended system removed.
void draw_momenta(std::mt19937 &rng, std::vector<double> &p, int n_beads, int n_mols, double sd_o, double sd_h) {
    std::normal_distribution<double> dev_o(0.0, sd_o), dev_h(0.0, sd_h);
    const int n_dof = 9 * n_mols, n_atoms = 3 * n_mols;
    double cm[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < n_beads; ++b)
        for (int i = 0; i < n_mols; ++i)
            for (int d = 0; d < 3; ++d) {
                double *m = p.data() + (size_t)b * n_dof + 9 * i + d;
                m[0] = dev_o(rng);
                m[3] = dev_h(rng);
                m[6] = dev_h(rng);
                cm[d] += m[0] + m[3] + m[6];
            }
    for (int d = 0; d < 3; ++d) cm[d] /= (double)n_atoms * n_beads;
    for (int b = 0; b < n_beads; ++b)
        for (int i = 0; i < n_atoms; ++i)
            for (int d = 0; d < 3; ++d) p[(size_t)b * n_dof + 3 * i + d] -= cm[d];
}

struct Phase {
    const char *label;
    int steps;
    bool nvt;
};

}  // namespace

int main(int argc, char **argv) {
    unsigned seed = 0;
    bool have_seed = false;
    int precision = QTG_MIXED;
    const char *dump = nullptr;
    for (int a = 1; a < argc; ++a) {
        if (!std::strcmp(argv[a], "--seed") && a + 1 < argc) {
            seed = (unsigned)std::strtoul(argv[++a], nullptr, 10);
            have_seed = true;
        } else if (!std::strcmp(argv[a], "--precision") && a + 1 < argc) {
            precision = std::strcmp(argv[++a], "fp64") == 0 ? QTG_FP64 : QTG_MIXED;
        } else if (!std::strcmp(argv[a], "--dump-sampling-start") && a + 1 < argc) {
            dump = argv[++a];
        } else {
            std::cerr << "usage: " << argv[0] << " [--seed N] [--precision mixed|fp64] [--dump-sampling-start FILE]\n";
            return 2;
        }
    }
    Config c;
    if (!read_config("config.txt", c)) {
        std::cerr << "qtg_water: cannot read config.txt\n";
        return 1;
    }
    if (c.n_beads != 1 && c.n_beads % 2 == 1) {  // water.cpp:66-69
        std::cerr << "n_beads should be even for Suzuki-Chin calculations, or set to 1 for classical calculations \n";
        return 1;
    }
    qtg_constants K;
    qtg_get_constants(&K);
    qtg_lattice::Cells g;
    if (c.cell_type == "fcc") {
        g = qtg_lattice::fcc_cells(c.ncx, c.ncy, c.ncz, c.rho, K.angs2bohr);
    } else if (c.cell_type == "orth") {
        g = qtg_lattice::orth_cells(c.ncx, c.ncy, c.ncz, c.rho, K.angs2bohr);
    } else {
        std::cerr << "cell type not supported, should be \"orth\" or \"fcc\" \n";
        return 1;
    }
    const int n_mols = (c.cell_type == "fcc" ? 4 : 8) * c.ncx * c.ncy * c.ncz;
    const int n_atoms = 3 * n_mols, n_dof = 9 * n_mols, P = c.n_beads;
    const double box[3] = {c.ncx * g.a, c.ncy * g.b, c.ncz * g.c};
    if (!have_seed) seed = std::random_device{}();
    std::ofstream out("output.txt");
    out << "rd output " << seed << "\n";
    out.flush();
    std::mt19937 rng(seed);
    if (2.0 * K.r_cut > std::min(std::min(box[0], box[1]), box[2]))
        std::cerr << "LJ cutoff is greater than half the smallest dimension of the simulation box! \n";

    std::vector<double> q((size_t)P * n_dof, 0.0), p((size_t)P * n_dof, 0.0);
    if (c.from_file == "yes") {
        qtg_lattice::from_file(c.filename, P, n_dof, q.data());
    } else if (c.cell_type == "fcc") {
        qtg_lattice::fcc(g, K.roheq, K.theta_eq, P, q.data());
    } else {
        qtg_lattice::ice_ih(g, K.roheq, P, rng, q.data(), &out);
    }
    out.flush();
    write_positions("initial_positions.txt", q, P, n_atoms);

    qtg_system_desc d;
    std::memset(&d, 0, sizeof(d));
    d.n_mols = n_mols;
    d.n_beads = P;
    for (int k = 0; k < 3; ++k) d.box_bohr[k] = box[k];
    d.temp_K = c.T_K;
    d.dt_fs = c.dtfs;
    d.eps_ewald = c.eps;
    d.eps_sc = c.eps_sc;
    d.propagator = P > 1 ? QTG_SUZUKI_CHIN : QTG_TROTTER;
    d.thermostat = QTG_THERMO_PILE_G;
    d.seed = seed;
    qtg_ctx *ctx = nullptr;
    check(qtg_create(&d, 1, precision, &ctx), ctx, "qtg_create");
    if (c.is_spline) {
        const char *names[3] = {"oo_spline.txt", "oh_spline.txt", "hh_spline.txt"};
        std::vector<double> tab[3];
        qtg_pair_spline s[3];
        for (int t = 0; t < 3; ++t) {
            tab[t] = read_table(names[t]);
            const double end = 0.01 * (tab[t].size() - 1);  // simulation.cpp:59-60
            s[t] = qtg_pair_spline{tab[t].data(), (int)tab[t].size(), 0.0, 0.01, NAN, NAN, end * end};
        }
        check(qtg_set_pair_splines(ctx, 0, &s[0], &s[1], &s[2]), ctx, "spline tables");
    }
    // standard deviations of the Maxwell-Boltzmann momenta at the bead temperature
    const double beta_n = 1.0 / (K.K2au * c.T_K) / P;
    const double sd_o = std::sqrt(K.mo / beta_n), sd_h = std::sqrt(K.mh / beta_n);
    draw_momenta(rng, p, P, n_mols, sd_o, sd_h);
    check(qtg_set_state(ctx, 0, q.data(), p.data()), ctx, "set_state");
    check(qtg_init_forces(ctx), ctx, "init_forces");

    // phases: classical NVE / NVE; PIMD NVT / NVE; PIMD with splines NVE / NVT
    const Phase phases[2] = {{"Equilibration", c.n_equil, P > 1 && !c.is_spline},
                             {"Sampling", c.n_samp, P > 1 && c.is_spline}};
    std::ofstream cons("cons.txt");
    double sum_pot = 0.0, sum_ke = 0.0;
    const int chunk = 4000;  // the device keeps the last 4096 step records
    std::vector<double> rec((size_t)chunk * 8);
    const auto t0 = std::chrono::steady_clock::now();
    long long total_steps = 0;
    for (int ph = 0; ph < 2; ++ph) {
        const Phase &f = phases[ph];
        if (ph == 1) {  // momenta resampled before sampling (simulation.cpp:397-423, :914-934)
            std::vector<double> qd((size_t)P * n_dof), fd((size_t)P * n_dof), fpd((size_t)P * n_dof);
            std::vector<double> dd((size_t)P * 3 * n_mols);
            check(qtg_get_state(ctx, 0, qd.data(), nullptr, fd.data(), fpd.data(), dd.data()), ctx, "get_state");
            draw_momenta(rng, p, P, n_mols, sd_o, sd_h);
            check(qtg_set_state(ctx, 0, qd.data(), p.data()), ctx, "set_state");
            check(qtg_init_forces(ctx), ctx, "init_forces");
            if (dump) {
                FILE *fp = std::fopen(dump, "wb");
                if (fp) {
                    const int hdr[2] = {n_mols, P};
                    const double par[7] = {box[0], box[1], box[2], c.T_K, c.dtfs, c.eps, c.eps_sc};
                    std::fwrite(hdr, sizeof(int), 2, fp);
                    std::fwrite(par, sizeof(double), 7, fp);
                    std::fwrite(qd.data(), sizeof(double), qd.size(), fp);
                    std::fwrite(p.data(), sizeof(double), p.size(), fp);
                    std::fclose(fp);
                }
            }
        }
        const int n_out = f.steps / 10;
        for (int i0 = 0; i0 < f.steps; i0 += chunk) {
            const int n = std::min(chunk, f.steps - i0);
            check(qtg_reset_estimators(ctx), ctx, "reset_estimators");
            check(qtg_run_steps(ctx, n, f.nvt ? 1 : 0), ctx, "run_steps");
            int got = 0;
            check(qtg_get_estimators(ctx, 0, rec.data(), n, &got), ctx, "get_estimators");
            if (got != n) {
                std::cerr << "qtg_water: expected " << n << " step records, got " << got << "\n";
                return 1;
            }
            for (int k = 0; k < n; ++k) {
                const int i = i0 + k;
                const double *r = rec.data() + (size_t)k * 8;
                if (n_out > 0 && i % n_out == 0) out << f.label << " is " << 10 * i / n_out << "% done \n";
                if (i % N_STEP == 0) cons << r[QTG_EST_CONSERVED] << "\n";
                if (ph == 1) {
                    sum_pot += P > 1 ? r[QTG_EST_POT] : r[QTG_EST_VTOT];
                    sum_ke += P > 1 ? r[QTG_EST_KCV] : r[QTG_EST_KIN];
                }
            }
            out.flush();
            cons.flush();
            total_steps += n;
        }
    }
    const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (c.n_samp > 0) {
        std::ofstream potf(P > 1 ? "pot_sc.txt" : "pot.txt");
        potf << sum_pot / c.n_samp << "\n";
        std::ofstream kf(P > 1 ? "kcv.txt" : "kin.txt");
        kf << sum_ke / c.n_samp << "\n";
    }
    check(qtg_get_state(ctx, 0, q.data(), nullptr, nullptr, nullptr, nullptr), ctx, "get_state");
    write_positions("final_positions.txt", q, P, n_atoms);
    if (total_steps > 0)
        std::cerr << "qtg_water: " << total_steps << " steps, " << n_mols << " waters, " << P << " beads: "
                  << c.dtfs * 1e-6 * total_steps / secs * 86400.0 << " ns/day\n";
    qtg_destroy(ctx);
    return 0;
}
