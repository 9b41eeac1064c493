// Drop-in driver: calls the force / neighbour / update / thermostat / estimator
// interface in the order the reference's run_sc_nospline does
// (simulation.cpp:829-961): per-bead neighbour lists, the first Suzuki-Chin
// force evaluation, then NVT steps of update_sc_nospline with a seeded
// std::mt19937, then get_kcv and get_conserved. It is linked either against
// the reference's own sources (to record the expected output) or against
// libqtip_compat.so (the GPU drop-in), and prints one line per step.
//
// With a fourth argument "spline" it runs the spline ("fast-CMD") path instead:
// force_eval_sc_wspline and update_sc_wspline with three synthetic pair tables
// y(r) = A exp(-r / lam) (1 - (r / r_end)^2)^2 on the reference's grid (knots
// 0, 0.01, ... bohr; simulation.cpp:36-116), built as boost::math::cubic_b_spline.
//
// usage: dropin_driver <start.bin> <n_steps> <seed> [spline]
// start.bin: int32 n_mols, int32 n_beads, double box[3], double T_K, double dt_fs,
//            double eps_ewald, double eps_sc, then q[P][9N], p[P][9N] (doubles)
#include <array>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>

#include <boost/math/interpolators/cubic_b_spline.hpp>

// the reference's configuration globals (declared extern in qtip4pfparams.h)
double T_K, epsilonsc, rho_inp, dtfs, eps, a_cell_angs, a_cell, b_cell, c_cell, rnn;
int n_beads, n_cell_x, n_cell_y, n_cell_z, n_cells;
int n_mols, n_atoms, n_dof, list_size;
double T_red, beta, piovern, beta_n, omega_p, omega_psq;
double v_cell, vol, rho_ox, sd_ox, sd_h, dt, halfdt;
double acc, rho, min_xy, min_box, kwald_prefactor, max_xy, max_box;
std::array<double, 3> boxl;
int n_equil, n_samp;
bool is_spline;

// the reference's function interface (neighbour.h, forces.h, update.h, path_integrals.h)
void neighbour_list(const double position_array[], int point[], int list[], double disp_array[], int bead);
double force_eval_sc_nospline(const double position_array[], double force_array[], const double charge_array[],
                              const double mass_array[], const int point[], const int list[], double &sc_pot,
                              double fphys[]);
double update_sc_nospline(double position_array[], double momentum_array[], const double mass_array[],
                          double force_array[], double fphys[], double charge_array[], int point[], int list[],
                          double disp_array[], std::mt19937 &rng, bool is_nvt, double &heat, double &sc_pot);
double get_kcv(const double position_array[], const double force_array[]);
using spline_t = boost::math::cubic_b_spline<double>;
double force_eval_sc_wspline(const double position_array[], double force_array[], const double charge_array[],
                             const double mass_array[], const int point[], const int list[], const spline_t &oo,
                             const spline_t &oh, const spline_t &hh, const double oo_cutsq, const double oh_cutsq,
                             const double hh_cutsq, double &sc_pot, double fphys[]);
double update_sc_wspline(double position_array[], double momentum_array[], const double mass_array[],
                         double force_array[], double fphys[], double charge_array[], int point[], int list[],
                         double disp_array[], std::mt19937 &rng, bool is_nvt, double &heat, double &sc_pot,
                         const spline_t &oo, const spline_t &oh, const spline_t &hh, const double oo_cutsq,
                         const double oh_cutsq, const double hh_cutsq);
double get_conserved(double position_array[], double momentum_array[], const double mass_array[], double energy);

int main(int argc, char **argv) {
    if (argc < 4) {
        std::fprintf(stderr, "usage: %s start.bin n_steps seed\n", argv[0]);
        return 2;
    }
    FILE *fp = std::fopen(argv[1], "rb");
    if (!fp) return 3;
    int hdr[2];
    double par[7];
    if (std::fread(hdr, sizeof(int), 2, fp) != 2 || std::fread(par, sizeof(double), 7, fp) != 7) return 4;
    n_mols = hdr[0];
    n_beads = hdr[1];
    boxl = {par[0], par[1], par[2]};
    T_K = par[3];
    dtfs = par[4];
    eps = par[5];
    epsilonsc = par[6];
    // derived globals, as water.cpp:76-157 derives them for a box given directly
    const double pi = 3.14159265359, r_skin = 1.30 * 9.0 / 0.529177210903;
    const double K2au = 1.38064852e-23 / 4.3597447222071e-18;
    const double fs2au = 1.0 / (1.054571817e-34 * 1e15 / 4.3597447222071e-18);
    n_atoms = 3 * n_mols;
    n_dof = 3 * n_atoms;
    T_red = K2au * T_K;
    beta = 1.0 / T_red;
    piovern = pi / n_beads;
    beta_n = beta / n_beads;
    omega_p = 1.0 / beta_n;
    omega_psq = omega_p * omega_p;
    vol = boxl[0] * boxl[1] * boxl[2];
    rho_ox = n_mols / vol;
    list_size = std::round(4.0 * r_skin * r_skin * r_skin * n_mols * rho_ox);
    dt = dtfs * fs2au;
    halfdt = 0.5 * dt;
    acc = std::sqrt(-std::log(eps));
    rho = n_atoms / vol;
    min_xy = std::min(boxl[0], boxl[1]);
    min_box = std::min(min_xy, boxl[2]);
    kwald_prefactor = 2.0 * pi / vol;
    max_xy = std::max(boxl[0], boxl[1]);
    max_box = std::max(max_xy, boxl[2]);

    const size_t nt = (size_t)n_beads * n_dof;
    std::vector<double> q(nt), p(nt), f(nt), fphys(nt), disp((size_t)n_beads * 3 * n_mols, 0.0);
    if (std::fread(q.data(), sizeof(double), nt, fp) != nt || std::fread(p.data(), sizeof(double), nt, fp) != nt)
        return 5;
    std::fclose(fp);
    std::vector<int> point((size_t)n_beads * n_mols), list((size_t)n_beads * list_size);
    std::vector<double> charge(n_atoms), mass(n_dof);
    const double me = 9.10938356e-31, Na = 6.0221409e23;
    const double mo = 0.001 * 15.9994 / (Na * me), mh = 0.001 * 1.0080 / (Na * me);
    for (int i = 0; i < n_mols; ++i) {
        charge[3 * i] = -1.1128;
        charge[3 * i + 1] = charge[3 * i + 2] = 0.5564;
        for (int d = 0; d < 3; ++d) {
            mass[9 * i + d] = mo;
            mass[9 * i + d + 3] = mh;
            mass[9 * i + d + 6] = mh;
        }
    }
    for (int b = 0; b < n_beads; ++b) neighbour_list(q.data(), point.data(), list.data(), disp.data(), b);
    const bool spline = argc > 4 && std::strcmp(argv[4], "spline") == 0;
    const double tabs[3][3] = {{5e-3, 1.2, 7.0}, {-3e-3, 1.0, 5.5}, {2e-3, 0.8, 4.5}};  // A, lam, r_end
    std::vector<spline_t> spl;
    double cutsq[3];
    for (int t = 0; t < 3; ++t) {
        const int n = (int)std::lround(tabs[t][2] / 0.01) + 1;
        std::vector<double> y(n);
        for (int i = 0; i < n; ++i) {
            const double r = 0.01 * i, x = r / tabs[t][2];
            y[i] = tabs[t][0] * std::exp(-r / tabs[t][1]) * (1.0 - x * x) * (1.0 - x * x);
        }
        spl.emplace_back(y.begin(), y.end(), 0.0, 0.01);
        cutsq[t] = (0.01 * (n - 1)) * (0.01 * (n - 1));  // simulation.cpp:59-60
    }
    double sc_pot = 0.0, heat = 0.0;
    double e = spline ? force_eval_sc_wspline(q.data(), f.data(), charge.data(), mass.data(), point.data(),
                                              list.data(), spl[0], spl[1], spl[2], cutsq[0], cutsq[1], cutsq[2],
                                              sc_pot, fphys.data())
                      : force_eval_sc_nospline(q.data(), f.data(), charge.data(), mass.data(), point.data(),
                                               list.data(), sc_pot, fphys.data());
    std::printf("init %.15e %.15e\n", e, sc_pot);
    std::mt19937 rng((unsigned)std::atoi(argv[3]));
    const int n_steps = std::atoi(argv[2]);
    for (int s = 0; s < n_steps; ++s) {
        if (spline)
            e = update_sc_wspline(q.data(), p.data(), mass.data(), f.data(), fphys.data(), charge.data(),
                                  point.data(), list.data(), disp.data(), rng, true, heat, sc_pot, spl[0], spl[1],
                                  spl[2], cutsq[0], cutsq[1], cutsq[2]);
        else
            e = update_sc_nospline(q.data(), p.data(), mass.data(), f.data(), fphys.data(), charge.data(),
                                   point.data(), list.data(), disp.data(), rng, true, heat, sc_pot);
        std::printf("step %d %.15e %.15e %.15e %.15e\n", s, e, sc_pot, heat, get_kcv(q.data(), fphys.data()));
    }
    double qsum = 0.0, psum = 0.0;
    for (size_t i = 0; i < nt; ++i) {
        qsum += q[i] * (1.0 + 1e-3 * (double)(i % 7));
        psum += p[i] * (1.0 + 1e-3 * (double)(i % 5));
    }
    const double cons = get_conserved(q.data(), p.data(), mass.data(), e) + heat;
    std::printf("final %.15e %.15e %.15e\n", cons, qsum, psum);
    return 0;
}
