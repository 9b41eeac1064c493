// End-to-end timing of the drop-in as the reference's run driver uses it: the
// sampling loop of run_sc_nospline (simulation.cpp:936-961) -- update_sc_nospline
// once per step on the caller's new[] arrays with the caller's std::mt19937 --
// linked against libqtip_compat.so. The thermostat's normal draws are made on
// the host from that generator, as thermostat.cpp makes them, so the time
// includes them; the arrays are plain heap memory that the drop-in registers
// with the library on its first call.
//
// usage: dropin_bench <start.bin> <warmup> <steps> <seed>
// start.bin: int32 n_mols, int32 n_beads, double box[3], double T_K, double dt_fs,
//            double eps_ewald, double eps_sc, then q[P][9N], p[P][9N] (doubles)
// Prints one line: ms_per_step draw_ms_per_step n_beads n_mols
#include <array>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

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

// the reference's interface (neighbour.h, forces.h, update.h)
void neighbour_list(const double position_array[], int point[], int list[], double disp_array[], int bead);
double force_eval_sc_nospline(const double position_array[], double force_array[], const double charge_array[],
                              const double mass_array[], const int point[], const int list[], double &sc_pot,
                              double fphys[]);
double update_sc_nospline(double position_array[], double momentum_array[], const double mass_array[],
                          double force_array[], double fphys[], double charge_array[], int point[], int list[],
                          double disp_array[], std::mt19937 &rng, bool is_nvt, double &heat, double &sc_pot);

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr, "usage: %s start.bin warmup steps seed\n", argv[0]);
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
    // the derived globals the drop-in reads, as water.cpp:76-157 derives them
    const double r_skin = 1.30 * 9.0 / 0.529177210903;
    n_atoms = 3 * n_mols;
    n_dof = 3 * n_atoms;
    vol = boxl[0] * boxl[1] * boxl[2];
    rho_ox = n_mols / vol;
    list_size = (int)std::round(4.0 * r_skin * r_skin * r_skin * n_mols * rho_ox);
    const size_t nt = (size_t)n_beads * n_dof;
    // the reference's state arrays: plain heap memory (simulation.cpp:797-805)
    double *q = new double[nt], *p = new double[nt], *f = new double[nt], *fphys = new double[nt];
    double *disp = new double[(size_t)n_beads * 3 * n_mols]();
    int *point = new int[(size_t)n_beads * n_mols], *list = new int[(size_t)n_beads * list_size];
    double *charge = new double[n_atoms], *mass = new double[n_dof];
    if (std::fread(q, sizeof(double), nt, fp) != nt || std::fread(p, sizeof(double), nt, fp) != nt) return 5;
    std::fclose(fp);
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
    for (int b = 0; b < n_beads; ++b) neighbour_list(q, point, list, disp, b);
    double sc_pot = 0.0, heat = 0.0;
    force_eval_sc_nospline(q, f, charge, mass, point, list, sc_pot, fphys);
    std::mt19937 rng((unsigned)std::atoi(argv[4]));
    const int warm = std::atoi(argv[2]), steps = std::atoi(argv[3]);
    for (int s = 0; s < warm; ++s)
        update_sc_nospline(q, p, mass, f, fphys, charge, point, list, disp, rng, true, heat, sc_pot);
    const auto t0 = std::chrono::steady_clock::now();
    for (int s = 0; s < steps; ++s)
        update_sc_nospline(q, p, mass, f, fphys, charge, point, list, disp, rng, true, heat, sc_pot);
    const auto t1 = std::chrono::steady_clock::now();
    // the host draws alone (the same distributions and count as one step's pile_g)
    std::mt19937 g2((unsigned)std::atoi(argv[4]) + 1u);
    std::normal_distribution<double> gauss(0.0, 1.0);
    double sink = 0.0;
    const auto t2 = std::chrono::steady_clock::now();
    for (int s = 0; s < steps; ++s)
        for (size_t k = 0; k < (size_t)(n_beads - 1) * n_dof + 2; ++k) sink += gauss(g2);
    const auto t3 = std::chrono::steady_clock::now();
    const double ms = std::chrono::duration<double, std::milli>(t1 - t0).count() / steps;
    const double draw_ms = std::chrono::duration<double, std::milli>(t3 - t2).count() / steps;
    std::printf("%.6f %.6f %d %d %s\n", ms, draw_ms, n_beads, n_mols, std::isfinite(sink + heat) ? "ok" : "nonfinite");
    return 0;
}
