// End-to-end timing of the per-call step through the C ABI from host C++, as a
// C++ host program (the reference's language) calls it: qtg_update_pimd -- the
// update_sc_nospline entry -- once per step on the caller's host arrays, which
// the program registers with the library once (qtg_register_host), so that each
// call moves them inside its step graph; the L2 cache is flushed before every
// call (outside the timer). Second-order PIMD with PILE-G, the thermostat's
// noise drawn on the device (noise = NULL), mixed precision, launch shapes
// autotuned once at set-up.
//
// usage: e2e_bench <start.bin> <warmup> <steps> <seed>
// start.bin: int32 n_mols, int32 n_beads, double box[3], double T_K, double dt_fs,
//            double eps_ewald, double eps_sc, then q[P][9N], p[P][9N] (doubles)
// Prints one line: mean_ms min_ms h2d_bytes_per_call d2h_bytes_per_call launches_per_call
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../../include/qtip4pf_gb300.h"

namespace {

// page-aligned host memory for an array of n elements (registered below)
template <typename T>
T *host_array(size_t n) {
    void *p = nullptr;
    const size_t bytes = ((n * sizeof(T) + 4095) / 4096) * 4096;
    if (posix_memalign(&p, 4096, bytes) != 0) return nullptr;
    std::memset(p, 0, bytes);
    return static_cast<T *>(p);
}

int fail(qtg_ctx *ctx, qtg_status st, const char *what) {
    std::fprintf(stderr, "e2e_bench: %s: %s (%s)\n", what, qtg_status_string(st), qtg_last_error(ctx));
    return 1;
}

}  // namespace

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
    const int N = hdr[0], P = hdr[1];
    const size_t nt = (size_t)P * 9 * N, nd = (size_t)P * 3 * N;
    qtg_system_desc d;
    std::memset(&d, 0, sizeof(d));
    d.n_mols = N;
    d.n_beads = P;
    for (int k = 0; k < 3; ++k) d.box_bohr[k] = par[k];
    d.temp_K = par[3];
    d.dt_fs = par[4];
    d.eps_ewald = par[5];
    d.eps_sc = par[6];
    d.propagator = QTG_TROTTER;
    d.thermostat = QTG_THERMO_PILE_G;
    d.seed = (uint64_t)std::strtoull(argv[4], nullptr, 10);
    qtg_ctx *ctx = nullptr;
    qtg_status st = qtg_create(&d, 1, QTG_MIXED, &ctx);
    if (st != QTG_OK) return fail(ctx, st, "qtg_create");
    qtg_system_info info;
    qtg_system_info_get(ctx, 0, &info);
    double *q = host_array<double>(nt), *p = host_array<double>(nt), *f = host_array<double>(nt);
    double *fphys = host_array<double>(nt), *disp = host_array<double>(nd);
    int *point = host_array<int>((size_t)P * N), *list = host_array<int>((size_t)P * info.list_size);
    if (!q || !p || !f || !fphys || !disp || !point || !list) return 5;
    if (std::fread(q, sizeof(double), nt, fp) != nt || std::fread(p, sizeof(double), nt, fp) != nt) return 6;
    std::fclose(fp);
    // the five state arrays are registered once; masses, charges, lists stay plain
    double *arr[5] = {q, p, f, fphys, disp};
    const size_t len[5] = {nt, nt, nt, nt, nd};
    for (int k = 0; k < 5; ++k)
        if ((st = qtg_register_host(arr[k], len[k] * sizeof(double))) != QTG_OK) return fail(ctx, st, "register");
    std::vector<double> mass(9 * (size_t)N), charge(3 * (size_t)N);
    qtg_constants K;
    qtg_get_constants(&K);
    for (int i = 0; i < N; ++i) {
        charge[3 * i] = K.qo;
        charge[3 * i + 1] = charge[3 * i + 2] = K.qh;
        for (int a = 0; a < 3; ++a)
            for (int k = 0; k < 3; ++k) mass[9 * i + 3 * a + k] = a == 0 ? K.mo : K.mh;
    }
    // launch shapes tuned once at set-up on the start, then the first forces and lists
    if ((st = qtg_set_state(ctx, 0, q, p)) != QTG_OK) return fail(ctx, st, "set_state");
    double t_h = 0.0, t_t = 0.0;
    if ((st = qtg_autotune(ctx, 10, &t_h, &t_t)) != QTG_OK) return fail(ctx, st, "autotune");
    for (int b = 0; b < P; ++b)
        if ((st = qtg_neighbour_list(ctx, 0, q, point, list, disp, b)) != QTG_OK) return fail(ctx, st, "lists");
    double pot = 0.0, energy = 0.0, heat = 0.0;
    if ((st = qtg_force_eval_trotter(ctx, 0, q, f, charge.data(), point, list, &pot, &energy)) != QTG_OK)
        return fail(ctx, st, "forces");
    std::memcpy(fphys, f, nt * sizeof(double));
    const int warm = std::atoi(argv[2]), steps = std::atoi(argv[3]);
    for (int s = 0; s < warm; ++s)
        if ((st = qtg_update_pimd(ctx, 0, q, p, mass.data(), f, fphys, charge.data(), point, list, disp, 1, nullptr,
                                  &heat, &pot, &energy)) != QTG_OK)
            return fail(ctx, st, "update");
    unsigned long long h0 = 0, d0 = 0, h1 = 0, d1 = 0;
    uint64_t l0 = 0, l1 = 0;
    qtg_transfer_bytes(ctx, &h0, &d0);
    qtg_kernel_launches(ctx, &l0);
    double tot = 0.0, best = 1e30;
    for (int s = 0; s < steps; ++s) {
        if ((st = qtg_flush_l2(ctx)) != QTG_OK) return fail(ctx, st, "flush");
        const auto t0 = std::chrono::steady_clock::now();
        st = qtg_update_pimd(ctx, 0, q, p, mass.data(), f, fphys, charge.data(), point, list, disp, 1, nullptr, &heat,
                             &pot, &energy);
        const double ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
        if (st != QTG_OK) return fail(ctx, st, "update");
        tot += ms;
        best = std::min(best, ms);
    }
    qtg_transfer_bytes(ctx, &h1, &d1);
    qtg_kernel_launches(ctx, &l1);
    if (!std::isfinite(energy)) return 7;
    std::printf("%.6f %.6f %llu %llu %.1f\n", tot / steps, best, (h1 - h0) / steps, (d1 - d0) / steps,
                (double)(l1 - l0) / steps);
    qtg_destroy(ctx);
    return 0;
}
