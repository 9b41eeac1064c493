// C ABI of the starting-configuration builders (lattice.h).
#include "../../include/qtip4pf_gb300.h"

#include <cmath>

#include "lattice.h"

namespace {
qtg_constants K() {
    qtg_constants k;
    qtg_get_constants(&k);
    return k;
}
}  // namespace

extern "C" qtg_status qtg_lattice_fcc(int nx, int ny, int nz, double rho_g_cm3, int n_beads, double *pos,
                                      double *box_bohr) {
    if (nx < 1 || ny < 1 || nz < 1 || !(rho_g_cm3 > 0) || n_beads < 1 || !pos) return QTG_ERR_ARG;
    const qtg_constants k = K();
    const qtg_lattice::Cells g = qtg_lattice::fcc_cells(nx, ny, nz, rho_g_cm3, k.angs2bohr);
    qtg_lattice::fcc(g, k.roheq, k.theta_eq, n_beads, pos);
    if (box_bohr) {
        box_bohr[0] = nx * g.a;
        box_bohr[1] = ny * g.b;
        box_bohr[2] = nz * g.c;
    }
    return QTG_OK;
}

extern "C" qtg_status qtg_lattice_ice_ih(int nx, int ny, int nz, double rho_g_cm3, int n_beads, unsigned int seed,
                                         double *pos, double *box_bohr) {
    if (nx < 1 || ny < 1 || nz < 1 || !(rho_g_cm3 > 0) || n_beads < 1 || !pos) return QTG_ERR_ARG;
    const qtg_constants k = K();
    const qtg_lattice::Cells g = qtg_lattice::orth_cells(nx, ny, nz, rho_g_cm3, k.angs2bohr);
    std::mt19937 rng(seed);
    qtg_lattice::ice_ih(g, k.roheq, n_beads, rng, pos, nullptr);
    if (box_bohr) {
        box_bohr[0] = nx * g.a;
        box_bohr[1] = ny * g.b;
        box_bohr[2] = nz * g.c;
    }
    return QTG_OK;
}
