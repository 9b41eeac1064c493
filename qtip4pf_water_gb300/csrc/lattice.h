// Starting configurations of the reference's run driver (initialise.cpp), as
// host C++: the water fcc lattice (initialise.cpp:19-95), the proton-disordered
// ice Ih lattice obeying the ice rules with zero dipole moment
// (initialise.cpp:137-541) and positions read from a file
// (initialise.cpp:104-135). Header-only, so that the run driver can draw from
// its own std::mt19937 and the C ABI (lattice.cpp) can wrap the same code.
//
// The ice Ih construction consumes the generator exactly as the reference
// does -- one uniform_int_distribution<int>(0, 1) draw per O-O bond to place
// its hydrogen, then per proposed hydrogen hop one
// uniform_int_distribution<int>(0, 2 n_mols - 1) draw and, only when the hop
// leaves the coordination imbalance unchanged, one more (0, 1) draw -- so a
// seeded generator gives the reference's configuration.
#pragma once

#include <array>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <random>
#include <sstream>
#include <string>
#include <vector>

namespace qtg_lattice {

// Cell geometry (water.cpp:90-114): fcc holds 4 molecules a cell, the
// orthorhombic ice Ih cell 8; box = cells x cell sides (bohr).
struct Cells {
    int nx, ny, nz;
    double a, b, c;  // cell sides (bohr)
    double rnn;      // ice Ih O-O nearest-neighbour distance (bohr)
};

// qtip4pfparams.h:64-95 constants these lattices use
constexpr double ZO = 1.0 / 16.0;
constexpr double ONE_THIRD = 1.0 / 3.0;

inline Cells fcc_cells(int nx, int ny, int nz, double rho_g_cm3, double angs2bohr) {
    // mh2o = (2 m_H + m_O) / N_A in grams (qtip4pfparams.h:88)
    const double mh2o = (1.0080 * 2.0 + 15.9994) / 6.0221409e23;
    const double a = 1e8 * std::cbrt(4 * mh2o / rho_g_cm3) * angs2bohr;
    return Cells{nx, ny, nz, a, a, a, 0.0};
}

inline Cells orth_cells(int nx, int ny, int nz, double rho_g_cm3, double angs2bohr) {
    const double mh2o = (1.0080 * 2.0 + 15.9994) / 6.0221409e23;
    const double a = 1e8 * std::cbrt(4 * mh2o / (std::sqrt(2.0) * rho_g_cm3)) * angs2bohr;
    const double c = 2.0 * std::sqrt(2.0 / 3.0) * a;
    return Cells{nx, ny, nz, a, std::sqrt(3.0) * a, c, (0.5 - 2.0 * ZO) * c};
}

// Copies bead 0 into beads 1 .. P-1 (every bead starts identical).
inline void replicate_beads(double *pos, int n_beads, int n_dof) {
    for (int b = 1; b < n_beads; ++b)
        for (int i = 0; i < n_dof; ++i) pos[(size_t)b * n_dof + i] = pos[i];
}

// Water on the fcc lattice, every molecule in the same orientation: the O at
// the four fcc sites of each cell (cell order x, then y, then z innermost), the
// hydrogens at O + (dx, dx, +-dz), dx = r_eq cos(theta/2) / sqrt 2, dz = r_eq
// sin(theta/2). pos: double[n_beads][9 n_mols].
inline void fcc(const Cells &g, double roheq, double theta_eq, int n_beads, double *pos) {
    const double dx = roheq * std::cos(theta_eq / 2.0) / std::sqrt(2.0);
    const double dz = roheq * std::sin(theta_eq / 2.0);
    static const double frac[4][3] = {{0.25, 0.25, 0.25}, {0.25, 0.75, 0.75}, {0.75, 0.25, 0.75}, {0.75, 0.75, 0.25}};
    const int n_dof = 36 * g.nx * g.ny * g.nz;
    for (int i = 0; i < g.nx; ++i)
        for (int j = 0; j < g.ny; ++j)
            for (int k = 0; k < g.nz; ++k) {
                double *m = pos + 36 * (k + g.nz * j + g.nz * g.ny * i);
                for (int s = 0; s < 4; ++s) {
                    double *o = m + 9 * s;
                    o[0] = (i + frac[s][0]) * g.a;
                    o[1] = (j + frac[s][1]) * g.a;
                    o[2] = (k + frac[s][2]) * g.a;
                    o[3] = o[0] + dx;
                    o[4] = o[1] + dx;
                    o[5] = o[2] + dz;
                    o[6] = o[0] + dx;
                    o[7] = o[1] + dx;
                    o[8] = o[2] - dz;
                }
            }
    replicate_beads(pos, n_beads, n_dof);
}

// The eight oxygens of each orthorhombic ice Ih cell (two interleaved
// hexagonal layers), in cell units: x, y, z of oxygen s.
inline void ice_oxygen_frac(int s, double *f) {
    const double one_sixth = 0.5 * ONE_THIRD, two_thirds = 2.0 * ONE_THIRD, five_sixths = 5.0 / 6.0;
    const double t[8][3] = {{0.5, one_sixth, ZO},        {0.5, one_sixth, 0.5 - ZO},      {0.0, ONE_THIRD, 0.5 + ZO},
                            {0.0, ONE_THIRD, 1.0 - ZO},  {0.0, two_thirds, ZO},           {0.0, two_thirds, 0.5 - ZO},
                            {0.5, five_sixths, 0.5 + ZO}, {0.5, five_sixths, 1.0 - ZO}};
    for (int d = 0; d < 3; ++d) f[d] = t[s][d];
}

// The 2 n_mols O-O hydrogen bonds of the lattice (16 a cell): pairs (oxygen in
// this cell, oxygen in this or a neighbouring cell), as initialise.cpp:256-331
// enumerates them. Returns pairs of molecule indices.
inline std::vector<std::array<int, 2>> ice_bonds(const Cells &g) {
    auto cell = [&](int i, int j, int k) {
        i = (i + g.nx) % g.nx;
        j = (j + g.ny) % g.ny;
        k = (k + g.nz) % g.nz;
        return k + g.nz * j + g.nz * g.ny * i;
    };
    // (own oxygen, di, dj, dk, other oxygen) for the 16 bonds of a cell
    static const int T[16][5] = {{0, 0, 0, 0, 1},  {0, 0, 0, -1, 3}, {0, 1, 0, -1, 3}, {0, 0, -1, -1, 7},
                                 {1, 0, 0, 0, 2},  {1, 1, 0, 0, 2},  {1, 0, -1, 0, 6}, {2, 0, 0, 0, 3},
                                 {2, 0, 0, 0, 5},  {3, 0, 0, 1, 4},  {4, 0, 0, 0, 5},  {4, 0, 0, -1, 7},
                                 {4, -1, 0, -1, 7}, {5, 0, 0, 0, 6}, {5, -1, 0, 0, 6}, {6, 0, 0, 0, 7}};
    std::vector<std::array<int, 2>> bonds((size_t)16 * g.nx * g.ny * g.nz);
    for (int i = 0; i < g.nx; ++i)
        for (int j = 0; j < g.ny; ++j)
            for (int k = 0; k < g.nz; ++k) {
                const int c = cell(i, j, k);
                for (int t = 0; t < 16; ++t)
                    bonds[(size_t)16 * c + t] = {8 * c + T[t][0], 8 * cell(i + T[t][1], j + T[t][2], k + T[t][3]) + T[t][4]};
            }
    return bonds;
}

// Sum over molecules of the unit bisector of the two O-H vectors (minimum
// image by one box shift, as initialise.cpp:137-187).
inline std::array<double, 3> dipole(const double *pos, int n_mols, const double box[3]) {
    std::array<double, 3> mu{0.0, 0.0, 0.0};
    auto wrap = [&](double r, int d) {
        if (r <= -0.5 * box[d]) return r + box[d];
        if (r > 0.5 * box[d]) return r - box[d];
        return r;
    };
    for (int i = 0; i < n_mols; ++i) {
        double b[3];
        for (int d = 0; d < 3; ++d)
            b[d] = wrap(pos[9 * i + 3 + d] - pos[9 * i + d], d) + wrap(pos[9 * i + 6 + d] - pos[9 * i + d], d);
        const double n = std::sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
        for (int d = 0; d < 3; ++d) mu[d] += b[d] / n;
    }
    return mu;
}

// Proton-disordered ice Ih obeying the ice rules (every oxygen holds two
// hydrogens) with zero dipole moment (initialise.cpp:334-541): hydrogens placed
// at random along each O-O bond, r_eq from one of its oxygens, then single
// hydrogen hops between the two ends of a random bond that never increase the
// coordination imbalance |c_i - c_j| (equal imbalance: a coin decides) until
// the ice rules hold; the whole construction is redrawn until every dipole
// component is below 1e-10. Progress lines go to `log` as the reference writes
// them to output.txt. pos: double[n_beads][9 n_mols].
inline void ice_ih(const Cells &g, double roheq, int n_beads, std::mt19937 &rng, double *pos, std::ostream *log) {
    const int n_mols = 8 * g.nx * g.ny * g.nz, n_dof = 9 * n_mols;
    const double box[3] = {g.nx * g.a, g.ny * g.b, g.nz * g.c};
    for (size_t i = 0; i < (size_t)n_beads * n_dof; ++i) pos[i] = 0.0;
    for (int i = 0; i < g.nx; ++i)
        for (int j = 0; j < g.ny; ++j)
            for (int k = 0; k < g.nz; ++k) {
                const int c = k + g.nz * j + g.nz * g.ny * i;
                for (int s = 0; s < 8; ++s) {
                    double f[3];
                    ice_oxygen_frac(s, f);
                    pos[72 * c + 9 * s] = (i + f[0]) * g.a;
                    pos[72 * c + 9 * s + 1] = (j + f[1]) * g.b;
                    pos[72 * c + 9 * s + 2] = (k + f[2]) * g.c;
                }
            }
    const std::vector<std::array<int, 2>> bonds = ice_bonds(g);
    const int nb = 2 * n_mols;
    std::uniform_int_distribution<int> coin(0, 1);
    std::uniform_int_distribution<int> pick(0, nb - 1);
    std::vector<int> coord(n_mols), owner(nb);
    std::vector<double> hyd((size_t)3 * nb);
    // unit O-O vector (first minus second oxygen) of bond b, one box shift
    auto unit = [&](int b, double *u) {
        for (int d = 0; d < 3; ++d) {
            double r = pos[9 * bonds[b][0] + d] - pos[9 * bonds[b][1] + d];
            if (r <= -0.5 * box[d]) r += box[d];
            else if (r > 0.5 * box[d]) r -= box[d];
            u[d] = r / g.rnn;
        }
    };
    // hydrogen of bond b on its first (side 0) or second (side 1) oxygen
    auto place = [&](int b, int side) {
        double u[3];
        unit(b, u);
        const int o = bonds[b][side];
        const double sg = side == 0 ? -1.0 : 1.0;
        for (int d = 0; d < 3; ++d) hyd[3 * b + d] = pos[9 * o + d] + sg * roheq * u[d];
        owner[b] = o;
    };
    for (int outer = 1;; ++outer) {
        std::fill(coord.begin(), coord.end(), 0);
        for (int b = 0; b < nb; ++b) {
            const int side = coin(rng) ? 0 : 1;
            place(b, side);
            coord[bonds[b][side]] += 1;
        }
        for (int inner = 1;; ++inner) {
            bool ok = true;
            for (int m = 0; m < n_mols; ++m) ok = ok && coord[m] == 2;
            if (ok) {
                if (log) *log << "configuration found which satisfies the ice rules in " << inner << " iterations \n";
                break;
            }
            const int b = pick(rng);
            const int o1 = bonds[b][0], o2 = bonds[b][1];
            const int before = std::abs(coord[o1] - coord[o2]);
            const bool on_first = owner[b] == o1;
            const int after = std::abs(coord[o1] - coord[o2] + (on_first ? -2 : 2));
            if (after < before || (after == before && coin(rng) == 0)) {
                place(b, on_first ? 1 : 0);
                coord[on_first ? o2 : o1] += 1;
                coord[on_first ? o1 : o2] -= 1;
            }
        }
        // each oxygen's two hydrogens follow it, in bond order
        std::vector<int> held(n_mols, 0);
        for (int b = 0; b < nb; ++b) {
            const int o = owner[b];
            held[o] += 1;
            for (int d = 0; d < 3; ++d) pos[9 * o + 3 * held[o] + d] = hyd[3 * b + d];
        }
        const std::array<double, 3> mu = dipole(pos, n_mols, box);
        if (log) *log << "dipole moment is " << mu[0] << " " << mu[1] << " " << mu[2] << "\n";
        if (std::fabs(mu[0]) < 1e-10 && std::fabs(mu[1]) < 1e-10 && std::fabs(mu[2]) < 1e-10) {
            if (log) *log << "configuration found that has zero dipole moment in " << outer << " outer iterations \n";
            break;
        }
    }
    replicate_beads(pos, n_beads, n_dof);
}

// Positions from a text file of "x y z" lines, one atom a line (O, H1, H2 of
// each molecule in turn; blank lines skipped), into bead 0, copied to every
// bead. Returns the number of atoms read.
inline int from_file(const std::string &name, int n_beads, int n_dof, double *pos) {
    std::ifstream in(name);
    std::string line;
    int count = 0;
    while (std::getline(in, line)) {
        if (line.empty()) continue;
        if (3 * count + 2 >= n_dof) break;
        std::stringstream ss(line);
        for (int d = 0; d < 3; ++d) ss >> pos[3 * count + d];
        ++count;
    }
    replicate_beads(pos, n_beads, n_dof);
    return count;
}

}  // namespace qtg_lattice
