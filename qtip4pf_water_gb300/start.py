"""Seeded synthetic starting states for qTIP4P/F water systems.

The reference builds its start from an fcc / ice lattice with identical or
ice-rule orientations and copies bead 0 to every bead (initialise.cpp:20-98,
:107-135). The workloads here instead need cubic boxes of 64..4096 waters, so
this module makes its own start, deterministically from a 64-bit seed:

* waters on an m^3 simple-cubic grid at the cell centres of a cubic box sized
  for 0.997 g/cm^3 (m = ceil(N^(1/3)); when N is not a cube the lowest-index N
  grid sites are used, x varying fastest);
* each molecule at the qTIP4P/F equilibrium geometry (r_OH = 0.9419 A,
  HOH = 107.4 deg) with the O atom on its grid site and a uniformly random
  orientation (normalised 4-D Gaussian quaternion);
* ring-polymer beads at the centroid plus free-ring-polymer Gaussian
  normal-mode displacements of variance 1 / (beta_P m omega_k^2), omega_k =
  (2 / beta_P hbar) sin(k pi / P), in the orthonormal normal-mode convention of
  fourier.cpp:12-69;
* Maxwell-Boltzmann momenta of standard deviation sqrt(m / beta_P) for every
  bead (simulation.cpp:826-827, :847-858), with the mean momentum per atom
  removed over the whole extended system (simulation.cpp:859-871).

Randomness comes from SplitMix64 and Box-Muller written out here, so the same
seed gives the same arrays on every machine and numpy version.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# unit conversions as the reference defines them (qtip4pfparams.h:45-61)
PI_REF = 3.14159265359
ANGS2BOHR = 1.0 / 0.529177210903
_ME = 9.10938356e-31
_KB = 1.38064852e-23
_NA = 6.0221409e23
_EH = 4.3597447222071e-18
MO = 0.001 * 15.9994 / (_NA * _ME)
MH = 0.001 * 1.0080 / (_NA * _ME)
K2AU = _KB / _EH
FS2AU = 1.0 / (1.054571817e-34 * 1e15 / _EH)
MH2O_G = (1.0080 * 2.0 + 15.9994) / _NA

R_OH_ANG = 0.9419
THETA_HOH_DEG = 107.4

_GOLDEN = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


class SplitMix64:
    """Counter-based SplitMix64 stream (Steele, Lea & Flood 2014)."""

    def __init__(self, seed: int):
        self.state = np.uint64(seed & 0xFFFFFFFFFFFFFFFF)

    def u64(self, n: int) -> np.ndarray:
        with np.errstate(over="ignore"):
            z = self.state + _GOLDEN * np.arange(1, n + 1, dtype=np.uint64)
            self.state = self.state + _GOLDEN * np.uint64(n)
            z = (z ^ (z >> np.uint64(30))) * _M1
            z = (z ^ (z >> np.uint64(27))) * _M2
            z = z ^ (z >> np.uint64(31))
        return z

    def uniform(self, n: int) -> np.ndarray:
        """Uniform doubles in the open interval (0, 1)."""
        return ((self.u64(n) >> np.uint64(11)).astype(np.float64) + 0.5) * (2.0 ** -53)

    def normal(self, n: int) -> np.ndarray:
        m = (n + 1) // 2
        u1 = self.uniform(m)
        u2 = self.uniform(m)
        rad = np.sqrt(-2.0 * np.log(u1))
        z = np.concatenate([rad * np.cos(2.0 * math.pi * u2), rad * np.sin(2.0 * math.pi * u2)])
        return z[:n]


def box_length_angstrom(n_mols: int, density_g_cm3: float = 0.997) -> float:
    """Edge of the cubic box holding n_mols waters at the given density."""
    return 1e8 * (n_mols * MH2O_G / density_g_cm3) ** (1.0 / 3.0)


def grid_side(n_mols: int) -> int:
    m = 1
    while m * m * m < n_mols:
        m += 1
    return m


def nm_matrix(n_beads: int) -> np.ndarray:
    """Orthonormal bead -> normal-mode matrix C (y = C x) in halfcomplex order."""
    P = n_beads
    C = np.zeros((P, P))
    b = np.arange(P)
    C[0, :] = math.sqrt(1.0 / P)
    for k in range(1, (P + 1) // 2):
        ang = 2.0 * math.pi * ((b * k) % P) / P
        C[k, :] = math.sqrt(2.0 / P) * np.cos(ang)
        C[P - k, :] = -math.sqrt(2.0 / P) * np.sin(ang)
    if P % 2 == 0 and P > 1:
        C[P // 2, :] = math.sqrt(1.0 / P) * np.where(b % 2 == 0, 1.0, -1.0)
    return C


@dataclass
class WaterStart:
    n_mols: int
    n_beads: int
    box_bohr: np.ndarray  # (3,)
    q: np.ndarray  # (P, 9N) bohr
    p: np.ndarray  # (P, 9N) a.u.
    temp_K: float
    seed: int


def seeded_start(n_mols: int, n_beads: int = 1, temp_K: float = 298.0, seed: int = 1,
                 box_angstrom: float | None = None, density_g_cm3: float = 0.997,
                 bead_spread: bool = True) -> WaterStart:
    """Deterministic start for n_mols waters and n_beads beads (see module doc)."""
    rng = SplitMix64(seed)
    L_ang = box_angstrom if box_angstrom is not None else box_length_angstrom(n_mols, density_g_cm3)
    L = L_ang * ANGS2BOHR
    m = grid_side(n_mols)
    idx = np.arange(n_mols)
    ix, iy, iz = idx % m, (idx // m) % m, idx // (m * m)
    sites = (np.stack([ix, iy, iz], axis=1) + 0.5) * (L / m)

    # body frame: O at the origin, H atoms in the xz plane
    r = R_OH_ANG * ANGS2BOHR
    half = 0.5 * THETA_HOH_DEG * math.pi / 180.0
    body = np.array([[0.0, 0.0, 0.0],
                     [r * math.sin(half), 0.0, r * math.cos(half)],
                     [-r * math.sin(half), 0.0, r * math.cos(half)]])
    quat = rng.normal(4 * n_mols).reshape(n_mols, 4)
    quat /= np.linalg.norm(quat, axis=1, keepdims=True)
    w, x, y, z = quat.T
    R = np.empty((n_mols, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    atoms = sites[:, None, :] + np.einsum("nij,aj->nai", R, body)  # (N, 3, 3)
    centroid = atoms.reshape(-1)  # (9N,)

    P = n_beads
    beta_n = 1.0 / (K2AU * temp_K) / P
    mass = np.tile(np.repeat(np.array([MO, MH, MH]), 3), n_mols)  # (9N,)
    q = np.tile(centroid, (P, 1))
    if P > 1 and bead_spread:
        C = nm_matrix(P)
        Q = np.zeros((P, 9 * n_mols))
        Q[0] = math.sqrt(P) * centroid
        # displacement is per atom (the same random draw is not shared across dims)
        for k in range(1, P):
            wk = (2.0 / beta_n) * math.sin(k * math.pi / P)
            Q[k] = rng.normal(9 * n_mols) / np.sqrt(beta_n * mass * wk * wk)
        q = C.T @ Q
    p = rng.normal(P * 9 * n_mols).reshape(P, 9 * n_mols) * np.sqrt(mass / beta_n)[None, :]
    pc = p.reshape(P, n_mols * 3, 3).sum(axis=(0, 1)) / (3 * n_mols * P)
    p = (p.reshape(P, n_mols * 3, 3) - pc[None, None, :]).reshape(P, 9 * n_mols)
    return WaterStart(n_mols, P, np.array([L, L, L]), np.ascontiguousarray(q),
                      np.ascontiguousarray(p), temp_K, seed)


def spread_beads(centroid: np.ndarray, n_beads: int, temp_K: float = 298.0, seed: int = 1):
    """Beads around a given centroid configuration (double[9N]): the centroid
    normal mode is the given centroid, modes k >= 1 are free-ring-polymer
    Gaussian displacements at temp_K, bead momenta Maxwell-Boltzmann at the bead
    temperature. Returns (q, p), each double[P][9N]."""
    rng = SplitMix64(seed)
    c = np.asarray(centroid, dtype=np.float64).reshape(-1)
    n_mols = c.size // 9
    P = n_beads
    beta_n = 1.0 / (K2AU * temp_K) / P
    mass = np.tile(np.repeat(np.array([MO, MH, MH]), 3), n_mols)
    Q = np.zeros((P, c.size))
    Q[0] = math.sqrt(P) * c
    for k in range(1, P):
        wk = (2.0 / beta_n) * math.sin(k * math.pi / P)
        Q[k] = rng.normal(c.size) / np.sqrt(beta_n * mass * wk * wk)
    q = nm_matrix(P).T @ Q
    p = rng.normal(P * c.size).reshape(P, c.size) * np.sqrt(mass / beta_n)[None, :]
    return np.ascontiguousarray(q), np.ascontiguousarray(p)


def default_charges(n_mols: int) -> np.ndarray:
    """Per-site charges (M, H1, H2) as simulation.cpp:811-816 sets them."""
    qo = -1.1128
    return np.tile(np.array([qo, -0.5 * qo, -0.5 * qo]), n_mols)


def default_masses(n_mols: int) -> np.ndarray:
    """Per-degree-of-freedom masses as simulation.cpp:817-821 sets them."""
    return np.tile(np.repeat(np.array([MO, MH, MH]), 3), n_mols)
