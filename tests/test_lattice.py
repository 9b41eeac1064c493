"""Starting configurations (initialise.cpp) from the library's host builders
against the reference's own initialise_fcc / initialise_orth (fixtures made by
tests/golden/make_lattice_golden.py): bit-identical positions and boxes, and
for ice Ih the same seeded draws -- so the same configuration -- as the
reference; plus the ice rules and the zero dipole moment themselves."""
import ctypes as C
import os

import numpy as np
import pytest

from conftest import GOLDEN

Z = np.load(os.path.join(GOLDEN, "lattice", "lattice.npz"))
CASES = sorted({k.split("__")[0] for k in Z.files})
D = C.POINTER(C.c_double)


def lib():
    import qtip4pf_water_gb300 as q

    L = q.load()
    L.qtg_lattice_fcc.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, D, D]
    L.qtg_lattice_ice_ih.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_uint, D, D]
    return L


@pytest.mark.parametrize("case", CASES)
def test_lattice_matches_the_reference(case):
    L = lib()
    nx, ny, nz, orth, seed = (int(v) for v in Z[case + "__spec"])
    rho = float(Z[case + "__rho"])
    ref = Z[case + "__pos"]
    n = ref.size // 9
    P = 3
    pos = np.zeros(P * 9 * n)
    box = np.zeros(3)
    if orth:
        st = L.qtg_lattice_ice_ih(nx, ny, nz, rho, P, seed, pos.ctypes.data_as(D), box.ctypes.data_as(D))
    else:
        st = L.qtg_lattice_fcc(nx, ny, nz, rho, P, pos.ctypes.data_as(D), box.ctypes.data_as(D))
    assert st == 0
    assert np.array_equal(box, Z[case + "__box"])
    assert np.array_equal(pos[: 9 * n], ref)
    for b in range(1, P):
        assert np.array_equal(pos[b * 9 * n:(b + 1) * 9 * n], ref)
    if orth:
        x = ref.reshape(n, 3, 3)
        bx = Z[case + "__box"]
        d = x[:, 1:, :] - x[:, :1, :]
        d -= bx * np.round(d / bx)
        r = np.linalg.norm(d, axis=-1)
        # every oxygen holds two hydrogens at the equilibrium bond length
        np.testing.assert_allclose(r, 0.9419 / 0.529177210903, rtol=1e-12)
        bis = d.sum(axis=1)
        mu = (bis / np.linalg.norm(bis, axis=-1, keepdims=True)).sum(axis=0)
        assert np.abs(mu).max() < 1e-10


def test_bad_arguments():
    L = lib()
    pos = np.zeros(72)
    assert L.qtg_lattice_fcc(0, 1, 1, 1.0, 1, pos.ctypes.data_as(D), None) == 1
    assert L.qtg_lattice_ice_ih(1, 1, 1, -1.0, 1, 3, pos.ctypes.data_as(D), None) == 1
