"""Seeded synthetic starts: determinism, geometry and momentum statistics (CPU)."""
import math

import numpy as np
import pytest

from qtip4pf_water_gb300.start import (ANGS2BOHR, K2AU, MH, MO, SplitMix64, box_length_angstrom, nm_matrix,
                                       seeded_start)


def _splitmix_scalar(seed, n):
    """Scalar SplitMix64 with Python integers (independent of the vectorised numpy form)."""
    m = (1 << 64) - 1
    x, out = seed, []
    for _ in range(n):
        x = (x + 0x9E3779B97F4A7C15) & m
        z = x
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & m
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & m
        out.append(z ^ (z >> 31))
    return out


def test_splitmix_matches_scalar_form():
    r = SplitMix64(1234567)
    first = [int(x) for x in r.u64(5)]
    second = [int(x) for x in r.u64(3)]
    assert first + second == _splitmix_scalar(1234567, 8)


def test_box_lengths():
    assert abs(box_length_angstrom(216) - 18.64) < 0.01
    assert abs(box_length_angstrom(512) - 24.85) < 0.01
    assert abs(box_length_angstrom(4096) - 49.7) < 0.02


@pytest.mark.parametrize("P", [1, 2, 3, 8, 32])
def test_nm_matrix_orthonormal(P):
    C = nm_matrix(P)
    np.testing.assert_allclose(C @ C.T, np.eye(P), atol=1e-14)


def test_deterministic_and_geometry():
    a = seeded_start(64, 4, 298.0, seed=5)
    b = seeded_start(64, 4, 298.0, seed=5)
    c = seeded_start(64, 4, 298.0, seed=6)
    assert np.array_equal(a.q, b.q) and np.array_equal(a.p, b.p)
    assert not np.array_equal(a.q, c.q)
    s = seeded_start(216, 1, 298.0, seed=3)
    x = s.q[0].reshape(216, 3, 3)
    r1 = np.linalg.norm(x[:, 1] - x[:, 0], axis=1) / ANGS2BOHR
    r2 = np.linalg.norm(x[:, 2] - x[:, 0], axis=1) / ANGS2BOHR
    np.testing.assert_allclose(r1, 0.9419, rtol=1e-12)
    np.testing.assert_allclose(r2, 0.9419, rtol=1e-12)
    cosang = np.sum((x[:, 1] - x[:, 0]) * (x[:, 2] - x[:, 0]), axis=1) / (r1 * r2 * ANGS2BOHR ** 2)
    np.testing.assert_allclose(np.degrees(np.arccos(cosang)), 107.4, atol=1e-9)


def test_momenta_and_bead_spread_statistics():
    P, N, T = 8, 512, 298.0
    s = seeded_start(N, P, T, seed=9)
    beta_n = 1.0 / (K2AU * T) / P
    mass = np.tile(np.repeat([MO, MH, MH], 3), N)
    # no net momentum of the extended system
    assert np.abs(s.p.reshape(-1, 3).sum(axis=0)).max() < 1e-9
    z = (s.p / np.sqrt(mass / beta_n)).ravel()
    assert abs(z.std() - 1.0) < 0.01
    # normal-mode coordinates of the bead displacements have variance 1/(beta_n m w_k^2)
    Q = nm_matrix(P) @ s.q
    for k in (1, P // 2):
        wk = (2.0 / beta_n) * math.sin(k * math.pi / P)
        zk = Q[k] * np.sqrt(beta_n * mass * wk * wk)
        assert abs(zk.std() - 1.0) < 0.03
