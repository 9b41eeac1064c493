"""Pins the C oracle to the reference's own compiled sources.

Every fixture in tests/golden was produced by running the reference's
forces.cpp / neighbour.cpp / fourier.cpp / update.cpp / thermostat.cpp /
path_integrals.cpp (built by `make -C oracle ref`) on seeded inputs; see
tests/golden/make_golden.py. Integer outputs (neighbour lists) must match
bit for bit; FP64 outputs to round-off.
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden
from oracle.binding import Oracle

CASES = golden_cases()
RTOL_F = 1e-11  # FP64 round-off of a differently ordered sum


def make(g):
    return Oracle(int(g["n_mols"]), int(g["n_beads"]), g["box"], float(g["temp_K"]), float(g["dt_fs"]),
                  float(g["eps_ewald"]), float(g["eps_sc"]))


def rel_rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


@pytest.mark.parametrize("case", CASES)
def test_parameters(case):
    g = load_golden(case)
    o = make(g)
    par = g["ewald_params"]
    assert o.s.kappa == par[0]
    assert o.s.rc_sq == par[1] * par[1]
    assert o.s.k_max == int(par[3])
    assert o.list_size == int(g["list_size"]) == int(par[4])
    assert o.s.dt == par[5] and o.s.beta_n == par[6] and o.s.omega_psq == par[7]


@pytest.mark.parametrize("case", CASES)
def test_neighbour_list_bit_exact(case):
    g = load_golden(case)
    o = make(g)
    point, lst, disp = o.new_lists()
    disp[:] = 1.0
    for b in range(o.P):
        n = o.neighbour_list(g["q"], point, lst, disp, b)
        assert n >= 0
    assert np.array_equal(point, g["point"])
    assert np.array_equal(lst, g["list"])
    assert not disp.any()


@pytest.mark.parametrize("case", CASES)
def test_single_configuration_forces(case):
    g = load_golden(case)
    o = make(g)
    f = np.zeros_like(g["forces"])
    e = np.array([o.get_forces(g["q"], f, g["point"], g["list"], b) for b in range(o.P)])
    np.testing.assert_allclose(e, g["energies"], rtol=1e-12, atol=1e-12)
    assert rel_rms(f, g["forces"]) < RTOL_F
    np.testing.assert_allclose(f, g["forces"], rtol=0, atol=1e-11 * np.abs(g["forces"]).max())


@pytest.mark.parametrize("case", CASES)
def test_kwald(case):
    g = load_golden(case)
    o = make(g)
    f = np.zeros_like(g["kw_forces"])
    e = o.kwald(np.ascontiguousarray(g["kw_sites"]), f)
    assert abs(e - float(g["kw_energy"])) <= 1e-12 * abs(float(g["kw_energy"]))
    assert rel_rms(f, g["kw_forces"]) < RTOL_F


@pytest.mark.parametrize("case", [c for c in CASES if c.endswith("_p1")])
def test_velocity_verlet_steps(case):
    g = load_golden(case)
    o = make(g)
    q, p, f = g["q"].copy(), g["p"].copy(), g["forces"].copy()
    point, lst, disp = g["point"].copy(), g["list"].copy(), np.zeros(3 * o.N)
    es = [o.update_class(q, p, f, point, lst, disp) for _ in range(3)]
    np.testing.assert_allclose(es, g["vv_energy"], rtol=1e-11, atol=1e-12)
    assert rel_rms(q, g["vv_q"]) < 1e-14
    assert rel_rms(p, g["vv_p"]) < 1e-11
    assert rel_rms(f, g["vv_f"]) < RTOL_F


PIMD = [c for c in CASES if not c.endswith("_p1") and "_p1_" not in c]


@pytest.mark.parametrize("case", PIMD)
def test_suzuki_chin_forces(case):
    g = load_golden(case)
    o = make(g)
    f = np.zeros_like(g["sc_f"])
    fp = np.zeros_like(g["sc_fphys"])
    e, scp = o.force_eval_sc(g["q"], f, g["point"], g["list"], fp)
    assert abs(e - float(g["sc_energy"])) <= 1e-11 * abs(float(g["sc_energy"])) + 1e-12
    assert abs(scp - float(g["sc_pot"])) <= 1e-11 * abs(float(g["sc_pot"])) + 1e-12
    assert rel_rms(fp, g["sc_fphys"]) < RTOL_F
    # the finite-difference force-gradient term amplifies round-off by ~1/eps_sc
    assert rel_rms(f, g["sc_f"]) < 1e-8


@pytest.mark.parametrize("case", PIMD)
def test_normal_mode_transform(case):
    g = load_golden(case)
    o = make(g)
    a = g["q"].copy()
    o.ftransform(a, 9 * o.N, True)
    np.testing.assert_allclose(a, g["nm_fwd"], rtol=0, atol=1e-12 * np.abs(g["nm_fwd"]).max())
    o.ftransform(a, 9 * o.N, False)
    np.testing.assert_allclose(a, g["nm_roundtrip"], rtol=0, atol=1e-12 * np.abs(g["q"]).max())
    d = g["nm3_in"].copy()
    o.ftransform(d, 3 * o.N, True)
    np.testing.assert_allclose(d, g["nm3_fwd"], rtol=0, atol=1e-13 * np.abs(d).max())


@pytest.mark.parametrize("case", CASES)
def test_bussi_with_recorded_noise(case):
    """thermostat.cpp:12-60 (global rescale of the first n_dof momenta)."""
    g = load_golden(case)
    o = make(g)
    p = g["bussi_p_in"].copy()
    heat = o.bussi(p, g["bussi_noise"])
    np.testing.assert_allclose(p, g["bussi_p_out"], rtol=1e-13, atol=1e-13 * np.abs(p).max())
    ke = 0.5 * float(np.sum(g["bussi_p_in"][: 9 * o.N] ** 2 / np.repeat(o.mass[0::3], 3)))
    assert abs(heat - float(g["bussi_heat"])) <= 1e-12 * ke


@pytest.mark.parametrize("case", PIMD)
def test_pile_g_with_recorded_noise(case):
    g = load_golden(case)
    o = make(g)
    p = g["pile_p_in"].copy()
    heat = o.pile_g(p, g["pile_noise"])
    np.testing.assert_allclose(p, g["pile_p_out"], rtol=1e-13, atol=1e-13 * np.abs(p).max())
    assert abs(heat - float(g["pile_heat"])) <= 1e-10 * abs(float(g["pile_heat"])) + 1e-12


@pytest.mark.parametrize("case", PIMD)
def test_estimators(case):
    g = load_golden(case)
    o = make(g)
    assert abs(o.get_kcv(g["q"], g["sc_fphys"]) - float(g["kcv"])) <= 1e-11 * abs(float(g["kcv"]))
    q, p = g["q"].copy(), g["p"].copy()
    c = o.get_conserved(q, p, 0.123)
    assert abs(c - float(g["conserved"])) <= 1e-11 * abs(float(g["conserved"]))
    np.testing.assert_allclose(q, g["conserved_q"], rtol=0, atol=1e-12 * np.abs(q).max())


@pytest.mark.parametrize("case", PIMD)
@pytest.mark.parametrize("tag", ["nve", "nvt"])
def test_ring_polymer_steps(case, tag):
    g = load_golden(case)
    o = make(g)
    q, p = g["q"].copy(), g["p"].copy()
    f, fp = g["sc_f"].copy(), g["sc_fphys"].copy()
    point, lst, disp = g["point"].copy(), g["list"].copy(), np.zeros(o.P * 3 * o.N)
    heat = 0.0
    es = []
    nsteps = len(g[f"{tag}_energy"])
    for k in range(nsteps):
        noise = g["nvt_noise"][k] if tag == "nvt" else None
        e, heat, scp = o.update_pimd(q, p, f, fp, point, lst, disp, is_nvt=(tag == "nvt"), noise=noise,
                                     heat=heat)
        es.append(e)
    np.testing.assert_allclose(es, g[f"{tag}_energy"], rtol=1e-10)
    assert rel_rms(q, g[f"{tag}_q"]) < 1e-13
    assert rel_rms(p, g[f"{tag}_p"]) < 1e-9
    assert rel_rms(fp, g[f"{tag}_fphys"]) < 1e-10
    assert rel_rms(f, g[f"{tag}_f"]) < 1e-7
    assert abs(heat - float(g[f"{tag}_heat"])) <= 1e-8 * (abs(float(g[f"{tag}_heat"])) + 1e-6)
    assert abs(scp - float(g[f"{tag}_sc_pot"])) <= 1e-10 * abs(float(g[f"{tag}_sc_pot"]))
