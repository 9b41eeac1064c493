"""The tabulated pair corrections (the reference's spline / "fast-CMD" force
path) on the GPU against the reference's own get_forces_wspline,
force_eval_sc_wspline, update_trajectory_class_wspline and update_sc_wspline
(fixtures from tests/golden/make_spline_golden.py), and inside the device
stepper against the oracle.

Tolerances as the other parity tests: FP64 1e-9 relative RMS (Suzuki-Chin
forces 1e-8: the finite difference amplifies round-off by 1/eps_sc), mixed
1e-4; the spline part of the forces alone (wspline minus nospline) within 1e-9
(FP64) and 1e-4 (mixed) of its own size. Positions after the steps: FP64 to
round-off; mixed within 1e-7 relative RMS (forces within 1e-4 move a 0.25 fs
step's positions by at most ~1e-6 bohr).
"""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "spline", "*.npz")))


def load(name):
    with np.load(os.path.join(GOLDEN, "spline", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def rel_rms(a, b):
    a, b = np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def make(q, g, precision):
    P = int(g["n_beads"])
    s = q.System.create(int(g["n_mols"]), P, g["box"], precision=precision, temp_K=float(g["temp_K"]),
                        dt_fs=float(g["dt_fs"]), propagator=q.TROTTER if P == 1 else q.SUZUKI_CHIN,
                        thermostat=q.PILE_G, seed=int(g["seed"]))
    s.set_pair_splines(oo=g["tab_oo"], oh=g["tab_oh"], hh=g["tab_hh"], step=float(g["step"]))
    return s


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES)
def test_spline_forces_match_the_reference(gpu_lib, case, precision):
    q = gpu_lib
    g = load(case)
    tol = 1e-9 if precision == "fp64" else 1e-4
    s = make(q, g, q.FP64 if precision == "fp64" else q.MIXED)
    P = s.P
    x = g["q"].reshape(-1).copy()
    f = np.zeros(P * 9 * s.N)
    e = np.array([s.get_forces_nospline(x, f, s.charges(), g["point"], g["list"], b) for b in range(P)])
    assert rel_rms(f, g["forces"]) < tol
    assert rel_rms(f - g["forces_nospline"].reshape(-1), g["forces"] - g["forces_nospline"]) < tol
    # mixed: the energy criterion of the other parity tests, 1e-6 of the Ewald self-energy
    self_e = float(np.sum(s.info.kappa / np.sqrt(3.14159265359) * s.charges() ** 2))
    e_tol = 1e-9 * np.abs(g["energies"]).max() if precision == "fp64" else 1e-6 * self_e
    assert np.abs(e - g["energies"]).max() < e_tol
    # removing the tables restores the plain forces
    s.set_pair_splines()
    f0 = np.zeros_like(f)
    s.get_forces_nospline(x, f0, s.charges(), g["point"], g["list"], 0)
    nd = 9 * s.N
    assert rel_rms(f0[:nd], g["forces_nospline"].reshape(-1)[:nd]) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES)
def test_spline_steps_match_the_reference(gpu_lib, case, precision):
    q = gpu_lib
    g = load(case)
    s = make(q, g, q.FP64 if precision == "fp64" else q.MIXED)
    P, N = s.P, s.N
    tol = 1e-9 if precision == "fp64" else 1e-4
    x, p = g["q"].reshape(-1).copy(), g["p"].reshape(-1).copy()
    point, lst = g["point"].copy(), g["list"].copy()
    if P == 1:
        f = g["forces"].reshape(-1).copy()
        disp = np.zeros(3 * N)
        es = [s.update_trajectory_class_nospline(x, p, s.masses(), f, s.charges(), point, lst, disp)
              for _ in range(3)]
        np.testing.assert_allclose(es, g["vv_energy"], rtol=tol)
        assert rel_rms(x, g["vv_q"]) < (1e-14 if precision == "fp64" else 1e-8)
        assert rel_rms(f, g["vv_f"]) < tol
    else:
        fsc = np.zeros(P * 9 * N)
        fph = np.zeros(P * 9 * N)
        e, scp = s.force_eval_sc_nospline(x, fsc, s.charges(), s.masses(), point, lst, fph)
        assert rel_rms(fph, g["sc_fphys"]) < tol
        assert rel_rms(fsc, g["sc_f"]) < (1e-8 if precision == "fp64" else 1e-4)
        f, fp = g["sc_f"].reshape(-1).copy(), g["sc_fphys"].reshape(-1).copy()
        disp = np.zeros(P * 3 * N)
        es = []
        heat = 0.0
        for _ in range(2):
            e, heat, _ = s.update_sc_nospline(x, p, s.masses(), f, fp, s.charges(), point, lst, disp, False, heat)
            es.append(e)
        np.testing.assert_allclose(es, g["nve_energy"], rtol=1e-8 if precision == "fp64" else 1e-5)
        assert rel_rms(x, g["nve_q"]) < (1e-13 if precision == "fp64" else 1e-7)
        assert rel_rms(fp, g["nve_fphys"]) < tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_device_stepper_with_splines_follows_the_oracle(gpu_lib, precision):
    """Device-resident second-order PIMD (P = 4, PILE-G) with the tables attached,
    four NVT steps, against the oracle's restatement of the stepper."""
    from oracle.binding import Oracle

    q = gpu_lib
    g = load("spline_n64_p4")
    tabs = {"oo": g["tab_oo"], "oh": g["tab_oh"], "hh": g["tab_hh"]}
    st = q.seeded_start(64, 4, 298.0, seed=31)
    ctx = q.Context([q.system_desc(64, 4, st.box_bohr, dt_fs=0.25, propagator=q.TROTTER, thermostat=q.PILE_G,
                                   seed=31)], q.FP64 if precision == "fp64" else q.MIXED)
    s = ctx.systems[0]
    s.set_state(st.q, st.p)
    s.set_pair_splines(**tabs)
    ctx.init_forces()
    ctx.run_steps(4, is_nvt=True)
    ctx.sync()
    out = s.get_state()
    o = Oracle(64, 4, st.box_bohr, 298.0, 0.25)
    o.set_splines(tabs)
    qq, pp = st.q.reshape(-1).copy(), st.p.reshape(-1).copy()
    point, lst, disp = o.build_lists(qq)
    f = np.zeros_like(qq)
    o.force_eval_trotter(qq, f, point, lst)
    fp = f.copy()
    stp = o.stepper(31, thermostat=1, trotter=True)
    for _ in range(4):
        o.stepper_step(stp, qq, pp, f, fp, point, lst, disp, is_nvt=True)
    assert np.abs(out["q"] - qq).max() < 1e-7
    assert rel_rms(out["fphys"], fp) < (1e-6 if precision == "fp64" else 1e-4)
