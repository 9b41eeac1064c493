"""The oracle's restatement of the spline ("fast-CMD") path, pinned to the
reference's own get_forces_wspline, force_eval_sc_wspline,
update_trajectory_class_wspline and update_sc_wspline (fixtures made by
tests/golden/make_spline_golden.py), and the spline interpolant's own
properties (it interpolates, reproduces cubics exactly, has the given end
slopes)."""
import glob
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle.binding import Oracle, spline_coefficients, spline_eval

CASES = sorted(os.path.splitext(os.path.basename(p))[0] for p in glob.glob(os.path.join(GOLDEN, "spline", "*.npz")))


def load(name):
    with np.load(os.path.join(GOLDEN, "spline", name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def rel_rms(a, b):
    a, b = np.asarray(a).reshape(-1), np.asarray(b).reshape(-1)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def test_interpolant_properties():
    h = 0.05
    x = np.arange(40) * h
    y = 0.3 * x ** 3 - x ** 2 + 0.5 * x - 2.0
    c = spline_coefficients(y, h, dl=0.5, dr=0.9 * x[-1] ** 2 - 2 * x[-1] + 0.5)
    for xi, yi in zip(x[:-1], y[:-1]):
        assert abs(spline_eval(c, len(y), 0.0, h, xi)[0] - yi) < 1e-12
    for xt in (0.013, 0.77, 1.234, 1.9):  # a cubic with its exact end slopes is reproduced
        v, d = spline_eval(c, len(y), 0.0, h, xt)
        assert abs(v - (0.3 * xt ** 3 - xt ** 2 + 0.5 * xt - 2.0)) < 1e-12
        assert abs(d - (0.9 * xt ** 2 - 2 * xt + 0.5)) < 1e-10
    # estimated end slopes (five-point differences) are exact for a cubic too
    c2 = spline_coefficients(y, h)
    assert np.abs(c2 - c).max() < 1e-11


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_the_reference_spline_path(case):
    g = load(case)
    N, P = int(g["n_mols"]), int(g["n_beads"])
    o = Oracle(N, P, g["box"], float(g["temp_K"]), float(g["dt_fs"]))
    o.set_splines({"oo": g["tab_oo"], "oh": g["tab_oh"], "hh": g["tab_hh"]})
    q = g["q"].reshape(-1).copy()
    f = np.zeros_like(q)
    e = np.array([o.get_forces(q, f, g["point"], g["list"], b) for b in range(P)])
    assert rel_rms(f, g["forces"]) < 1e-12
    # the spline part alone
    assert rel_rms(f - g["forces_nospline"], g["forces"] - g["forces_nospline"]) < 1e-10
    np.testing.assert_allclose(e, g["energies"], rtol=1e-12)
    if P == 1:
        qq, pp, ff = q.copy(), g["p"].reshape(-1).copy(), g["forces"].copy()
        pt, ls, dsp = g["point"].copy(), g["list"].copy(), np.zeros(3 * N)
        es = [o.update_class(qq, pp, ff, pt, ls, dsp) for _ in range(3)]
        np.testing.assert_allclose(es, g["vv_energy"], rtol=1e-12)
        assert rel_rms(qq, g["vv_q"]) < 1e-14 and rel_rms(pp, g["vv_p"]) < 1e-10
    else:
        fsc = np.zeros_like(q)
        fph = np.zeros_like(q)
        esc, scp = o.force_eval_sc(q, fsc, g["point"], g["list"], fph)
        assert abs(esc - float(g["sc_energy"])) < 1e-12 * abs(float(g["sc_energy"]))
        assert rel_rms(fph, g["sc_fphys"]) < 1e-12 and rel_rms(fsc, g["sc_f"]) < 1e-9
        qq, pp, ff, fp = q.copy(), g["p"].reshape(-1).copy(), g["sc_f"].copy(), g["sc_fphys"].copy()
        pt, ls, dsp = g["point"].copy(), g["list"].copy(), np.zeros(P * 3 * N)
        es = [o.update_pimd(qq, pp, ff, fp, pt, ls, dsp)[0] for _ in range(2)]
        np.testing.assert_allclose(es, g["nve_energy"], rtol=1e-11)
        assert rel_rms(qq, g["nve_q"]) < 1e-14 and rel_rms(fp, g["nve_fphys"]) < 1e-11
