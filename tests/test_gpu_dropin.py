"""The reference's function interface served by the GPU drop-in (libqtip_compat.so).

tests/compat/dropin_driver.cpp calls neighbour_list, force_eval_sc_nospline,
update_sc_nospline (NVT, seeded std::mt19937), get_kcv and get_conserved in
run_sc_nospline's order -- or, in its spline mode, force_eval_sc_wspline and
update_sc_wspline with boost::math::cubic_b_spline tables. tests/golden/
dropin_*.txt is its output when linked against the reference's own sources;
here it is linked against the drop-in and must reproduce that output: the shim
consumes the caller's mt19937 exactly as thermostat.cpp does, so even the
thermostatted trajectory agrees to round-off. Also run with the drop-in in
mixed precision (QTG_PRECISION=mixed), at the mixed-mode tolerance.
"""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

pytestmark = pytest.mark.gpu

CASES = ["dropin_n64_p4", "dropin_spline_n64_p4"]


def build_driver():
    from qtip4pf_water_gb300 import build

    build.build()
    exe = os.path.join(build.BUILD, "dropin_driver")
    src = os.path.join(ROOT, "tests", "compat", "dropin_driver.cpp")
    if not os.path.exists(exe) or os.path.getmtime(exe) < os.path.getmtime(src):
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-idirafter", build.COMPAT_INCLUDE, src, "-o", exe,
                               "-L", build.BUILD, "-lqtip_compat", "-lqtipgpu", f"-Wl,-rpath,{build.BUILD}"])
    return exe


def parse(text):
    rows = {}
    for line in text.splitlines():
        if not line or line.startswith("#"):
            continue
        parts = line.split()
        key = parts[0] if parts[0] != "step" else f"step{parts[1]}"
        vals = parts[1:] if parts[0] != "step" else parts[2:]
        rows[key] = np.array([float(v) for v in vals])
    return rows


def run(case, env=None):
    exe = build_driver()
    with open(os.path.join(GOLDEN, case + ".txt")) as f:
        text = f.read()
    args = text.splitlines()[0][1:].split()
    out = subprocess.check_output([exe, os.path.join(GOLDEN, case + ".bin")] + args, text=True, timeout=300,
                                  env=env)
    return parse(text), parse(out)


@pytest.mark.parametrize("case", CASES)
def test_dropin_reproduces_reference_run(case):
    want, got = run(case)
    assert set(want) == set(got)
    for k in want:
        # energies / heat / estimators to 1e-8 relative (Suzuki-Chin finite differences
        # amplify FP64 round-off); the position checksum to 1e-12
        tol = 1e-12 if k == "final" else 1e-8
        if k == "final":
            np.testing.assert_allclose(got[k][1], want[k][1], rtol=tol)
            np.testing.assert_allclose(got[k][[0, 2]], want[k][[0, 2]], rtol=1e-8)
        else:
            np.testing.assert_allclose(got[k], want[k], rtol=tol, atol=1e-12)


@pytest.mark.parametrize("case", CASES)
def test_dropin_mixed_precision(case):
    """The drop-in in mixed precision against the same reference output: energies
    within 1e-4 Hartree (the mixed-mode criterion, 1e-6 of the Ewald self-energy,
    is ~2e-5 Hartree a bead at 64 waters, and four beads enter the Suzuki-Chin
    sums), the thermostatted steps close (the same caller noise; position
    checksum to 1e-8 relative)."""
    env = dict(os.environ, QTG_PRECISION="mixed")
    want, got = run(case, env)
    np.testing.assert_allclose(got["init"], want["init"], rtol=0, atol=1e-4)
    np.testing.assert_allclose(got["final"][1], want["final"][1], rtol=1e-8)
    for k in want:
        if k.startswith("step"):
            np.testing.assert_allclose(got[k], want[k], rtol=1e-4, atol=1e-4)
