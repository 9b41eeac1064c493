"""The run driver qtg_water on the GPU: a classical and a Suzuki-Chin PIMD run
from config.txt, their output files in the reference's formats, and the NVE
sampling phase replayed by the oracle from the state the driver hands to it
(--dump-sampling-start): the final positions, the mean potential and kinetic
(classical) or Suzuki-Chin potential and centroid-virial kinetic energy (PIMD),
and the conserved-quantity lines of the sampling phase agree to the files'
six significant digits. FP64 runs, so the replay is exact to round-off."""
import os
import struct
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CONFIG = """n_beads {P}
T_K 298.0
epsilon_sc 0.00001
n_cell_x 2
n_cell_y 2
n_cell_z 2
rho_inp 0.997
dtfs {dt}
eps_ewald 0.000001
n_equil {ne}
n_samp {ns}
is_spline 0
cell_type fcc
from_file no
"""


def read_start(path):
    with open(path, "rb") as f:
        N, P = struct.unpack("<2i", f.read(8))
        par = struct.unpack("<7d", f.read(56))
        nt = P * 9 * N
        q = np.frombuffer(f.read(8 * nt), dtype="<f8").copy()
        p = np.frombuffer(f.read(8 * nt), dtype="<f8").copy()
    return N, P, np.array(par[:3]), par[3], par[4], q, p


def run_driver(tmp_path, P, dt, ne, ns):
    from qtip4pf_water_gb300 import build

    build.build()
    (tmp_path / "config.txt").write_text(CONFIG.format(P=P, dt=dt, ne=ne, ns=ns))
    r = subprocess.run([build.RUN_DRIVER, "--seed", "12", "--precision", "fp64", "--dump-sampling-start", "start.bin"],
                       cwd=tmp_path, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    return r


def floats(path):
    return np.array([float(x) for x in path.read_text().split()])


@pytest.mark.parametrize("P", [1, 4])
def test_run_driver_matches_the_oracle(tmp_path, P):
    from oracle.binding import Oracle

    dt = 0.5 if P == 1 else 0.25
    ne, ns = 150, 250
    run_driver(tmp_path, P, dt, ne, ns)
    names = ["output.txt", "initial_positions.txt", "cons.txt", "final_positions.txt"]
    names += ["pot.txt", "kin.txt"] if P == 1 else ["pot_sc.txt", "kcv.txt"]
    for n in names:
        assert (tmp_path / n).exists(), n
    out = (tmp_path / "output.txt").read_text().splitlines()
    assert out[0] == "rd output 12"
    assert out[1:11] == [f"Equilibration is {10 * k}% done " for k in range(10)]
    assert out[11:21] == [f"Sampling is {10 * k}% done " for k in range(10)]
    cons = floats(tmp_path / "cons.txt")
    assert len(cons) == 2 + 3  # every 100 steps of each phase
    N, P_, box, T, dtf, q, p = read_start(tmp_path / "start.bin")
    assert P_ == P and N == 32
    o = Oracle(N, P, box, T, dtf)
    point, lst, disp = o.build_lists(q)
    f = np.zeros_like(q)
    fp = np.zeros_like(q)
    pots, kins, cons_o = [], [], []
    m = np.tile(np.repeat([o.s.mo, o.s.mh, o.s.mh], 3), N)
    if P == 1:
        o.get_forces(q, f, point, lst, 0)
        for i in range(ns):
            e = o.update_class(q, p, f, point, lst, disp)
            ke = 0.5 * float(np.sum(p * p / m))
            pots.append(e)
            kins.append(ke)
            if i % 100 == 0:
                cons_o.append(e + ke)
        pot_file, kin_file = "pot.txt", "kin.txt"
    else:
        o.force_eval_sc(q, f, point, lst, fp)
        for i in range(ns):
            e, _, scp = o.update_pimd(q, p, f, fp, point, lst, disp)
            pots.append(scp)
            kins.append(o.get_kcv(q, fp))
            if i % 100 == 0:
                qq, pp = q.copy(), p.copy()
                cons_o.append(o.get_conserved(qq, pp, e))
        pot_file, kin_file = "pot_sc.txt", "kcv.txt"
    np.testing.assert_allclose(floats(tmp_path / pot_file), np.mean(pots), rtol=1e-5)
    np.testing.assert_allclose(floats(tmp_path / kin_file), np.mean(kins), rtol=1e-5)
    # the sampling phase is NVE: the heat term is the same constant for every line
    d = cons[2:] - np.array(cons_o)
    assert np.abs(d - d[0]).max() < 1e-5 * np.abs(cons).max()
    fin = floats(tmp_path / "final_positions.txt")
    np.testing.assert_allclose(fin, q, rtol=1e-5, atol=1e-5)
