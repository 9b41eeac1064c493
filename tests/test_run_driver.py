"""The run driver qtg_water (config.txt in, the reference's output files out)
up to the point where it needs a GPU: the config is read as water.cpp reads
it, the start is built as initialise.cpp builds it (ice Ih from the run's
seeded std::mt19937, with the reference's log lines in output.txt), and
initial_positions.txt is written in the reference's format (water.cpp:195-207,
default stream precision). Without a GPU it then stops at context creation,
with an error."""
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN

Z = np.load(os.path.join(GOLDEN, "lattice", "lattice.npz"))

CONFIG = """n_beads {P}
T_K 298.0
epsilon_sc 0.00001
n_cell_x {nx}
n_cell_y {ny}
n_cell_z {nz}
rho_inp {rho}
dtfs 0.25
eps_ewald 0.000001
n_equil 0
n_samp 0
is_spline 0
cell_type {cell}
from_file no
"""


def driver():
    from qtip4pf_water_gb300 import build

    build.build()
    return build.RUN_DRIVER


def fmt(x):
    return f"{x:g}"  # std::ostream's default: 6 significant digits, %g


@pytest.mark.parametrize("case", ["ice_1x1x1", "ice_2x1x1", "fcc_2x3x4"])
def test_driver_start_matches_the_reference(tmp_path, case):
    nx, ny, nz, orth, seed = (int(v) for v in Z[case + "__spec"])
    rho = float(Z[case + "__rho"])
    P = 2
    (tmp_path / "config.txt").write_text(CONFIG.format(P=P, nx=nx, ny=ny, nz=nz, rho=rho,
                                                       cell="orth" if orth else "fcc"))
    r = subprocess.run([driver(), "--seed", str(seed)], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    out = (tmp_path / "output.txt").read_text()
    assert out.splitlines()[0] == f"rd output {seed}"
    if orth:
        assert out.split("\n", 1)[1] == str(Z[case + "__log"])
    pos = Z[case + "__pos"].reshape(-1, 3)
    want = "".join(" ".join(fmt(v) for v in row) + "\n" for row in np.concatenate([pos] * P))
    assert (tmp_path / "initial_positions.txt").read_text() == want
    if r.returncode != 0:  # no GPU here: it stops at context creation
        assert "qtg_create" in r.stderr


def test_driver_rejects_odd_bead_counts(tmp_path):
    (tmp_path / "config.txt").write_text(CONFIG.format(P=3, nx=1, ny=1, nz=1, rho=0.92, cell="fcc"))
    r = subprocess.run([driver(), "--seed", "1"], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert r.returncode == 1 and "n_beads should be even" in r.stderr
