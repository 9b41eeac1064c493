"""Record the expected output of tests/compat/dropin_driver.cpp linked against the
reference's own sources (forces.cpp, neighbour.cpp, fourier.cpp, update.cpp,
thermostat.cpp, path_integrals.cpp, compiled in place with the oracle's FFTW /
Boost shims). Writes tests/golden/dropin_<case>.bin (the start) and .txt (the
driver's output). Needs the reference checkout (REF_DIR, default
/root/reference); run it in the development container.
"""
import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from qtip4pf_water_gb300.start import seeded_start  # noqa: E402

REF_DIR = os.environ.get("REF_DIR", "/root/reference")
REF_SRCS = ["forces.cpp", "neighbour.cpp", "fourier.cpp", "update.cpp", "thermostat.cpp", "path_integrals.cpp"]
CASES = {"dropin_n64_p4": (64, 4, 298.0, 0.25, 31, 6, 77)}


def write_start(path, st, dt_fs, eps_ewald=1e-6, eps_sc=1e-5):
    with open(path, "wb") as f:
        f.write(struct.pack("<2i", st.n_mols, st.n_beads))
        f.write(struct.pack("<7d", *st.box_bohr, st.temp_K, dt_fs, eps_ewald, eps_sc))
        f.write(np.ascontiguousarray(st.q, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(st.p, dtype="<f8").tobytes())


def main():
    drv = os.path.join(ROOT, "tests", "compat", "dropin_driver.cpp")
    with tempfile.TemporaryDirectory() as tmp:
        exe = os.path.join(tmp, "dropin_ref")
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-w", "-fopenmp", "-I", os.path.join(ROOT, "oracle", "shim"),
                               "-I", REF_DIR, drv] + [os.path.join(REF_DIR, s) for s in REF_SRCS] + ["-o", exe])
        for name, (N, P, T, dt, seed, steps, rng) in CASES.items():
            st = seeded_start(N, P, T, seed=seed)
            binp = os.path.join(HERE, name + ".bin")
            write_start(binp, st, dt)
            out = subprocess.check_output([exe, binp, str(steps), str(rng)], text=True)
            with open(os.path.join(HERE, name + ".txt"), "w") as f:
                f.write(f"# {steps} {rng}\n" + out)
            print(name, out.splitlines()[-1])


if __name__ == "__main__":
    main()
