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
# name: (n_mols, n_beads, temp_K, dt_fs, start seed, steps, mt19937 seed[, "spline"])
CASES = {"dropin_n64_p4": (64, 4, 298.0, 0.25, 31, 6, 77),
         "dropin_spline_n64_p4": (64, 4, 298.0, 0.25, 32, 4, 78, "spline")}


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
        # the oracle's Boost stand-in evaluates splines with liboracle.so's restatement
        odir = os.path.join(ROOT, "oracle", "_build")
        subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-w", "-fopenmp", "-I", os.path.join(ROOT, "oracle", "shim"),
                               "-I", REF_DIR, drv] + [os.path.join(REF_DIR, s) for s in REF_SRCS] +
                              ["-L", odir, "-loracle", f"-Wl,-rpath,{odir}", "-o", exe])
        for name, spec in CASES.items():
            N, P, T, dt, seed, steps, rng = spec[:7]
            mode = list(spec[7:])
            st = seeded_start(N, P, T, seed=seed)
            binp = os.path.join(HERE, name + ".bin")
            write_start(binp, st, dt)
            out = subprocess.check_output([exe, binp, str(steps), str(rng)] + mode, text=True)
            with open(os.path.join(HERE, name + ".txt"), "w") as f:
                f.write(f"# {steps} {rng}{' ' + mode[0] if mode else ''}\n" + out)
            print(name, out.splitlines()[-1])


if __name__ == "__main__":
    main()
