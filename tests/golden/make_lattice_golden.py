"""Golden starting configurations from the reference's own initialise.cpp
(initialise_fcc, initialise_orth), compiled into oracle/_ref/libqtipref.so by
`make -C oracle ref`. Writes tests/golden/lattice.npz: for each case the box,
positions (bead 0) and, for ice Ih, the seed and the lines initialise_orth
wrote to its log.

Usage:  python tests/golden/make_lattice_golden.py
"""
import ctypes as C
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libqtipref.so")
D = C.POINTER(C.c_double)
# name: (nx, ny, nz, rho, orth, seed)
CASES = {"fcc_3x3x3": (3, 3, 3, 0.997, 0, 0), "fcc_2x3x4": (2, 3, 4, 0.92, 0, 0),
         "ice_1x1x1": (1, 1, 1, 0.92, 1, 5), "ice_2x1x1": (2, 1, 1, 0.92, 1, 11), "ice_2x2x1": (2, 2, 1, 0.92, 1, 17),
         "ice_2x2x2": (2, 2, 2, 0.92, 1, 23)}


def run(name):
    nx, ny, nz, rho, orth, seed = CASES[name]
    lib = C.CDLL(REF_SO)
    lib.ref_setup_cells.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int]
    lib.ref_n_mols.restype = C.c_int
    lib.ref_box.argtypes = [D]
    lib.ref_initialise_fcc.argtypes = [D]
    lib.ref_initialise_orth.argtypes = [C.c_uint, C.c_char_p, D]
    lib.ref_setup_cells(nx, ny, nz, rho, orth, 1)
    n = lib.ref_n_mols()
    box = np.zeros(3)
    lib.ref_box(box.ctypes.data_as(D))
    pos = np.zeros(9 * n)
    log = ""
    if orth:
        with tempfile.TemporaryDirectory() as tmp:
            lp = os.path.join(tmp, "log.txt")
            lib.ref_initialise_orth(seed, lp.encode(), pos.ctypes.data_as(D))
            log = open(lp).read()
    else:
        lib.ref_initialise_fcc(pos.ctypes.data_as(D))
    out = os.path.join(HERE, "_lattice_" + name + ".npz")
    np.savez(out, box=box, pos=pos, log=np.array(log), spec=np.array([nx, ny, nz, orth, seed]), rho=rho)


def main():
    if len(sys.argv) > 2 and sys.argv[1] == "--case":
        run(sys.argv[2])
        return
    if not os.path.exists(REF_SO):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref"])
    allv = {}
    for name in CASES:  # the reference keeps process globals: one process per case
        subprocess.check_call([sys.executable, __file__, "--case", name], timeout=600)
        part = os.path.join(HERE, "_lattice_" + name + ".npz")
        with np.load(part) as z:
            for k in z.files:
                allv[f"{name}__{k}"] = z[k]
        os.remove(part)
        print(name, allv[f"{name}__pos"].size // 9, "molecules")
    np.savez_compressed(os.path.join(HERE, "lattice", "lattice.npz"), **allv)


if __name__ == "__main__":
    main()
