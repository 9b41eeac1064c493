"""The drop-in (libqtip_compat.so) as the reference's own run driver sees it,
without a GPU:

* water.cpp, simulation.cpp and initialise.cpp -- the caller side, unmodified --
  compile and link against the drop-in alone (every function they call,
  nospline and spline paths, is defined);
* the per-pair helpers of forces.h it exports (lj_oxygen, intra_morse_bond,
  intra_harm_angle, rwald) and get_q_centroid return what the reference's own
  compiled functions return, bit for bit, and write the same forces.

Both need the reference's sources (the checkout recorded by `make -C oracle
ref` in oracle/_ref/ref_dir.txt); they are skipped where it is absent.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT

REF_TXT = os.path.join(ROOT, "oracle", "_ref", "ref_dir.txt")
REF_SO = os.path.join(ROOT, "oracle", "_ref", "libqtipref.so")


def ref_dir():
    d = os.environ.get("REF_DIR")
    if not d and os.path.exists(REF_TXT):
        d = open(REF_TXT).read().strip()
    if not d or not os.path.isdir(d) or not os.path.exists(os.path.join(d, "simulation.cpp")):
        pytest.skip("the reference's sources are not available here")
    return d


def test_reference_driver_links_against_the_dropin(tmp_path):
    from qtip4pf_water_gb300 import build

    src = ref_dir()
    build.build()
    exe = tmp_path / "water_gb300"
    # the Boost spline type from the drop-in's stand-in header (the same definition
    # the drop-in was compiled with); water.cpp also includes fftw3.h, which the
    # drop-in does not use: the oracle's shim supplies the declarations
    cmd = ["g++", "-O1", "-std=c++17", "-fopenmp", "-w", "-I", build.COMPAT_INCLUDE, "-idirafter",
           os.path.join(ROOT, "oracle", "shim"), "-I", src] + \
          [os.path.join(src, f) for f in ("water.cpp", "simulation.cpp", "initialise.cpp")] + \
          ["-L", build.BUILD, "-lqtip_compat", "-lqtipgpu", f"-Wl,-rpath,{build.BUILD}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    und = subprocess.run(["nm", "-uC", str(exe)], capture_output=True, text=True).stdout
    for name in ("get_forces_wspline", "update_sc_wspline", "update_trajectory_class_wspline",
                 "force_eval_sc_wspline", "update_sc_nospline", "neighbour_list"):
        assert name in und  # the driver calls it, and the drop-in resolved it (the link succeeded)


class Arr3(C.Structure):
    _fields_ = [("v", C.c_double * 3)]


def _libs():
    ref_dir()
    if not os.path.exists(REF_SO):
        pytest.skip("oracle/_ref is not built")
    from qtip4pf_water_gb300 import build

    build.build()
    # the reference build defines the configuration globals the drop-in reads
    ref = C.CDLL(REF_SO, mode=C.RTLD_GLOBAL)
    compat = C.CDLL(build.COMPAT)
    return ref, compat


def test_pair_helpers_match_the_reference():
    ref, compat = _libs()
    D = C.POINTER(C.c_double)
    ref.ref_setup.argtypes = [C.c_int, C.c_int, D, C.c_double, C.c_double, C.c_double, C.c_double]
    box = np.array([23.5, 23.5, 23.5])
    ref.ref_setup(8, 2, box.ctypes.data_as(D), 298.0, 0.25, 1e-6, 1e-5)
    rng = np.random.default_rng(4)
    A = C.POINTER(Arr3)
    sigs = {
        "_Z9lj_oxygenRKSt5arrayIdLm3EEdPdiii": [A, C.c_double, D, C.c_int, C.c_int, C.c_int],
        "_Z16intra_morse_bondRKSt5arrayIdLm3EEdPdiii": [A, C.c_double, D, C.c_int, C.c_int, C.c_int],
        "_Z16intra_harm_angleRKSt5arrayIdLm3EES2_ddPdii": [A, A, C.c_double, C.c_double, D, C.c_int, C.c_int],
        "_Z5rwaldRKSt5arrayIdLm3EEdPdPKdiidi": [A, C.c_double, D, D, C.c_int, C.c_int, C.c_double, C.c_int],
    }
    fns = {}
    for name, args in sigs.items():
        for lib in (ref, compat):
            fn = getattr(lib, name)
            fn.argtypes = args
            fn.restype = C.c_double
        fns[name] = (getattr(ref, name), getattr(compat, name))
    charge = np.tile([-1.1128, 0.5564, 0.5564], 8)
    for trial in range(20):
        r1 = Arr3((C.c_double * 3)(*rng.normal(size=3) * 3.0))
        r2 = Arr3((C.c_double * 3)(*(rng.normal(size=3) * 0.3 + 1.8)))
        d1 = float(np.sqrt(sum(x * x for x in r1.v)))
        d2 = float(np.sqrt(sum(x * x for x in r2.v)))
        i, j, bead = int(rng.integers(0, 4)), int(rng.integers(4, 8)), int(rng.integers(0, 2))
        calls = {
            "_Z9lj_oxygenRKSt5arrayIdLm3EEdPdiii": lambda f, fa: f(C.byref(r1), d1 * d1, fa, i, j, bead),
            "_Z16intra_morse_bondRKSt5arrayIdLm3EEdPdiii": lambda f, fa: f(C.byref(r2), d2, fa, i, 1 + trial % 2, bead),
            "_Z16intra_harm_angleRKSt5arrayIdLm3EES2_ddPdii":
                lambda f, fa: f(C.byref(r2), C.byref(Arr3((C.c_double * 3)(r2.v[1], -r2.v[0], r2.v[2]))), d2,
                                d2, fa, i, bead),
            "_Z5rwaldRKSt5arrayIdLm3EEdPdPKdiidi":
                lambda f, fa: f(C.byref(r1), d1 * d1, fa, charge.ctypes.data_as(D), 3 * i + trial % 3,
                                3 * (i if trial % 2 else j) + 1, 0.19, bead),
        }
        for name, call in calls.items():
            fr, fc = np.zeros(2 * 72), np.zeros(2 * 72)
            er = call(fns[name][0], fr.ctypes.data_as(D))
            ec = call(fns[name][1], fc.ctypes.data_as(D))
            assert er == ec, name
            assert np.array_equal(fr, fc), name


def test_q_centroid_matches_the_reference():
    ref, compat = _libs()
    D = C.POINTER(C.c_double)
    ref.ref_setup.argtypes = [C.c_int, C.c_int, D, C.c_double, C.c_double, C.c_double, C.c_double]
    box = np.array([23.5, 23.5, 23.5])
    ref.ref_setup(8, 6, box.ctypes.data_as(D), 298.0, 0.25, 1e-6, 1e-5)
    x = np.random.default_rng(1).normal(size=6 * 72)
    out = []
    for lib in (ref, compat):
        fn = lib._Z14get_q_centroidPKdi
        fn.argtypes = [D, C.c_int]
        fn.restype = D
        p = fn(x.ctypes.data_as(D), 72)
        out.append(np.array(p[:72]))
    assert np.array_equal(out[0], out[1])
