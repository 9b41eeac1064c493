"""Generate the golden fixtures of the spline ("fast-CMD") path from the
reference's own sources.

Runs get_forces_wspline, force_eval_sc_wspline, update_trajectory_class_wspline
and update_sc_wspline (forces.cpp:634-691, :791-882; update.cpp:16-75,
:139-269), compiled unmodified into oracle/_ref/libqtipref.so by
`make -C oracle ref`, on seeded starts with synthetic pair tables, and stores
inputs and outputs as tests/golden/spline/<case>.npz.

The reference reads its tables from oo/oh/hh_spline.txt, which it does not
ship. The tables here are smooth synthetic pair corrections on the reference's
grid (knots 0, 0.01, ... bohr, simulation.cpp:38-39, :66-67, :93-94):
    y(r) = A exp(-r / lam) (1 - (r / r_end)^2)^2,  r in [0, r_end],
with (A [Hartree], lam [bohr], r_end [bohr]) = (5e-3, 1.2, 7.0) O-O,
(-3e-3, 1.0, 5.5) O-H and (2e-3, 0.8, 4.5) H-H. The Boost spline type the
reference evaluates them with is the oracle's stand-in (oracle/shim), so these
fixtures pin the pair loop, cutoffs, force assembly and propagation of the
spline path; the spline interpolant itself is the oracle's restatement.

Usage:  python tests/golden/make_spline_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from qtip4pf_water_gb300.start import seeded_start  # noqa: E402

REF_SO = os.path.join(ROOT, "oracle", "_ref", "libqtipref.so")
D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)
TABLES = {"oo": (5e-3, 1.2, 7.0), "oh": (-3e-3, 1.0, 5.5), "hh": (2e-3, 0.8, 4.5)}
# name: (n_mols, n_beads, temp_K, dt_fs, seed)
CASES = {"spline_n64_p1": (64, 1, 298.0, 0.5, 21), "spline_n64_p4": (64, 4, 298.0, 0.25, 22)}


def table(A, lam, r_end, step=0.01):
    n = int(round(r_end / step)) + 1
    r = np.arange(n) * step
    return np.ascontiguousarray(A * np.exp(-r / lam) * (1.0 - (r / r_end) ** 2) ** 2)


def _p(a, t=D):
    return a.ctypes.data_as(t)


def run_case(name):
    N, P, T, dt_fs, seed = CASES[name]
    lib = C.CDLL(REF_SO)
    lib.ref_setup.argtypes = [C.c_int, C.c_int, D, C.c_double, C.c_double, C.c_double, C.c_double]
    lib.ref_list_size.restype = C.c_int
    lib.ref_neighbour_list.argtypes = [D, I, I, D, C.c_int]
    lib.ref_set_splines.argtypes = [D, C.c_int, D, C.c_int, D, C.c_int]
    lib.ref_get_forces.argtypes = [D, D, I, I, C.c_int]
    lib.ref_get_forces.restype = C.c_double
    lib.ref_get_forces_wspline.argtypes = [D, D, I, I, C.c_int]
    lib.ref_get_forces_wspline.restype = C.c_double
    lib.ref_force_eval_sc_wspline.argtypes = [D, D, I, I, D, D]
    lib.ref_force_eval_sc_wspline.restype = C.c_double
    lib.ref_update_class_wspline.argtypes = [D, D, D, I, I, D]
    lib.ref_update_class_wspline.restype = C.c_double
    lib.ref_update_sc_wspline.argtypes = [D, D, D, D, I, I, D, D]
    lib.ref_update_sc_wspline.restype = C.c_double
    st = seeded_start(N, P, T, seed)
    q, p = st.q.copy(), st.p.copy()
    box = np.ascontiguousarray(st.box_bohr, dtype=np.float64)
    lib.ref_setup(N, P, _p(box), T, dt_fs, 1e-6, 1e-5)
    ls = lib.ref_list_size()
    tabs = {k: table(*v) for k, v in TABLES.items()}
    lib.ref_set_splines(_p(tabs["oo"]), len(tabs["oo"]), _p(tabs["oh"]), len(tabs["oh"]), _p(tabs["hh"]),
                        len(tabs["hh"]))
    point = np.zeros(P * N, dtype=np.int32)
    lst = np.zeros(P * ls, dtype=np.int32)
    disp = np.zeros(P * 3 * N)
    for b in range(P):
        lib.ref_neighbour_list(_p(q), _p(point, I), _p(lst, I), _p(disp), b)
    out = dict(n_mols=N, n_beads=P, temp_K=T, dt_fs=dt_fs, seed=seed, box=box, eps_ewald=1e-6, eps_sc=1e-5,
               q=q, p=p, point=point.copy(), list=lst.copy(), list_size=ls, step=0.01,
               tab_oo=tabs["oo"], tab_oh=tabs["oh"], tab_hh=tabs["hh"])
    f0 = np.zeros(P * 9 * N)
    f = np.zeros(P * 9 * N)
    e0 = np.array([lib.ref_get_forces(_p(q), _p(f0), _p(point, I), _p(lst, I), b) for b in range(P)])
    e = np.array([lib.ref_get_forces_wspline(_p(q), _p(f), _p(point, I), _p(lst, I), b) for b in range(P)])
    out.update(forces_nospline=f0, energies_nospline=e0, forces=f.copy(), energies=e)
    if P == 1:
        q1, p1, f1 = q.copy(), p.copy(), f.copy()
        pt1, ls1, d1 = point.copy(), lst.copy(), np.zeros(3 * N)
        es = [lib.ref_update_class_wspline(_p(q1), _p(p1), _p(f1), _p(pt1, I), _p(ls1, I), _p(d1)) for _ in range(3)]
        out.update(vv_q=q1, vv_p=p1, vv_f=f1, vv_energy=np.array(es))
    else:
        fsc = np.zeros(P * 9 * N)
        fph = np.zeros(P * 9 * N)
        scp = C.c_double(0.0)
        esc = lib.ref_force_eval_sc_wspline(_p(q), _p(fsc), _p(point, I), _p(lst, I), C.byref(scp), _p(fph))
        out.update(sc_f=fsc.copy(), sc_fphys=fph.copy(), sc_energy=esc, sc_pot=scp.value)
        q2, p2, f2, fp2 = q.copy(), p.copy(), fsc.copy(), fph.copy()
        pt2, ls2, d2 = point.copy(), lst.copy(), np.zeros(P * 3 * N)
        es = []
        for _ in range(2):
            scp2 = C.c_double(0.0)
            es.append(lib.ref_update_sc_wspline(_p(q2), _p(p2), _p(f2), _p(fp2), _p(pt2, I), _p(ls2, I), _p(d2),
                                                C.byref(scp2)))
        out.update(nve_q=q2, nve_p=p2, nve_f=f2, nve_fphys=fp2, nve_energy=np.array(es))
    np.savez_compressed(os.path.join(HERE, "spline", f"{name}.npz"), **out)
    d = f - f0
    print(f"{name}: spline part of the forces: rms {np.sqrt(np.mean(d ** 2)):.3e} of {np.sqrt(np.mean(f ** 2)):.3e}; "
          f"energy {e[0] - e0[0]:.3e}")


def main():
    if len(sys.argv) > 2 and sys.argv[1] == "--case":
        run_case(sys.argv[2])
        return
    if not os.path.exists(REF_SO):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref"])
    for name in CASES:  # the reference keeps process globals: one process per case
        subprocess.check_call([sys.executable, __file__, "--case", name])


if __name__ == "__main__":
    main()
