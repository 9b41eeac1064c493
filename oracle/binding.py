"""ctypes binding of the C oracle (oracle/qtip_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by __graft_entry__.smoke() as
the checker, and by bench.py for its CPU-baseline leg. The product package
never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_build", "liboracle.so")

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)


class QoSys(C.Structure):
    _fields_ = [
        ("n_mols", C.c_int), ("n_atoms", C.c_int), ("n_dof", C.c_int), ("n_beads", C.c_int),
        ("list_size", C.c_int), ("k_max", C.c_int),
        ("box", C.c_double * 3), ("vol", C.c_double), ("min_box", C.c_double), ("max_box", C.c_double),
        ("temp_K", C.c_double), ("beta", C.c_double), ("beta_n", C.c_double), ("omega_psq", C.c_double),
        ("pi_over_p", C.c_double),
        ("dt", C.c_double), ("halfdt", C.c_double), ("eps_sc", C.c_double),
        ("acc", C.c_double), ("kappa", C.c_double), ("rc_sq", C.c_double), ("kc_sq", C.c_double),
        ("k_pref", C.c_double), ("ewald_pref", C.c_double),
        ("r_cut", C.c_double), ("r_cut_sq", C.c_double), ("r_skin", C.c_double), ("r_skin_sq", C.c_double),
        ("mo", C.c_double), ("mh", C.c_double), ("qo", C.c_double), ("qh", C.c_double),
        ("gamma_m", C.c_double),
        ("spl", C.c_void_p),
    ]


class QoSpline(C.Structure):
    _fields_ = [("n", C.c_int), ("start", C.c_double), ("step", C.c_double), ("cut_sq", C.c_double),
                ("c", C.POINTER(C.c_double))]


class QoSplines(C.Structure):
    _fields_ = [("t", QoSpline * 3)]


class QoStepper(C.Structure):
    _fields_ = [("seed", C.c_ulonglong), ("sys", C.c_int), ("thermostat", C.c_int), ("trotter", C.c_int),
                ("centroid_fixed", C.c_int), ("tau0_fs", C.c_double), ("step", C.c_ulonglong),
                ("cf_samples", C.c_double)]


def build(force: bool = False) -> str:
    src = os.path.join(HERE, "qtip_oracle.c")
    if force or not os.path.exists(SO) or os.path.getmtime(SO) < os.path.getmtime(src):
        subprocess.check_call(["make", "-s", "-C", HERE], stdout=subprocess.DEVNULL)
    return SO


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(SO)
        S = C.POINTER(QoSys)
        L.qo_init.argtypes = [S, C.c_int, C.c_int, D, C.c_double, C.c_double, C.c_double, C.c_double]
        L.qo_constants.argtypes = [D]
        L.qo_neighbour_list.argtypes = [S, D, I, I, D, C.c_int]
        L.qo_neighbour_list.restype = C.c_int
        L.qo_get_forces.argtypes = [S, D, D, D, I, I, C.c_int]
        L.qo_get_forces.restype = C.c_double
        L.qo_kwald.argtypes = [S, D, D, D, C.c_int]
        L.qo_kwald.restype = C.c_double
        L.qo_force_eval_sc.argtypes = [S, D, D, D, D, I, I, D, D]
        L.qo_force_eval_sc.restype = C.c_double
        L.qo_force_eval_trotter.argtypes = [S, D, D, D, I, I, D]
        L.qo_force_eval_trotter.restype = C.c_double
        L.qo_ftransform.argtypes = [S, D, C.c_int, C.c_int]
        L.qo_pile_g.argtypes = [S, D, D, D]
        L.qo_pile_g.restype = C.c_double
        L.qo_bussi.argtypes = [S, D, D, D]
        L.qo_bussi.restype = C.c_double
        L.qo_get_kcv.argtypes = [S, D, D]
        L.qo_get_kcv.restype = C.c_double
        L.qo_get_conserved.argtypes = [S, D, D, D, C.c_double]
        L.qo_get_conserved.restype = C.c_double
        L.qo_update_class.argtypes = [S, D, D, D, D, D, I, I, D]
        L.qo_update_class.restype = C.c_double
        L.qo_update_pimd.argtypes = [S, D, D, D, D, D, D, I, I, D, C.c_int, D, D, D, C.c_int]
        L.qo_update_pimd.restype = C.c_double
        U = C.POINTER(C.c_uint)
        L.qo_philox4x32_10.argtypes = [U, C.c_uint, C.c_uint, U]
        L.qo_stepper_normal_f32.argtypes = [C.c_uint, C.c_uint]
        L.qo_stepper_normal_f32.restype = C.c_double
        L.qo_stepper_centroid_draw.argtypes = [C.c_ulonglong, C.c_int, C.c_int, C.c_ulonglong, D, D]
        L.qo_stepper_centroid_draw.restype = C.c_int
        L.qo_stepper_step.argtypes = [S, C.POINTER(QoStepper), D, D, D, D, D, D, I, I, D, C.c_int, D, D]
        L.qo_stepper_step.restype = C.c_double
        L.qo_spline_build.argtypes = [D, C.c_int, C.c_double, C.c_double, C.c_double, D]
        L.qo_spline_build.restype = C.c_int
        L.qo_spline_eval.argtypes = [D, C.c_int, C.c_double, C.c_double, C.c_double, D]
        L.qo_spline_eval.restype = C.c_double
        L.qo_set_splines.argtypes = [S, C.POINTER(QoSplines)]
        L.qo_count_kvectors.argtypes = [S]
        L.qo_count_kvectors.restype = C.c_int
        _lib = L
    return _lib


def philox4x32_10(ctr, key):
    """Philox4x32-10 block of the oracle (four 32-bit words)."""
    L = lib()
    c = (C.c_uint * 4)(*[int(x) & 0xFFFFFFFF for x in ctr])
    o = (C.c_uint * 4)()
    L.qo_philox4x32_10(c, int(key[0]) & 0xFFFFFFFF, int(key[1]) & 0xFFFFFFFF, o)
    return [int(x) for x in o]


def spline_eval(c, n, start, step, x):
    """Value and derivative of the oracle's spline with coefficients c at x."""
    L = lib()
    d = C.c_double(0.0)
    c = np.ascontiguousarray(c, dtype=np.float64)
    v = L.qo_spline_eval(_d(c), int(n), float(start), float(step), float(x), C.byref(d))
    return v, d.value


def spline_coefficients(y, step, dl=float("nan"), dr=float("nan")):
    L = lib()
    y = np.ascontiguousarray(y, dtype=np.float64)
    c = np.zeros(len(y) + 2)
    assert L.qo_spline_build(_d(y), len(y), float(step), float(dl), float(dr), _d(c)) == 1
    return c


def _d(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(D)


def _i(a):
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(I)


class Oracle:
    """One system (n_mols waters, n_beads beads) with the reference's derived parameters."""

    def __init__(self, n_mols, n_beads, box_bohr, temp_K=298.0, dt_fs=0.25, eps_ewald=1e-6,
                 eps_sc=1e-5):
        self.L = lib()
        self.s = QoSys()
        box = np.ascontiguousarray(np.asarray(box_bohr, dtype=np.float64).reshape(3))
        self.L.qo_init(C.byref(self.s), int(n_mols), int(n_beads), _d(box), float(temp_K), float(dt_fs),
                       float(eps_ewald), float(eps_sc))
        N = n_mols
        self.N, self.P = N, n_beads
        self.charge = np.tile(np.array([self.s.qo, self.s.qh, self.s.qh]), N)
        self.mass = np.tile(np.repeat(np.array([self.s.mo, self.s.mh, self.s.mh]), 3), N)

    @property
    def list_size(self):
        return self.s.list_size

    def new_lists(self):
        return (np.zeros(self.P * self.N, np.int32), np.zeros(self.P * self.s.list_size, np.int32),
                np.zeros(self.P * 3 * self.N))

    def neighbour_list(self, q, point, lst, disp, bead=0):
        return self.L.qo_neighbour_list(C.byref(self.s), _d(q), _i(point), _i(lst), _d(disp), bead)

    def build_lists(self, q):
        point, lst, disp = self.new_lists()
        for b in range(self.P):
            n = self.neighbour_list(q, point, lst, disp, b)
            if n < 0:
                raise RuntimeError("neighbour list overflow")
        return point, lst, disp

    def get_forces(self, q, f, point, lst, bead=0):
        return self.L.qo_get_forces(C.byref(self.s), _d(q), _d(f), _d(self.charge), _i(point), _i(lst), bead)

    def kwald(self, sites, f, bead=0):
        return self.L.qo_kwald(C.byref(self.s), _d(sites), _d(f), _d(self.charge), bead)

    def force_eval_sc(self, q, f, point, lst, fphys):
        scp = C.c_double(0.0)
        e = self.L.qo_force_eval_sc(C.byref(self.s), _d(q), _d(f), _d(self.charge), _d(self.mass),
                                    _i(point), _i(lst), C.byref(scp), _d(fphys))
        return e, scp.value

    def force_eval_trotter(self, q, f, point, lst):
        pot = C.c_double(0.0)
        e = self.L.qo_force_eval_trotter(C.byref(self.s), _d(q), _d(f), _d(self.charge), _i(point),
                                         _i(lst), C.byref(pot))
        return e, pot.value

    def ftransform(self, a, length, forwards):
        self.L.qo_ftransform(C.byref(self.s), _d(a), int(length), 1 if forwards else 0)

    def pile_g(self, p, noise):
        return self.L.qo_pile_g(C.byref(self.s), _d(p), _d(self.mass), _d(noise))

    def bussi(self, p, noise):
        return self.L.qo_bussi(C.byref(self.s), _d(p), _d(self.mass), _d(noise))

    def get_kcv(self, q, f):
        return self.L.qo_get_kcv(C.byref(self.s), _d(q), _d(f))

    def get_conserved(self, q, p, energy):
        return self.L.qo_get_conserved(C.byref(self.s), _d(q), _d(p), _d(self.mass), float(energy))

    def update_class(self, q, p, f, point, lst, disp):
        return self.L.qo_update_class(C.byref(self.s), _d(q), _d(p), _d(self.mass), _d(f), _d(self.charge),
                                      _i(point), _i(lst), _d(disp))

    def update_pimd(self, q, p, f, fphys, point, lst, disp, is_nvt=False, noise=None, heat=0.0,
                    trotter=False):
        h = C.c_double(heat)
        pot = C.c_double(0.0)
        nz = noise if noise is not None else np.zeros(2)
        e = self.L.qo_update_pimd(C.byref(self.s), _d(q), _d(p), _d(self.mass), _d(f), _d(fphys),
                                  _d(self.charge), _i(point), _i(lst), _d(disp), 1 if is_nvt else 0,
                                  _d(nz), C.byref(h), C.byref(pot), 1 if trotter else 0)
        return e, h.value, pot.value

    def stepper(self, seed, sys=0, thermostat=1, trotter=True, centroid_fixed=False, tau0_fs=100.0):
        """State of the device stepper's propagation for this system (counter at 1,
        as the device's stands after its first force evaluation)."""
        return QoStepper(seed=int(seed), sys=int(sys), thermostat=int(thermostat), trotter=1 if trotter else 0,
                         centroid_fixed=1 if centroid_fixed else 0, tau0_fs=float(tau0_fs), step=1, cf_samples=0.0)

    def stepper_step(self, st, q, p, f, fphys, point, lst, disp, is_nvt=True, cf_acc=None):
        pot = C.c_double(0.0)
        e = self.L.qo_stepper_step(C.byref(self.s), C.byref(st), _d(q), _d(p), _d(self.mass), _d(f), _d(fphys),
                                   _d(self.charge), _i(point), _i(lst), _d(disp), 1 if is_nvt else 0,
                                   None if cf_acc is None else _d(cf_acc), C.byref(pot))
        return e, pot.value

    def set_splines(self, tables, start=0.0, step=0.01):
        """Attach pair tables {"oo"|"oh"|"hh": values on start + i step}, cutoff at the
        last knot (simulation.cpp:59-60), end slopes estimated; None removes them."""
        if tables is None:
            self.L.qo_set_splines(C.byref(self.s), None)
            self._spl = None
            return
        spl = QoSplines()
        keep = []
        for t, key in enumerate(("oo", "oh", "hh")):
            y = tables.get(key)
            if y is None:
                continue
            y = np.ascontiguousarray(y, dtype=np.float64)
            c = np.zeros(len(y) + 2)
            assert self.L.qo_spline_build(_d(y), len(y), step, float("nan"), float("nan"), _d(c)) == 1
            end = start + step * (len(y) - 1)
            spl.t[t] = QoSpline(len(y), start, step, end * end, _d(c))
            keep.append(c)
        self._spl = (spl, keep)
        self.L.qo_set_splines(C.byref(self.s), C.byref(spl))

    def count_kvectors(self):
        return self.L.qo_count_kvectors(C.byref(self.s))

    def constants(self):
        out = np.zeros(19)
        self.L.qo_constants(_d(out))
        return out
