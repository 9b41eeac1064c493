"""qtip4pf_water_gb300 -- GB300 (sm_103a) force and ring-polymer propagation for
flexible qTIP4P/F water, a drop-in for the hot path of rayseashyn/qtip4pf_water.

The compute lives in libqtipgpu.so (CUDA, include/qtip4pf_gb300.h). This module
is its Python binding, mirroring the reference's function interface
(forces.h, neighbour.h, fourier.h, update.h, thermostat.h, path_integrals.h):
the same names, the same array layouts and argument meaning, on numpy arrays.
Where the reference prints a warning and continues (e.g. Verlet-list
overflow, neighbour.cpp:56-58) this binding raises QtgError.

There is no CPU fallback: importing works anywhere, but creating a System
requires the library and an sm_103 GPU and raises otherwise.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from .start import WaterStart, default_charges, default_masses, seeded_start  # noqa: F401

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libqtipgpu.so")

FP64, MIXED = 0, 1
SUZUKI_CHIN, TROTTER = 0, 1
THERMO_NONE, PILE_G, PILE_L = 0, 1, 2
EST_FIELDS = ("pot", "kcv", "conserved", "heat", "kin", "vtot", "rebuilds", "step")

_STATUS = {0: "ok", 1: "invalid argument", 2: "CUDA error", 3: "Verlet list overflow",
           4: "non-finite value", 5: "invalid state", 6: "no sm_103 device"}


class QtgError(RuntimeError):
    def __init__(self, status, msg=""):
        self.status = status
        super().__init__(f"{_STATUS.get(status, status)}: {msg}")


class SystemDesc(C.Structure):
    _fields_ = [("n_mols", C.c_int), ("n_beads", C.c_int), ("box_bohr", C.c_double * 3),
                ("temp_K", C.c_double), ("dt_fs", C.c_double), ("eps_ewald", C.c_double),
                ("eps_sc", C.c_double), ("propagator", C.c_int), ("thermostat", C.c_int),
                ("tau0_fs", C.c_double), ("seed", C.c_uint64)]


class SystemInfo(C.Structure):
    _fields_ = [("n_mols", C.c_int), ("n_beads", C.c_int), ("n_dof", C.c_int), ("list_size", C.c_int),
                ("k_max", C.c_int), ("n_kvectors", C.c_int), ("kappa", C.c_double), ("rc", C.c_double),
                ("kc", C.c_double), ("dt", C.c_double), ("beta_n", C.c_double), ("omega_psq", C.c_double)]


D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)
V = C.c_void_p


class PairSpline(C.Structure):
    """qtg_pair_spline: one pair type's table (values on start + i step)."""
    _fields_ = [("values", D), ("n", C.c_int), ("start", C.c_double), ("step", C.c_double),
                ("left_deriv", C.c_double), ("right_deriv", C.c_double), ("cut_sq", C.c_double)]


class MlpWeights(C.Structure):
    """qtg_mlp_weights: device pointers of the BF16 weights and FP32 biases."""
    _fields_ = [("w1", V), ("w2", V), ("w3", V), ("b1", V), ("b2", V), ("b3", V)]

_lib = None


def load(build_if_missing: bool = True):
    """Load libqtipgpu.so (building it with nvcc if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH) and build_if_missing:
        from . import build as _b
        _b.build()
    if not os.path.exists(LIB_PATH):
        raise QtgError(6, f"{LIB_PATH} is missing; run python -m qtip4pf_water_gb300.build")
    L = C.CDLL(LIB_PATH)
    sig = {
        "qtg_create": ([C.POINTER(SystemDesc), C.c_int, C.c_int, C.POINTER(V)], C.c_int),
        "qtg_destroy": ([V], None),
        "qtg_last_error": ([V], C.c_char_p),
        "qtg_status_string": ([C.c_int], C.c_char_p),
        "qtg_set_stream": ([V, V], C.c_int),
        "qtg_system_info_get": ([V, C.c_int, C.POINTER(SystemInfo)], C.c_int),
        "qtg_kernel_launches": ([V, C.POINTER(C.c_uint64)], C.c_int),
        "qtg_set_charges": ([V, C.c_int, D], C.c_int),
        "qtg_set_masses": ([V, C.c_int, D], C.c_int),
        "qtg_neighbour_list": ([V, C.c_int, D, I, I, D, C.c_int], C.c_int),
        "qtg_get_forces": ([V, C.c_int, D, D, D, I, I, C.c_int, D], C.c_int),
        "qtg_kwald": ([V, C.c_int, D, D, D, C.c_int, D], C.c_int),
        "qtg_force_eval_sc": ([V, C.c_int, D, D, D, D, I, I, D, D, D], C.c_int),
        "qtg_force_eval_trotter": ([V, C.c_int, D, D, D, I, I, D, D], C.c_int),
        "qtg_ftransform": ([V, C.c_int, D, C.c_int, C.c_int], C.c_int),
        "qtg_pile_g": ([V, C.c_int, D, D, D, D], C.c_int),
        "qtg_bussi": ([V, C.c_int, D, D, D, D], C.c_int),
        "qtg_get_kcv": ([V, C.c_int, D, D, D], C.c_int),
        "qtg_get_conserved": ([V, C.c_int, D, D, D, C.c_double, D], C.c_int),
        "qtg_update_class": ([V, C.c_int, V, V, V, V, V, V, V, V, D], C.c_int),
        "qtg_update_pimd": ([V, C.c_int, V, V, V, V, V, V, V, V, V, C.c_int, V, D, D, D], C.c_int),
        "qtg_set_state": ([V, C.c_int, D, D], C.c_int),
        "qtg_get_state": ([V, C.c_int, D, D, D, D, D], C.c_int),
        "qtg_init_forces": ([V], C.c_int),
        "qtg_run_steps": ([V, C.c_int, C.c_int], C.c_int),
        "qtg_sync": ([V], C.c_int),
        "qtg_get_estimators": ([V, C.c_int, D, C.c_int, I], C.c_int),
        "qtg_reset_estimators": ([V], C.c_int),
        "qtg_time_kernel": ([V, C.c_char_p, C.c_int, D], C.c_int),
        "qtg_fp32_peak": ([D], C.c_int),
        "qtg_fp64_peak": ([D], C.c_int),
        "qtg_autotune": ([V, C.c_int, D, D], C.c_int),
        "qtg_transfer_bytes": ([V, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)], C.c_int),
        "qtg_sym_descriptors": ([V, C.c_int, C.c_int, D, V, V], C.c_int),
        "qtg_mlp_forward": ([C.POINTER(MlpWeights), V, C.c_int, V, V], C.c_int),
        "qtg_surrogate_status": ([C.POINTER(C.c_uint), C.c_int], C.c_int),
        "qtg_mlp_train_batch": ([C.POINTER(MlpWeights), V, V, C.c_int, C.c_float, V, C.c_int, V, V], C.c_int),
        "qtg_attach_surrogate": ([V, C.c_int, C.POINTER(MlpWeights), C.POINTER(C.c_float), C.c_float], C.c_int),
        "qtg_detach_surrogate": ([V, C.c_int], C.c_int),
        "qtg_adam_step": ([V, V, V, V, C.c_int, C.c_int, C.c_float, C.c_float, C.c_float, C.c_float, V, C.c_int, V],
                          C.c_int),
        "qtg_set_centroid_fixed": ([V, C.c_int, C.c_int], C.c_int),
        "qtg_set_pair_splines": ([V, C.c_int, C.POINTER(PairSpline), C.POINTER(PairSpline),
                                  C.POINTER(PairSpline)], C.c_int),
        "qtg_reset_centroid_force": ([V, C.c_int], C.c_int),
        "qtg_get_centroid_force": ([V, C.c_int, D, D], C.c_int),
        "qtg_set_tuning": ([V, C.c_int, C.c_int, C.c_int], C.c_int),
        "qtg_get_tuning": ([V, I, I, I], C.c_int),
        "qtg_set_real_space": ([V, C.c_int], C.c_int),
        "qtg_get_real_space": ([V, I, I], C.c_int),
        "qtg_kwald_noalloc": ([V, V, C.c_int, D, C.c_double, V, V, V], C.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def _d(a):
    if a is None:
        return None
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("arrays must be C-contiguous float64")
    return a.ctypes.data_as(D)


def _i(a):
    if a.dtype != np.int32 or not a.flags.c_contiguous:
        raise TypeError("index arrays must be C-contiguous int32")
    return a.ctypes.data_as(I)


_F64, _I32 = np.dtype(np.float64), np.dtype(np.int32)


def _vd(a):
    """Address of a C-contiguous float64 array as a plain integer (the per-step
    entries take void pointers: cheaper to pass than typed ctypes pointers)."""
    if a is None:
        return None
    if a.dtype != _F64 or not a.flags.c_contiguous:
        raise TypeError("arrays must be C-contiguous float64")
    return a.ctypes.data


def _vi(a):
    if a.dtype != _I32 or not a.flags.c_contiguous:
        raise TypeError("index arrays must be C-contiguous int32")
    return a.ctypes.data


class Context:
    """Device context holding one or more independent systems (replicas)."""

    def __init__(self, descs, precision=FP64):
        self.L = load()
        arr = (SystemDesc * len(descs))(*descs)
        h = V()
        st = self.L.qtg_create(arr, len(descs), int(precision), C.byref(h))
        if st != 0:
            raise QtgError(st, "qtg_create failed")
        self.h = h
        self.precision = precision
        self.descs = list(descs)
        self.systems = [System(self, k) for k in range(len(descs))]

    def check(self, st):
        if st != 0:
            raise QtgError(st, self.L.qtg_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            self.L.qtg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_ptr):
        self.check(self.L.qtg_set_stream(self.h, V(stream_ptr)))

    def kernel_launches(self):
        n = C.c_uint64(0)
        self.check(self.L.qtg_kernel_launches(self.h, C.byref(n)))
        return int(n.value)

    def init_forces(self):
        self.check(self.L.qtg_init_forces(self.h))

    def transfer_bytes(self):
        """(host -> device, device -> host) bytes moved by this context so far."""
        a, b = C.c_uint64(0), C.c_uint64(0)
        self.check(self.L.qtg_transfer_bytes(self.h, C.byref(a), C.byref(b)))
        return int(a.value), int(b.value)

    def autotune(self, iters=10):
        """Pick the chunk counts of k_real / k_ksk / k_kforce for this batch
        (qtg_autotune); returns (heuristic ms, tuned ms) of one force evaluation.
        Call after set_state and before init_forces."""
        t0, t1 = C.c_double(0.0), C.c_double(0.0)
        self.check(self.L.qtg_autotune(self.h, int(iters), C.byref(t0), C.byref(t1)))
        return t0.value, t1.value

    def set_tuning(self, n_rj=0, n_sc=0, n_kc=0):
        self.check(self.L.qtg_set_tuning(self.h, int(n_rj), int(n_sc), int(n_kc)))

    def tuning(self):
        a, b, c = C.c_int(0), C.c_int(0), C.c_int(0)
        self.check(self.L.qtg_get_tuning(self.h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    def set_real_space(self, form):
        """Mixed real space of large beads: 0 over the pair list (where eligible), 1 over all pairs."""
        self.check(self.L.qtg_set_real_space(self.h, int(form)))

    def real_space(self):
        """(form, list_eligible) of the context's mixed real space."""
        a, b = C.c_int(0), C.c_int(0)
        self.check(self.L.qtg_get_real_space(self.h, C.byref(a), C.byref(b)))
        return a.value, bool(b.value)

    def run_steps(self, n_steps, is_nvt=True):
        self.check(self.L.qtg_run_steps(self.h, int(n_steps), 1 if is_nvt else 0))

    def sync(self):
        self.check(self.L.qtg_sync(self.h))

    def reset_estimators(self):
        self.check(self.L.qtg_reset_estimators(self.h))

    def time_kernel(self, name, iters=20):
        """Average duration (ms) of one pipeline kernel over all systems (destroys the state)."""
        ms = C.c_double(0.0)
        self.check(self.L.qtg_time_kernel(self.h, name.encode(), int(iters), C.byref(ms)))
        return ms.value


def fp32_peak_tflops():
    """Measured FP32 FMA throughput of the current device (TFLOP/s)."""
    t = C.c_double(0.0)
    st = load().qtg_fp32_peak(C.byref(t))
    if st != 0:
        raise QtgError(st, "fp32 probe failed")
    return t.value


def fp64_peak_tflops():
    """Measured FP64 FMA throughput of the current device (TFLOP/s)."""
    t = C.c_double(0.0)
    st = load().qtg_fp64_peak(C.byref(t))
    if st != 0:
        raise QtgError(st, "fp64 probe failed")
    return t.value


def _check(st, what):
    if st != 0:
        raise QtgError(st, what + " failed")


def sym_descriptors(pos_ptr, n_conf, n_mols, box_bohr, desc_ptr, stream=0):
    """qtg_sym_descriptors on device buffers (pos double[n_conf][9N] -> desc float[n_conf][3N][32])."""
    box = np.ascontiguousarray(np.broadcast_to(np.asarray(box_bohr, dtype=np.float64), (3,)))
    _check(load().qtg_sym_descriptors(V(pos_ptr), int(n_conf), int(n_mols), _d(box), V(desc_ptr), V(stream)),
           "qtg_sym_descriptors")


def mlp_forward(weights: MlpWeights, x_ptr, m, y_ptr, stream=0):
    """qtg_mlp_forward on device buffers (x BF16 [m][96] -> y float[m][16])."""
    _check(load().qtg_mlp_forward(C.byref(weights), V(x_ptr), int(m), V(y_ptr), V(stream)), "qtg_mlp_forward")


def mlp_train_batch(weights: MlpWeights, x_ptr, t_ptr, m, grad_scale, partial_ptr, max_ctas, grad_ptr, stream=0):
    """qtg_mlp_train_batch: summed gradients and squared error of m rows into grad (float[NPARAMS + 1])."""
    _check(load().qtg_mlp_train_batch(C.byref(weights), V(x_ptr), V(t_ptr), int(m), float(grad_scale), V(partial_ptr),
                                      int(max_ctas), V(grad_ptr), V(stream)), "qtg_mlp_train_batch")


def adam_step(params_ptr, m1_ptr, m2_ptr, grad_ptr, n, step, lr, w_bf16_ptr, n_bf16, beta1=0.9, beta2=0.999,
              eps=1e-8, stream=0):
    _check(load().qtg_adam_step(V(params_ptr), V(m1_ptr), V(m2_ptr), V(grad_ptr), int(n), int(step), float(lr),
                                float(beta1), float(beta2), float(eps), V(w_bf16_ptr), int(n_bf16), V(stream)),
           "qtg_adam_step")


MLP_NPARAMS = 11408
MLP_NW = 64 * 96 + 64 * 64 + 16 * 64  # weights, stored first in the parameter vector


def surrogate_status(clear=True):
    """Error bits of the surrogate kernels (synchronises the device)."""
    b = C.c_uint(0)
    _check(load().qtg_surrogate_status(C.byref(b), 1 if clear else 0), "qtg_surrogate_status")
    return int(b.value)


def system_desc(n_mols, n_beads, box_bohr, temp_K=298.0, dt_fs=0.25, eps_ewald=1e-6, eps_sc=1e-5,
                propagator=SUZUKI_CHIN, thermostat=PILE_G, tau0_fs=100.0, seed=1):
    d = SystemDesc()
    d.n_mols = int(n_mols)
    d.n_beads = int(n_beads)
    b = np.broadcast_to(np.asarray(box_bohr, dtype=np.float64), (3,))
    for k in range(3):
        d.box_bohr[k] = float(b[k])
    d.temp_K, d.dt_fs, d.eps_ewald, d.eps_sc = float(temp_K), float(dt_fs), float(eps_ewald), float(eps_sc)
    d.propagator, d.thermostat, d.tau0_fs, d.seed = int(propagator), int(thermostat), float(tau0_fs), int(seed)
    return d


@dataclass
class Info:
    n_mols: int
    n_beads: int
    n_dof: int
    list_size: int
    k_max: int
    n_kvectors: int
    kappa: float
    rc: float
    kc: float
    dt: float
    beta_n: float
    omega_psq: float


class System:
    """One system of a Context, with the reference's per-system operations."""

    def __init__(self, ctx: Context, idx: int):
        self.ctx, self.idx = ctx, idx
        inf = SystemInfo()
        ctx.check(ctx.L.qtg_system_info_get(ctx.h, idx, C.byref(inf)))
        self.info = Info(*[getattr(inf, f[0]) for f in SystemInfo._fields_])
        self.N, self.P = inf.n_mols, inf.n_beads

    @classmethod
    def create(cls, n_mols, n_beads, box_bohr, precision=FP64, **kw):
        return Context([system_desc(n_mols, n_beads, box_bohr, **kw)], precision).systems[0]

    # ---- array helpers (the reference's layouts, indexing.h:6-24)
    def new_lists(self):
        return (np.zeros(self.P * self.N, np.int32), np.zeros(self.P * self.info.list_size, np.int32),
                np.zeros(self.P * 3 * self.N))

    def charges(self):
        return default_charges(self.N)

    def masses(self):
        return default_masses(self.N)

    def _c(self, st):
        self.ctx.check(st)

    # ---- tier 1: the reference's functions -------------------------------------------
    def neighbour_list(self, pos, point, lst, disp, bead=0):
        self._c(self.ctx.L.qtg_neighbour_list(self.ctx.h, self.idx, _d(pos), _i(point), _i(lst), _d(disp), bead))

    def build_lists(self, pos):
        point, lst, disp = self.new_lists()
        for b in range(self.P):
            self.neighbour_list(pos, point, lst, disp, b)
        return point, lst, disp

    def get_forces_nospline(self, pos, f, charge, point, lst, bead=0):
        e = C.c_double(0.0)
        self._c(self.ctx.L.qtg_get_forces(self.ctx.h, self.idx, _d(pos), _d(f), _d(charge), _i(point), _i(lst),
                                          bead, C.byref(e)))
        return e.value

    def kwald(self, sites, f_sites, charge, bead=0):
        e = C.c_double(0.0)
        self._c(self.ctx.L.qtg_kwald(self.ctx.h, self.idx, _d(sites), _d(f_sites), _d(charge), bead, C.byref(e)))
        return e.value

    def force_eval_sc_nospline(self, pos, f, charge, mass, point, lst, fphys):
        e, scp = C.c_double(0.0), C.c_double(0.0)
        self._c(self.ctx.L.qtg_force_eval_sc(self.ctx.h, self.idx, _d(pos), _d(f), _d(charge), _d(mass), _i(point),
                                             _i(lst), C.byref(scp), _d(fphys), C.byref(e)))
        return e.value, scp.value

    def force_eval_trotter(self, pos, f, charge, point, lst):
        e, pot = C.c_double(0.0), C.c_double(0.0)
        self._c(self.ctx.L.qtg_force_eval_trotter(self.ctx.h, self.idx, _d(pos), _d(f), _d(charge), _i(point),
                                                  _i(lst), C.byref(pot), C.byref(e)))
        return e.value, pot.value

    def ftransform(self, a, length, is_forwards):
        self._c(self.ctx.L.qtg_ftransform(self.ctx.h, self.idx, _d(a), int(length), 1 if is_forwards else 0))

    def pile_g(self, p, mass, noise=None):
        h = C.c_double(0.0)
        self._c(self.ctx.L.qtg_pile_g(self.ctx.h, self.idx, _d(p), _d(mass), _d(noise), C.byref(h)))
        return h.value

    def bussi(self, p, mass, noise=None):
        """thermostat.cpp:12-60 on the first n_dof momenta; returns the heat."""
        h = C.c_double(0.0)
        self._c(self.ctx.L.qtg_bussi(self.ctx.h, self.idx, _d(p), _d(mass), _d(noise), C.byref(h)))
        return h.value

    def get_kcv(self, q, f):
        o = C.c_double(0.0)
        self._c(self.ctx.L.qtg_get_kcv(self.ctx.h, self.idx, _d(q), _d(f), C.byref(o)))
        return o.value

    def get_conserved(self, q, p, mass, energy):
        o = C.c_double(0.0)
        self._c(self.ctx.L.qtg_get_conserved(self.ctx.h, self.idx, _d(q), _d(p), _d(mass), float(energy),
                                             C.byref(o)))
        return o.value

    def update_trajectory_class_nospline(self, q, p, mass, f, charge, point, lst, disp):
        e = C.c_double(0.0)
        self._c(self.ctx.L.qtg_update_class(self.ctx.h, self.idx, _vd(q), _vd(p), _vd(mass), _vd(f), _vd(charge),
                                            _vi(point), _vi(lst), _vd(disp), C.byref(e)))
        return e.value

    def update_sc_nospline(self, q, p, mass, f, fphys, charge, point, lst, disp, is_nvt, heat, noise=None):
        """One ring-polymer step (update.cpp:271-401). Returns (energy, heat, potential estimator)."""
        h, pot, e = C.c_double(heat), C.c_double(0.0), C.c_double(0.0)
        self._c(self.ctx.L.qtg_update_pimd(self.ctx.h, self.idx, _vd(q), _vd(p), _vd(mass), _vd(f), _vd(fphys),
                                           _vd(charge), _vi(point), _vi(lst), _vd(disp), 1 if is_nvt else 0,
                                           _vd(noise), C.byref(h), C.byref(pot), C.byref(e)))
        return e.value, h.value, pot.value

    # ---- tier 2: device-resident state -------------------------------------------------
    def set_state(self, q, p=None):
        self._c(self.ctx.L.qtg_set_state(self.ctx.h, self.idx, _d(np.ascontiguousarray(q, dtype=np.float64)),
                                         _d(None if p is None else np.ascontiguousarray(p, dtype=np.float64))))

    def get_state(self):
        n = self.P * 9 * self.N
        q, p, f, fp = (np.zeros(n) for _ in range(4))
        disp = np.zeros(self.P * 3 * self.N)
        self._c(self.ctx.L.qtg_get_state(self.ctx.h, self.idx, _d(q), _d(p), _d(f), _d(fp), _d(disp)))
        return dict(q=q, p=p, f=f, fphys=fp, disp=disp)

    def set_pair_splines(self, oo=None, oh=None, hh=None, start=0.0, step=0.01):
        """Attach tabulated pair corrections (the reference's *_wspline force path):
        values on the knots start + i step (bohr, Hartree), cutoff at the last knot
        (simulation.cpp:59-60), end slopes estimated. All None removes them."""
        keep, args = [], []
        for y in (oo, oh, hh):
            if y is None:
                args.append(None)
                continue
            y = np.ascontiguousarray(y, dtype=np.float64)
            keep.append(y)
            end = start + step * (len(y) - 1)
            args.append(C.byref(PairSpline(_d(y), len(y), start, step, float("nan"), float("nan"), end * end)))
        self._c(self.ctx.L.qtg_set_pair_splines(self.ctx.h, self.idx, *args))

    def set_centroid_fixed(self, fixed=True):
        """Centroid-constrained PIMD: hold the bead centroid fixed (Trotter systems)."""
        self._c(self.ctx.L.qtg_set_centroid_fixed(self.ctx.h, self.idx, 1 if fixed else 0))

    def reset_centroid_force(self):
        self._c(self.ctx.L.qtg_reset_centroid_force(self.ctx.h, self.idx))

    def centroid_force(self):
        """Mean over the steps so far of (1/P) sum_b F_b, double[9N], and the step count."""
        out = np.zeros(9 * self.N)
        n = C.c_double(0.0)
        self._c(self.ctx.L.qtg_get_centroid_force(self.ctx.h, self.idx, _d(out), C.byref(n)))
        return out, int(n.value)

    def attach_surrogate(self, weights, norm, out_scale):
        """Attach a trained centroid correction (qtg_attach_surrogate; P = 1 systems)."""
        nm = np.ascontiguousarray(norm, dtype=np.float32)
        self._c(self.ctx.L.qtg_attach_surrogate(self.ctx.h, self.idx, C.byref(weights),
                                                nm.ctypes.data_as(C.POINTER(C.c_float)), float(out_scale)))

    def detach_surrogate(self):
        self._c(self.ctx.L.qtg_detach_surrogate(self.ctx.h, self.idx))

    def estimators(self, max_records=1 << 20):
        n = C.c_int(0)
        cap = min(max_records, 4096)
        out = np.zeros(cap * 8)
        self._c(self.ctx.L.qtg_get_estimators(self.ctx.h, self.idx, _d(out), cap, C.byref(n)))
        rec = out[: n.value * 8].reshape(n.value, 8)
        return {k: rec[:, i].copy() for i, k in enumerate(EST_FIELDS)}
