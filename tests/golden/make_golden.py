"""Generate the golden fixtures that pin the oracle to the reference.

Runs the reference's own force / neighbour / fourier / update / thermostat /
estimator sources, compiled unmodified into oracle/_ref/libqtipref.so by
`make -C oracle ref`, on seeded inputs from qtip4pf_water_gb300.start, and
stores inputs and outputs as tests/golden/<case>.npz.

The reference keeps its configuration in process globals and ftransform keeps
a function-static FFTW plan sized by the first n_beads it sees
(fourier.cpp:16-18), so every case runs in a fresh subprocess.

Usage:  python tests/golden/make_golden.py            # all cases
        python tests/golden/make_golden.py --case n64_p1
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from qtip4pf_water_gb300.start import ANGS2BOHR, seeded_start  # noqa: E402

REF_SO = os.path.join(ROOT, "oracle", "_ref", "libqtipref.so")

D = C.POINTER(C.c_double)
I = C.POINTER(C.c_int)

# name: (n_mols, n_beads, temp_K, dt_fs, seed, box_angstrom or None, unwrap)
CASES = {
    "n64_p1": (64, 1, 298.0, 0.5, 11, None, False),
    "n64_p1_unwrapped": (64, 1, 298.0, 0.5, 12, None, True),
    "n128_p1": (128, 1, 298.0, 0.5, 13, 15.66, False),
    "n216_p1": (216, 1, 298.0, 0.5, 14, None, False),
    "n512_p1": (512, 1, 298.0, 0.25, 15, None, False),
    "n64_p4": (64, 4, 298.0, 0.25, 16, None, False),
    "n64_p8": (64, 8, 250.0, 0.25, 17, None, False),
    "n8_p32": (8, 32, 298.0, 0.25, 18, None, False),
}
EPS_EWALD = 1e-6
EPS_SC = 1e-5


def _p(a, t=D):
    return a.ctypes.data_as(t)


def load_ref():
    lib = C.CDLL(REF_SO)
    lib.ref_setup.argtypes = [C.c_int, C.c_int, D, C.c_double, C.c_double, C.c_double, C.c_double]
    lib.ref_list_size.restype = C.c_int
    lib.ref_ewald_params.argtypes = [D]
    lib.ref_neighbour_list.argtypes = [D, I, I, D, C.c_int]
    lib.ref_get_forces.argtypes = [D, D, I, I, C.c_int]
    lib.ref_get_forces.restype = C.c_double
    lib.ref_kwald.argtypes = [D, D, C.c_int]
    lib.ref_kwald.restype = C.c_double
    lib.ref_force_eval_sc.argtypes = [D, D, I, I, D, D]
    lib.ref_force_eval_sc.restype = C.c_double
    lib.ref_ftransform.argtypes = [D, C.c_int, C.c_int]
    lib.ref_get_kcv.argtypes = [D, D]
    lib.ref_get_kcv.restype = C.c_double
    lib.ref_get_conserved.argtypes = [D, D, C.c_double]
    lib.ref_get_conserved.restype = C.c_double
    lib.ref_update_class.argtypes = [D, D, D, I, I, D]
    lib.ref_update_class.restype = C.c_double
    lib.ref_update_sc.argtypes = [D, D, D, D, I, I, D, C.c_uint, C.c_int, D, D]
    lib.ref_update_sc.restype = C.c_double
    lib.ref_pile_g.argtypes = [D, C.c_uint, D]
    lib.ref_pile_g.restype = C.c_double
    lib.ref_bussi.argtypes = [D, C.c_uint, D]
    lib.ref_bussi.restype = C.c_double
    return lib


def run_case(name: str) -> None:
    N, P, T, dt_fs, seed, box_ang, unwrap = CASES[name]
    st = seeded_start(N, P, T, seed, box_angstrom=box_ang)
    q = st.q.copy()
    if unwrap:
        # move whole molecules by random whole-box multiples: coordinates far
        # outside the primary box exercise the minimum-image arithmetic
        rs = np.random.default_rng(seed)
        shift = rs.integers(-3, 4, size=(N, 1, 3)) * st.box_bohr[None, None, :]
        q = (q.reshape(P, N, 3, 3) + shift[None]).reshape(P, 9 * N)
    p = st.p.copy()
    lib = load_ref()
    box = np.ascontiguousarray(st.box_bohr, dtype=np.float64)
    lib.ref_setup(N, P, _p(box), T, dt_fs, EPS_EWALD, EPS_SC)
    ls = lib.ref_list_size()
    par = np.zeros(8)
    lib.ref_ewald_params(_p(par))
    out = dict(n_mols=N, n_beads=P, temp_K=T, dt_fs=dt_fs, seed=seed, box=box, eps_ewald=EPS_EWALD,
               eps_sc=EPS_SC, q=q, p=p, list_size=ls, ewald_params=par)

    point = np.zeros(P * N, dtype=np.int32)
    lst = np.zeros(P * ls, dtype=np.int32)
    disp = np.zeros(P * 3 * N)
    for b in range(P):
        lib.ref_neighbour_list(_p(q), _p(point, I), _p(lst, I), _p(disp), b)
    out.update(point=point.copy(), list=lst.copy())

    # one configuration per bead
    f = np.zeros(P * 9 * N)
    e = np.array([lib.ref_get_forces(_p(q), _p(f), _p(point, I), _p(lst, I), b) for b in range(P)])
    out.update(forces=f.copy(), energies=e)

    # reciprocal space alone on the charge-site array of bead 0
    g = 0.73612
    qa = q[0].reshape(N, 3, 3)
    sites = qa.copy()
    sites[:, 0, :] = g * qa[:, 0, :] + 0.5 * (1.0 - g) * (qa[:, 1, :] + qa[:, 2, :])
    sites = np.ascontiguousarray(sites.reshape(-1))
    fk = np.zeros(9 * N)
    ek = lib.ref_kwald(_p(sites), _p(fk), 0)
    out.update(kw_sites=sites, kw_forces=fk, kw_energy=ek)
    # Bussi rescale (thermostat.cpp:12-60) of the first n_dof momenta with a recorded draw
    pb = p.copy()
    noise_b = np.zeros(2)
    heat_b = lib.ref_bussi(_p(pb), seed + 7, _p(noise_b))
    out.update(bussi_p_in=p.copy(), bussi_p_out=pb, bussi_noise=noise_b, bussi_heat=heat_b)

    if P == 1:
        q1, p1, f1 = q.copy(), p.copy(), f.copy()
        pt1, ls1, d1 = point.copy(), lst.copy(), np.zeros(3 * N)
        steps = []
        for _ in range(3):
            steps.append(lib.ref_update_class(_p(q1), _p(p1), _p(f1), _p(pt1, I), _p(ls1, I), _p(d1)))
        out.update(vv_q=q1, vv_p=p1, vv_f=f1, vv_energy=np.array(steps), vv_disp=d1)
    else:
        fsc = np.zeros(P * 9 * N)
        fph = np.zeros(P * 9 * N)
        scp = C.c_double(0.0)
        esc = lib.ref_force_eval_sc(_p(q), _p(fsc), _p(point, I), _p(lst, I), C.byref(scp), _p(fph))
        out.update(sc_f=fsc.copy(), sc_fphys=fph.copy(), sc_energy=esc, sc_pot=scp.value)
        out.update(kcv=lib.ref_get_kcv(_p(q), _p(fph)))
        qc, pc = q.copy(), p.copy()
        cons = lib.ref_get_conserved(_p(qc), _p(pc), 0.123)
        out.update(conserved=cons, conserved_q=qc, conserved_p=pc)
        # normal-mode transform of positions (length 9N) and of a 3N array
        a = q.copy()
        lib.ref_ftransform(_p(a), 9 * N, 1)
        out.update(nm_fwd=a.copy())
        lib.ref_ftransform(_p(a), 9 * N, 0)
        out.update(nm_roundtrip=a.copy())
        d3 = np.ascontiguousarray(np.random.default_rng(seed + 1).normal(size=P * 3 * N))
        d3f = d3.copy()
        lib.ref_ftransform(_p(d3f), 3 * N, 1)
        out.update(nm3_in=d3, nm3_fwd=d3f)
        # PILE-G on normal-mode momenta with a recorded noise stream
        pn = p.copy()
        lib.ref_ftransform(_p(pn), 9 * N, 1)
        noise = np.zeros(2 + (P - 1) * 9 * N)
        pin = pn.copy()
        heat = lib.ref_pile_g(_p(pn), seed, _p(noise))
        out.update(pile_p_in=pin, pile_p_out=pn, pile_noise=noise, pile_heat=heat)
        # two deterministic NVE steps and one NVT step (noise recorded)
        for tag, nvt in (("nve", 0), ("nvt", 1)):
            q2, p2, f2, fp2 = q.copy(), p.copy(), fsc.copy(), fph.copy()
            pt2, ls2, d2 = point.copy(), lst.copy(), np.zeros(P * 3 * N)
            heat = C.c_double(0.0)
            scp2 = C.c_double(0.0)
            nst = 2 if tag == "nve" else 1
            es = []
            noises = []
            for k in range(nst):
                if nvt:
                    # replay the stream the step's pile_g will consume
                    ptmp = np.zeros(P * 9 * N) + 1.0
                    nz = np.zeros(2 + (P - 1) * 9 * N)
                    lib.ref_pile_g(_p(ptmp), seed + 100 + k, _p(nz))
                    noises.append(nz)
                es.append(lib.ref_update_sc(_p(q2), _p(p2), _p(f2), _p(fp2), _p(pt2, I), _p(ls2, I),
                                            _p(d2), seed + 100 + k, nvt, C.byref(heat), C.byref(scp2)))
            out.update({f"{tag}_q": q2, f"{tag}_p": p2, f"{tag}_f": f2, f"{tag}_fphys": fp2,
                        f"{tag}_disp": d2, f"{tag}_energy": np.array(es), f"{tag}_heat": heat.value,
                        f"{tag}_sc_pot": scp2.value})
            if nvt:
                out.update(nvt_noise=np.stack(noises))
    np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **out)
    print(f"{name}: list_size={ls} pairs={point[-1] if P == 1 else 'per-bead'} "
          f"E0={e[0]:.10f} kmax={int(par[3])}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default=None)
    a = ap.parse_args()
    if a.case:
        run_case(a.case)
        return
    if not os.path.exists(REF_SO):
        subprocess.check_call(["make", "-C", os.path.join(ROOT, "oracle"), "ref"])
    for name in CASES:
        subprocess.check_call([sys.executable, os.path.abspath(__file__), "--case", name])


if __name__ == "__main__":
    main()
