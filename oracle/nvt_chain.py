"""Test infrastructure (the oracle, never the product): one NVT chain of the
oracle's restatement of the device stepper from a given state, returning its
run averages of the potential energy per bead and of the centroid-virial
kinetic energy (the estimators simulation.cpp:936-961 averages). Run in spawned
worker processes by the statistical comparison in
tests/test_gpu_oracle_stepper.py, one chain per replica."""
from __future__ import annotations

import numpy as np


def nvt_chain(args):
    """args: (n_mols, n_beads, box_bohr, q, p, temp_K, dt_fs, seed, steps, discard[, sys[, head]]).
    The noise is the device's for system index sys (default 0) of a context
    with that seed. Returns the two run averages and the per-step values of
    the first `head` steps (default none)."""
    n_mols, n_beads, box, q, p, temp, dt, seed, steps, discard = args[:10]
    sys = args[10] if len(args) > 10 else 0
    head = args[11] if len(args) > 11 else 0
    from oracle.binding import Oracle

    o = Oracle(n_mols, n_beads, np.asarray(box), temp, dt)
    qq = np.array(q, dtype=np.float64).reshape(-1)
    pp = np.array(p, dtype=np.float64).reshape(-1)
    point, lst, disp = o.build_lists(qq)
    f = np.zeros_like(qq)
    o.force_eval_trotter(qq, f, point, lst)
    fp = f.copy()
    stp = o.stepper(seed, sys=sys, thermostat=1, trotter=True)
    beta = 1.0 / (temp * o.constants()[2])
    nd = 9 * n_mols
    pots, kcvs, head_pot, head_kcv = [], [], [], []
    for k in range(steps):
        _, pot = o.stepper_step(stp, qq, pp, f, fp, point, lst, disp, is_nvt=True)
        x = qq.reshape(n_beads, nd)
        tq = -np.sum((x - x.mean(axis=0)) * fp.reshape(n_beads, nd))
        kcv = 0.5 * nd / beta + 0.5 * tq / n_beads
        if k < head:
            head_pot.append(pot)
            head_kcv.append(kcv)
        if k < discard:
            continue
        pots.append(pot)
        kcvs.append(kcv)
    return float(np.mean(pots)), float(np.mean(kcvs)), head_pot, head_kcv
