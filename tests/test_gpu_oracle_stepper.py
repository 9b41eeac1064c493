"""The device-resident stepper against the oracle's restatement of it, step for
step with the same counter-based thermostat noise (the oracle recomputes the
Philox4x32-10 draws the device makes), and statistically over 2 ps chains
that part by chaos.

Paths covered (update.cpp:271-401 with the stepper's thermostats):
* PILE-G, second-order and Suzuki-Chin assembly;
* classical Langevin (P = 1, the centroid a Langevin mode with time constant tau0);
* centroid-constrained PIMD (centroid momentum held at zero, internal modes
  PILE-L) and its mean centroid force (1/P) sum_b F_b;
* the benchmark's own system: 512 waters, P = 32, mixed precision, second
  order, PILE-G, forked force evaluation with autotuned launch shapes.

Tolerances: positions within 1e-7 bohr after the steps, 3e-7 for the ten
0.5 fs classical steps (the device's single-precision Box-Muller differs from
the oracle's by an ulp or two, 1e-7 of a draw, and the mixed forces differ
from FP64 by ~1e-7 relative; a step moves an atom ~1e-2 bohr); forces within
the mixed-mode 1e-4 relative RMS, and 1e-6 in FP64 (forces at positions that
differ by those 1e-8 bohr; the FP64 forces of one configuration are pinned
at 1e-9 by the single-configuration tests); the mean centroid force within
1e-6 (FP64) or 1e-4 (mixed) relative RMS. Statistics: 32 oracle chains and
32 device chains from the same equilibrated states with the same noise
streams (the per-step estimator records while the trajectories stay
together, then the run averages), and 32 device chains with independent
noise streams: the run averages of the potential and the centroid-virial
kinetic energy within two standard errors of the two sides' means.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel_rms(a, b):
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def _device(q, st, precision, propagator, thermostat, seed, temp=298.0, dt=0.25, tau0=100.0, fixed=False,
            autotune=False):
    ctx = q.Context([q.system_desc(st.n_mols, st.n_beads, st.box_bohr, temp_K=temp, dt_fs=dt,
                                   propagator=propagator, thermostat=thermostat, tau0_fs=tau0, seed=seed)],
                    precision)
    s = ctx.systems[0]
    s.set_state(st.q, st.p)
    if fixed:
        s.set_centroid_fixed(True)
    if autotune:
        ctx.autotune(10)
    ctx.init_forces()
    return ctx, s


def _oracle(st, propagator_trotter, thermostat, seed, temp=298.0, dt=0.25, tau0=100.0, fixed=False):
    from oracle.binding import Oracle

    o = Oracle(st.n_mols, st.n_beads, st.box_bohr, temp, dt)
    qq, pp = st.q.copy().reshape(-1), st.p.copy().reshape(-1)
    point, lst, disp = o.build_lists(qq)
    f = np.zeros_like(qq)
    fp = np.zeros_like(qq)
    if propagator_trotter:
        o.force_eval_trotter(qq, f, point, lst)
        fp[:] = f
    else:
        o.force_eval_sc(qq, f, point, lst, fp)
    stp = o.stepper(seed, thermostat=thermostat, trotter=propagator_trotter, centroid_fixed=fixed, tau0_fs=tau0)
    return o, stp, [qq, pp, f, fp, point, lst, disp]


CASES = [
    # name, N, P, precision, propagator, thermostat, dt, steps, fixed
    ("pile_g_trotter_fp64", 64, 4, "fp64", "trotter", "pile_g", 0.25, 6, False),
    ("pile_g_trotter_mixed", 64, 4, "mixed", "trotter", "pile_g", 0.25, 6, False),
    ("pile_g_sc_fp64", 64, 4, "fp64", "sc", "pile_g", 0.25, 4, False),
    ("langevin_classical_fp64", 216, 1, "fp64", "trotter", "pile_l", 0.5, 10, False),
    ("langevin_classical_mixed", 216, 1, "mixed", "trotter", "pile_l", 0.5, 10, False),
    ("constrained_pile_l_fp64", 64, 8, "fp64", "trotter", "pile_l", 0.25, 6, True),
    ("constrained_pile_l_mixed", 64, 8, "mixed", "trotter", "pile_l", 0.25, 6, True),
]


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_thermostatted_steps_follow_the_oracle(gpu_lib, case):
    q = gpu_lib
    name, N, P, prec, prop, thermo, dt, nsteps, fixed = case
    seed = 1000 + N + P
    st = q.seeded_start(N, P, 298.0, seed=seed)
    precision = q.FP64 if prec == "fp64" else q.MIXED
    propagator = q.TROTTER if prop == "trotter" else q.SUZUKI_CHIN
    thermostat = q.PILE_G if thermo == "pile_g" else q.PILE_L
    ctx, s = _device(q, st, precision, propagator, thermostat, seed, dt=dt, fixed=fixed)
    if fixed:
        s.reset_centroid_force()
    ctx.run_steps(nsteps, is_nvt=True)
    ctx.sync()
    out = s.get_state()
    o, stp, (qq, pp, f, fp, point, lst, disp) = _oracle(st, prop == "trotter", 1 if thermo == "pile_g" else 2,
                                                       seed, dt=dt, fixed=fixed)
    cf = np.zeros(9 * N)
    for _ in range(nsteps):
        o.stepper_step(stp, qq, pp, f, fp, point, lst, disp, is_nvt=True, cf_acc=cf)
    assert stp.step == nsteps + 1
    dq = float(np.abs(out["q"] - qq).max())
    tol_q = 3e-7 if P == 1 else 1e-7
    assert dq < tol_q, f"{name}: positions differ by {dq:.2e} bohr after {nsteps} steps"
    assert rel_rms(out["p"], pp) < (1e-6 if prec == "fp64" else 1e-4), name
    tol_f = 1e-4 if prec == "mixed" else 1e-6
    assert rel_rms(out["fphys"], fp) < tol_f, name
    assert rel_rms(out["f"], f) < tol_f, name
    if fixed:
        g, n = s.centroid_force()
        assert n == nsteps and stp.cf_samples == nsteps
        assert rel_rms(g, cf / nsteps) < (1e-6 if prec == "fp64" else 1e-4), name
        c0 = st.q.reshape(P, -1).mean(axis=0)
        assert np.abs(out["q"].reshape(P, -1).mean(axis=0) - c0).max() < 1e-10


def test_nvt_after_nve_takes_a_current_centroid_factor(gpu_lib):
    """An NVT step after NVE steps rescales the centroid with its own step's
    draws and the current centroid kinetic energy (the oracle's rule), not a
    factor left from an earlier step."""
    q = gpu_lib
    st = q.seeded_start(64, 4, 298.0, seed=5)
    ctx, s = _device(q, st, q.FP64, q.TROTTER, q.PILE_G, 5)
    ctx.run_steps(3, is_nvt=False)
    ctx.run_steps(2, is_nvt=True)
    ctx.sync()
    out = s.get_state()
    o, stp, (qq, pp, f, fp, point, lst, disp) = _oracle(st, True, 1, 5)
    for k in range(5):
        o.stepper_step(stp, qq, pp, f, fp, point, lst, disp, is_nvt=k >= 3)
    assert np.abs(out["q"] - qq).max() < 1e-7
    assert rel_rms(out["p"], pp) < 1e-6


def test_headline_stepper_matches_the_oracle(gpu_lib):
    """The benchmark's system as the benchmark builds it: 512 waters, P = 32,
    mixed precision, second-order assembly, PILE-G, launch shapes autotuned,
    forked force evaluation. Forces of the start and three NVT steps against the
    oracle's FP64 restatement."""
    q = gpu_lib
    seed = 2024
    st = q.seeded_start(512, 32, 298.0, seed=seed)
    ctx, s = _device(q, st, q.MIXED, q.TROTTER, q.PILE_G, seed, autotune=True)
    f0 = s.get_state()["fphys"]
    o, stp, (qq, pp, f, fp, point, lst, disp) = _oracle(st, True, 1, seed)
    err0 = rel_rms(f0, fp)
    assert err0 < 1e-4, f"mixed forces of the start: {err0:.2e}"
    ctx.run_steps(3, is_nvt=True)
    ctx.sync()
    out = s.get_state()
    for _ in range(3):
        o.stepper_step(stp, qq, pp, f, fp, point, lst, disp, is_nvt=True)
    dq = float(np.abs(out["q"] - qq).max())
    assert dq < 1e-7, f"positions differ by {dq:.2e} bohr"
    assert rel_rms(out["fphys"], fp) < 1e-4
    assert rel_rms(out["p"], pp) < 1e-4


def test_nvt_averages_match_the_oracle_within_two_standard_errors(gpu_lib):
    """64 waters, P = 8, second order, PILE-G at 298 K, dt = 0.5 fs, 32 replica
    chains a side. 32 systems start from 32 seeded lattices and equilibrate
    20 ps on the device (one context). From each equilibrated state the device
    (a new context, mixed precision) and the oracle (spawned worker processes,
    FP64) each run a 2 ps chain with the same thermostat noise (seed and system
    index alike). The run averages are the potential energy per bead and the
    centroid-virial kinetic energy (the estimators simulation.cpp:936-961
    averages).

    * The two trajectories stay together for the first few hundred fs: over the
      first 100 steps the device's per-step estimator records equal the oracle's
      values (kinetic within 1e-6 relative; potential within 2e-5 relative, the
      FP32 Ewald energy sums of the mixed form).
    * They part by chaos within about 1 ps; the two sides' means of the chain
      averages agree within two standard errors, each side's the spread of its
      32 chain averages / sqrt(32), combined in quadrature (the chains of a pair
      share a start and a noise stream, so the difference's own spread is
      smaller and this bound conservative).
    * The same holds for 32 more device chains from the same states with
      independent noise streams (other seeds)."""
    import multiprocessing as mp
    import os

    from oracle.nvt_chain import nvt_chain

    q = gpu_lib
    N, P, T, dt = 64, 8, 298.0, 0.5
    n_chain, steps, head = 32, 4000, 100

    def desc(st, seed):
        return q.system_desc(N, P, st.box_bohr, temp_K=T, dt_fs=dt, propagator=q.TROTTER,
                             thermostat=q.PILE_G, tau0_fs=100.0, seed=seed)

    starts = [q.seeded_start(N, P, T, seed=9100 + i) for i in range(n_chain)]
    ctx = q.Context([desc(st, 9100 + i) for i, st in enumerate(starts)], q.MIXED)
    for s, st in zip(ctx.systems, starts):
        s.set_state(st.q, st.p)
    ctx.init_forces()
    ctx.run_steps(40000, is_nvt=True)
    ctx.sync()
    eq = [s.get_state() for s in ctx.systems]

    jobs = [(N, P, starts[i].box_bohr, e["q"], e["p"], T, dt, 9300 + i, steps, 0, i, head)
            for i, e in enumerate(eq)]
    pool = mp.get_context("spawn").Pool(max(1, min(n_chain, os.cpu_count() or 1)))
    orc_async = pool.map_async(nvt_chain, jobs)

    def device_chains(seed0):
        c = q.Context([desc(st, seed0 + i) for i, st in enumerate(starts)], q.MIXED)
        for s, e in zip(c.systems, eq):
            s.set_state(e["q"], e["p"])
        c.init_forces()
        c.reset_estimators()
        c.run_steps(steps, is_nvt=True)
        c.sync()
        out = [s.estimators() for s in c.systems]
        c.close()
        return out

    ests = device_chains(9300)  # the oracle's noise streams
    ests_ind = device_chains(9500)  # independent noise streams
    try:
        orc = orc_async.get()
    finally:
        pool.close()
        pool.join()

    for est, o in zip(ests, orc):
        assert len(est["pot"]) == steps
        dk = np.abs(est["kcv"][:head] - np.asarray(o[3])) / np.abs(np.asarray(o[3]))
        dp = np.abs(est["pot"][:head] - np.asarray(o[2])) / np.abs(np.asarray(o[2]))
        assert dk.max() < 1e-6, f"per-step kinetic estimator differs by {dk.max():.1e} relative"
        assert dp.max() < 2e-5, f"per-step potential differs by {dp.max():.1e} relative"

    report, ok = [], True
    for k, key, name in ((0, "pot", "potential"), (1, "kcv", "kinetic (centroid virial)")):
        c = np.array([r[k] for r in orc])
        for label, chains in (("same noise", ests), ("independent noise", ests_ind)):
            g = np.array([float(np.mean(e[key])) for e in chains])
            se = float(np.hypot(g.std(ddof=1), c.std(ddof=1)) / np.sqrt(n_chain))
            d = g - c
            ok = ok and abs(d.mean()) < 2.0 * se
            report.append(f"{name}, {label}: device {g.mean():.6f}, oracle {c.mean():.6f}, difference "
                          f"{d.mean():.2e} = {abs(d.mean()) / se:.2f} SE (SE {se:.1e}; paired "
                          f"{abs(d.mean()) / (d.std(ddof=1) / np.sqrt(n_chain)):.2f})")
    print("; ".join(report))
    assert ok, "; ".join(report)
