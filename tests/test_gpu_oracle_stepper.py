"""The device-resident stepper against the oracle's restatement of it, step for
step with the same counter-based thermostat noise (the oracle recomputes the
Philox4x32-10 draws the device makes), and statistically with independent
noise streams.

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
1e-6 (FP64) or 1e-4 (mixed) relative RMS. Statistics: mean potential and
centroid-virial kinetic energy within two combined standard errors of block
averages.
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


def _block_stats(x, nblocks):
    n = len(x) // nblocks * nblocks
    b = np.asarray(x[:n]).reshape(nblocks, -1).mean(axis=1)
    return float(b.mean()), float(b.std(ddof=1) / np.sqrt(nblocks))


def test_nvt_averages_match_the_oracle_within_two_standard_errors(gpu_lib):
    """64 waters, P = 8, second order, PILE-G at 298 K, dt = 0.5 fs. Both sides
    start from one state equilibrated on the device (20 ps from the lattice) and
    sample with independent noise streams (different seeds): the device 20,000
    steps, the oracle 8,200 steps (200 discarded). Mean potential energy per bead and
    centroid-virial kinetic energy (the estimators simulation.cpp:936-961
    averages) agree within two combined standard errors of block means, the
    blocks 1000 steps (500 fs) long on both sides: longer than the potential
    energy's correlation time, so that the block means are independent and the
    standard errors not underestimated."""
    q = gpu_lib
    N, P, T, dt = 64, 8, 298.0, 0.5
    st = q.seeded_start(N, P, T, seed=91)
    ctx, s = _device(q, st, q.MIXED, q.TROTTER, q.PILE_G, 91, dt=dt)
    ctx.run_steps(40000, is_nvt=True)
    ctx.sync()
    eq = s.get_state()

    class Eq:
        n_mols, n_beads, box_bohr = N, P, st.box_bohr
        q = eq["q"].copy()
        p = eq["p"].copy()

    ctx2, s2 = _device(q, Eq, q.MIXED, q.TROTTER, q.PILE_G, 92, dt=dt)
    pot_g, kcv_g = [], []
    for _ in range(5):  # the device keeps the last 4096 records: read them every 4000 steps
        ctx2.reset_estimators()
        ctx2.run_steps(4000, is_nvt=True)
        ctx2.sync()
        est = s2.estimators()
        assert len(est["pot"]) == 4000
        pot_g.extend(est["pot"])
        kcv_g.extend(est["kcv"])

    o, stp, (qq, pp, f, fp, point, lst, disp) = _oracle(Eq, True, 1, 93, dt=dt)
    beta = 1.0 / (T * o.constants()[2])
    nd = 9 * N
    pot_o, kcv_o = [], []
    for k in range(8200):
        _, pot = o.stepper_step(stp, qq, pp, f, fp, point, lst, disp, is_nvt=True)
        if k < 200:
            continue
        x = qq.reshape(P, nd)
        tq = -np.sum((x - x.mean(axis=0)) * fp.reshape(P, nd))
        pot_o.append(pot)
        kcv_o.append(0.5 * nd / beta + 0.5 * tq / P)
    report, ok = [], True
    for name, g, c in (("potential", pot_g, pot_o), ("kinetic (centroid virial)", kcv_g, kcv_o)):
        mg, sg = _block_stats(g, 20)  # blocks of 1000 steps (500 fs) on both sides
        mo, so = _block_stats(c, 8)
        se = float(np.hypot(sg, so))
        ok = ok and abs(mg - mo) < 2.0 * se
        report.append(f"{name}: device {mg:.6f} +- {sg:.1e}, oracle {mo:.6f} +- {so:.1e}, "
                      f"difference {abs(mg - mo) / se:.2f} SE")
    assert ok, "; ".join(report)
