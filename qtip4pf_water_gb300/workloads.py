"""Named workloads of the benchmark configurations, each with the error report
that goes with its throughput.

    python -m qtip4pf_water_gb300.workloads <name> [--steps K] [--seed S]

prints one JSON line. Workloads (seeded lattice starts from start.py; the
reference names no dataset):

  headline      512 waters (L = 24.85 A), P = 32, Trotter + PILE-G, 298 K,
                dt = 0.25 fs, mixed precision: device steps only (the workload
                bench.py times; a light command for profiler captures).
  classical216  216 waters (L = 18.64 A), P = 1, Langevin (centroid PILE-L),
                298 K, dt = 0.5 fs: FP64 and mixed, ns/day, force RMS error of
                mixed against FP64, run-averaged kinetic / potential energy
                with standard errors for both.
  trotter216    216 waters, P = 32, Trotter + PILE-G, 298 K, dt = 0.25 fs:
                the same report.
  sc512         512 waters, P = 16, Suzuki-Chin, 298 K, dt = 0.25 fs: NVE
                energy drift per ns of the conserved quantity (mixed over
                --steps, FP64 over a shorter run), ns/day of both, force error.
  cmd           learned centroid correction: constrained-PIMD training data
                (216 waters, P = 32), training on the tensor cores, held-out
                error; surrogate CMD of 4096 waters (L = 49.7 A) against plain
                P = 32 PIMD centroid sampling, and the surrogate's error against
                fresh constrained-PIMD samples of that system.
  replicas48    48 independent replicas, N from {64, 128, 216, 343, 512},
                P from {8, 16, 32}, T uniform in [250, 350] K (seeded choice),
                Trotter + PILE-G, mixed: all replicas in one context (one
                CUDA-graph step for all, launch shapes autotuned) against the
                same systems run one context at a time; aggregate bead-steps/s.
  large4096     4096 waters (L = 49.7 A), P = 1, dt = 0.5 fs, mixed: NVE from
                one Langevin-equilibrated state with the real space over the
                pair list and over all pairs: drift and fluctuation of the
                conserved quantity, ns/day, force difference of the two forms.

Energies are in Hartree; drift is reported per ns and per molecule.
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np

from . import (FP64, MIXED, PILE_G, PILE_L, SUZUKI_CHIN, TROTTER, Context, system_desc)
from .start import SplitMix64, seeded_start

HARTREE_KCAL = 627.509474


def ns_per_day(step_seconds: float, dt_fs: float) -> float:
    return dt_fs * 1e-6 * 86400.0 / step_seconds


def block_se(x: np.ndarray, n_blocks: int = 10) -> float:
    """Standard error of the mean of a correlated series by block averaging."""
    x = np.asarray(x, dtype=np.float64)
    nb = min(n_blocks, len(x))
    if nb < 2:
        return float("nan")
    m = len(x) // nb
    b = x[: m * nb].reshape(nb, m).mean(axis=1)
    return float(b.std(ddof=1) / np.sqrt(nb))


def run_records(ctx: Context, sys_idx, n_steps: int, is_nvt: bool, chunk: int = 2000):
    """Advance the context n_steps (in chunks below the record ring's size) and
    return every step's estimators of the given systems, plus the wall time."""
    idx = [sys_idx] if isinstance(sys_idx, int) else list(sys_idx)
    out = {i: [] for i in idx}
    ctx.reset_estimators()
    t = 0.0
    done = 0
    while done < n_steps:
        n = min(chunk, n_steps - done)
        t0 = time.perf_counter()
        ctx.run_steps(n, is_nvt=is_nvt)
        ctx.sync()
        t += time.perf_counter() - t0
        for i in idx:
            out[i].append(ctx.systems[i].estimators())
        ctx.reset_estimators()
        done += n
    cat = {i: {k: np.concatenate([r[k] for r in out[i]]) for k in out[i][0]} for i in idx}
    return (cat[idx[0]] if isinstance(sys_idx, int) else cat), t


def make_ctx(descs, starts, precision, autotune=False):
    ctx = Context(descs, precision)
    for s, st in zip(ctx.systems, starts):
        s.set_state(st.q, st.p)
    tuned = ctx.autotune(5) if autotune else None
    ctx.init_forces()
    return ctx, tuned


def force_rms_error(q, box, n_mols, n_beads, temp, dt, prop, thermo):
    """Per-atom force RMS error of the mixed form relative to FP64 on one configuration."""
    f = {}
    for prec in (FP64, MIXED):
        ctx = Context([system_desc(n_mols, n_beads, box, temp_K=temp, dt_fs=dt, propagator=prop,
                                   thermostat=thermo)], prec)
        ctx.systems[0].set_state(q)
        ctx.init_forces()
        f[prec] = ctx.systems[0].get_state()["fphys"]
        ctx.close()
    d, r = f[MIXED] - f[FP64], f[FP64]
    return float(np.sqrt(np.mean(d * d) / np.mean(r * r)))


def _thermo_report(name, n_mols, n_beads, dt, prop, thermo, steps, seed, temp=298.0, warm=200):
    st = seeded_start(n_mols, n_beads, temp, seed=seed)
    rep = {"workload": name, "n_mols": n_mols, "n_beads": n_beads, "dt_fs": dt, "temp_K": temp, "steps": steps,
           "warmup_steps": warm}
    for prec, tag in ((FP64, "fp64"), (MIXED, "mixed")):
        d = system_desc(n_mols, n_beads, st.box_bohr, temp_K=temp, dt_fs=dt, propagator=prop, thermostat=thermo,
                        seed=seed)
        ctx, _ = make_ctx([d], [st], prec)
        run_records(ctx, 0, warm, True)
        rec, t = run_records(ctx, 0, steps, True)
        ke = rec["kcv"] if n_beads > 1 else rec["kin"]
        rep[tag] = {"ns_day": ns_per_day(t / steps, dt), "ms_per_step": t / steps * 1e3,
                    "kinetic_mean": float(np.mean(ke)), "kinetic_se": block_se(ke),
                    "potential_mean": float(np.mean(rec["pot"])), "potential_se": block_se(rec["pot"]),
                    "kinetic_estimator": "centroid virial" if n_beads > 1 else "classical"}
        ctx.close()
    for k in ("kinetic", "potential"):
        a, b = rep["fp64"], rep["mixed"]
        se = np.hypot(a[k + "_se"], b[k + "_se"])
        rep[k + "_diff_in_se"] = float(abs(a[k + "_mean"] - b[k + "_mean"]) / se) if se > 0 else None
    rep["mixed_over_fp64_speed"] = rep["mixed"]["ns_day"] / rep["fp64"]["ns_day"]
    rep["force_rms_rel_err_mixed_vs_fp64"] = force_rms_error(st.q, st.box_bohr, n_mols, n_beads, temp, dt, prop,
                                                             thermo)
    return rep


def classical216(steps=2000, seed=11):
    return _thermo_report("classical216", 216, 1, 0.5, TROTTER, PILE_L, steps, seed)


def trotter216(steps=1000, seed=12):
    return _thermo_report("trotter216", 216, 32, 0.25, TROTTER, PILE_G, steps, seed)


def _drift(rec, dt, n_mols):
    e = rec["conserved"]
    t_ns = np.arange(len(e)) * dt * 1e-6
    slope = np.polyfit(t_ns, e, 1)[0]
    return {"drift_hartree_per_ns": float(slope), "drift_hartree_per_ns_per_molecule": float(slope / n_mols),
            "drift_kcal_mol_per_ns_per_molecule": float(slope / n_mols * HARTREE_KCAL),
            "conserved_std_hartree": float(np.std(e)), "steps": int(len(e))}


def sc512(steps=40000, seed=13, fp64_steps=8000, equil=4000):
    """NVE drift of Suzuki-Chin PIMD: equil PILE-G steps in the mixed form from the
    lattice start, then the same state advanced NVE by the mixed form (steps) and
    by the FP64 form (fp64_steps); drift is also compared over the common window."""
    n, P, dt = 512, 16, 0.25
    st = seeded_start(n, P, 298.0, seed=seed)
    d = system_desc(n, P, st.box_bohr, dt_fs=dt, propagator=SUZUKI_CHIN, thermostat=PILE_G, seed=seed)
    ctx, _ = make_ctx([d], [st], MIXED)
    run_records(ctx, 0, equil, True)
    eq = ctx.systems[0].get_state()
    ctx.close()
    rep = {"workload": "sc512", "n_mols": n, "n_beads": P, "dt_fs": dt, "nvt_equilibration_steps": equil,
           "equilibration": "PILE-G, mixed form, from the seeded lattice start; both forms start NVE from its end state"}
    recs = {}
    for prec, tag, k in ((MIXED, "mixed", steps), (FP64, "fp64", fp64_steps)):
        ctx = Context([d], prec)
        ctx.systems[0].set_state(eq["q"], eq["p"])
        ctx.init_forces()
        rec, t = run_records(ctx, 0, k, False)
        recs[tag] = rec
        rep[tag] = dict(_drift(rec, dt, n), ns_day=ns_per_day(t / k, dt), ms_per_step=t / k * 1e3,
                        run_ps=k * dt * 1e-3)
        ctx.close()
    w = min(steps, fp64_steps)
    rep["common_window_steps"] = w
    rep["common_window_drift_kcal_mol_per_ns_per_molecule"] = {
        tag: _drift({"conserved": recs[tag]["conserved"][:w]}, dt, n)["drift_kcal_mol_per_ns_per_molecule"]
        for tag in recs}
    rep["mixed_over_fp64_speed"] = rep["mixed"]["ns_day"] / rep["fp64"]["ns_day"]
    rep["force_rms_rel_err_mixed_vs_fp64"] = force_rms_error(eq["q"], st.box_bohr, n, P, 298.0, dt, SUZUKI_CHIN,
                                                             PILE_G)
    return rep


def large4096(steps=20000, seed=15, equil=4000, n=4096, beads=1, dt=0.5):
    """Real space of large beads over the pair list against all pairs: n waters,
    P = beads, mixed; equil Langevin (PILE-L) steps from the seeded lattice start,
    then the same state advanced NVE with each real-space form. Reports the
    conserved-quantity drift and fluctuation of both runs, their step times, and
    the RMS difference of the two forms' forces on the list run's end state."""
    st = seeded_start(n, beads, 298.0, seed=seed)
    d = system_desc(n, beads, st.box_bohr, dt_fs=dt, propagator=TROTTER, thermostat=PILE_L, seed=seed)
    ctx, _ = make_ctx([d], [st], MIXED)
    run_records(ctx, 0, equil, True)
    eq = ctx.systems[0].get_state()
    ctx.close()
    rep = {"workload": "large4096", "n_mols": n, "n_beads": beads, "dt_fs": dt, "nvt_equilibration_steps": equil,
           "equilibration": "PILE-L, mixed form, pair-list real space, from the seeded lattice start"}
    end = None
    for form, tag in ((0, "pair_list"), (1, "all_pairs")):
        ctx = Context([d], MIXED)
        ctx.set_real_space(form)
        ctx.systems[0].set_state(eq["q"], eq["p"])
        ctx.init_forces()
        rec, t = run_records(ctx, 0, steps, False)
        rep[tag] = dict(_drift(rec, dt, n), ns_day=ns_per_day(t / steps, dt), ms_per_step=t / steps * 1e3,
                        run_ps=steps * dt * 1e-3)
        if form == 0:
            end = ctx.systems[0].get_state()
        else:  # the all-pairs forces at the list run's end state
            ctx.systems[0].set_state(end["q"], end["p"])
            ctx.init_forces()
            fa = ctx.systems[0].get_state()["fphys"]
            rep["force_rms_rel_diff_list_vs_all_pairs"] = float(
                np.sqrt(np.mean((end["fphys"] - fa) ** 2) / np.mean(fa ** 2)))
        ctx.close()
    rep["list_over_all_pairs_speed"] = rep["pair_list"]["ns_day"] / rep["all_pairs"]["ns_day"]
    return rep


def replica_set(seed=48, n=48):
    """The 48 replicas: (N, P, T, seed) by seeded choice."""
    rng = SplitMix64(seed)
    ns, ps = (64, 128, 216, 343, 512), (8, 16, 32)
    u = rng.u64(3 * n).reshape(n, 3)
    return [(ns[int(a % 5)], ps[int(b % 3)], 250.0 + 100.0 * (int(c >> 11) / float(1 << 53)), seed * 1000 + k)
            for k, (a, b, c) in enumerate(u)]


def replicas48(steps=200, seed=48, warm=10, compare=1, autotune=1):
    """The 48 uneven replicas in one context (one graph replay a step); with
    compare=1 also the same systems one context at a time; autotune=0 keeps the
    launcher's heuristic shapes (fewer launches ahead of the steps, for
    launch-list captures)."""
    reps = replica_set(seed)
    starts = [seeded_start(N, P, T, seed=s) for N, P, T, s in reps]
    descs = [system_desc(N, P, st.box_bohr, temp_K=T, dt_fs=0.25, propagator=TROTTER, thermostat=PILE_G, seed=s)
             for (N, P, T, s), st in zip(reps, starts)]
    bead_steps = sum(P for _, P, _, _ in reps) * steps
    # all replicas in one context
    ctx, tuned = make_ctx(descs, starts, MIXED, autotune=bool(autotune))
    ctx.run_steps(warm, is_nvt=True)
    ctx.sync()
    l0 = ctx.kernel_launches()
    t0 = time.perf_counter()
    ctx.run_steps(steps, is_nvt=True)
    ctx.sync()
    t_batch = time.perf_counter() - t0
    launches_per_step = (ctx.kernel_launches() - l0) / steps
    shape = ctx.tuning()
    ctx.close()
    # the same systems, one context at a time
    t_single = 0.0
    for d, st in zip(descs, starts) if compare else ():
        c1, _ = make_ctx([d], [st], MIXED, autotune=True)
        c1.run_steps(warm, is_nvt=True)
        c1.sync()
        t0 = time.perf_counter()
        c1.run_steps(steps, is_nvt=True)
        c1.sync()
        t_single += time.perf_counter() - t0
        c1.close()
    return {"workload": "replicas48", "replicas": len(reps), "steps": steps,
            "systems": [{"n_mols": N, "n_beads": P, "temp_K": round(T, 2)} for N, P, T, _ in reps],
            "total_beads": sum(P for _, P, _, _ in reps), "total_waters": sum(N for N, _, _, _ in reps),
            "batched_bead_steps_per_s": bead_steps / t_batch,
            "one_at_a_time_bead_steps_per_s": bead_steps / t_single if compare else None,
            "batched_speedup": t_single / t_batch if compare else None, "batched_ms_per_step": t_batch / steps * 1e3,
            "autotune_ms_heuristic_vs_tuned": tuned, "tuned_chunks_rj_sc_kc": shape,
            "launches_per_step": launches_per_step}


def cmd(n_configs=4096, constrained_steps=2000, replicas=64, fit_steps=2000, deploy_mols=4096, deploy_beads=32,
        fresh_configs=8, fresh_steps=2000, fresh_repeats=2, timing_steps=50, seed=5, train_mols=216, train_beads=32,
        held_out=256):
    """Learned centroid correction: training data from constrained PIMD of
    train_mols waters (train_beads beads), training on the tensor cores, held-out
    error; then surrogate CMD of deploy_mols waters against plain PIMD centroid
    sampling (deploy_beads beads), and the surrogate's centroid-force error
    judged against fresh constrained-PIMD samples of the deployed system.

    Each fresh centroid gets fresh_repeats independent constrained runs
    (different internal-mode starts and noise); the target is their mean, and
    the targets' own sampling noise is reported beside the errors: the noise
    floor is the RMS error a perfect predictor would show against the averaged
    target, RMS(run a - run b) / 2 over RMS(target) for two runs."""
    from . import surrogate as sg
    from .start import spread_beads

    rep = {"workload": "cmd", "train": {"n_mols": train_mols, "n_beads": train_beads, "configs": n_configs,
                                        "constrained_steps": constrained_steps, "replicas": replicas,
                                        "fit_steps": fit_steps}}
    t0 = time.perf_counter()
    ds = sg.generate(n_mols=train_mols, n_beads=train_beads, n_configs=n_configs, replicas=replicas,
                     equil_steps=2000, sample_every=200, constrained_steps=constrained_steps, seed=seed)
    rep["train"]["generate_s"] = time.perf_counter() - t0
    n_ho = min(held_out, max(1, n_configs // 8))
    train, test = ds.split(n_configs - n_ho)
    X, T = sg.features(train)
    model = sg.Correction(seed=seed)
    t0 = time.perf_counter()
    rep["train"]["final_loss"] = model.fit(X, T, steps=fit_steps)
    rep["train"]["fit_s"] = time.perf_counter() - t0
    rep["train"]["rows"] = int(len(X))
    rep["train"]["fit_ms_per_step"] = rep["train"]["fit_s"] / fit_steps * 1e3
    rep["held_out"] = model.evaluate(test)
    rep["held_out"]["on"] = f"{len(test)} configurations of {train_mols} waters not used in training"

    # deployment: surrogate CMD (P = 1 + correction) against plain PIMD centroid sampling
    st = seeded_start(deploy_mols, deploy_beads, 298.0, seed=seed + 7)
    box = st.box_bohr
    cents = st.q.reshape(deploy_beads, -1).mean(axis=0)
    c_ctx = Context([system_desc(deploy_mols, 1, box, dt_fs=0.25, propagator=TROTTER, thermostat=PILE_L,
                                 seed=seed)], MIXED)
    cs = c_ctx.systems[0]
    cs.set_state(cents)
    model.attach(cs)
    c_ctx.init_forces()
    c_ctx.run_steps(2000, is_nvt=True)  # equilibrate the centroids with the surrogate
    c_ctx.sync()
    t0 = time.perf_counter()
    c_ctx.run_steps(timing_steps * 10, is_nvt=True)
    c_ctx.sync()
    t_cmd = (time.perf_counter() - t0) / (timing_steps * 10)
    snaps = []
    for k in range(fresh_configs):
        c_ctx.run_steps(400, is_nvt=True)
        c_ctx.sync()
        snaps.append(cs.get_state()["q"].copy())
    c_ctx.close()
    p_ctx = Context([system_desc(deploy_mols, deploy_beads, box, dt_fs=0.25, propagator=TROTTER, thermostat=PILE_G,
                                 seed=seed)], MIXED)
    ps = p_ctx.systems[0]
    ps.set_state(st.q, st.p)
    p_ctx.init_forces()
    p_ctx.run_steps(5, is_nvt=True)
    p_ctx.sync()
    t0 = time.perf_counter()
    p_ctx.run_steps(timing_steps, is_nvt=True)
    p_ctx.sync()
    t_pimd = (time.perf_counter() - t0) / timing_steps
    # fresh constrained-PIMD mean centroid forces at the surrogate-CMD centroids,
    # fresh_repeats independent runs each (own bead spread; the stepper's noise
    # counter moves on between runs)
    runs = []
    for k, c in enumerate(snaps):
        per = []
        for r in range(fresh_repeats):
            q, p = spread_beads(c, deploy_beads, 298.0, seed=seed * 100 + 17 * k + r)
            ps.set_state(q, p)
            ps.set_centroid_fixed(True)
            p_ctx.init_forces()
            p_ctx.run_steps(200, is_nvt=True)  # internal modes relax around the fixed centroid
            ps.reset_centroid_force()
            p_ctx.run_steps(fresh_steps, is_nvt=True)
            p_ctx.sync()
            f, n = ps.centroid_force()
            per.append(f)
            ps.set_centroid_fixed(False)
        runs.append(per)
    p_ctx.close()
    runs = np.array(runs)  # [config][repeat][9N]
    snaps, fmean = np.array(snaps), runs.mean(axis=1)
    fclass = sg.classical_forces(snaps, deploy_mols, box)
    fresh = sg.Dataset(deploy_mols, box, snaps, fmean, fclass, {})
    den = float(np.sqrt(np.mean(fmean ** 2)))
    noise = None
    if fresh_repeats >= 2:
        diff = runs[:, 0] - runs[:, 1]
        # one run's noise is RMS(diff) / sqrt 2; the mean of R runs carries 1 / sqrt R of it
        noise = float(np.sqrt(np.mean(diff ** 2)) / np.sqrt(2.0) / np.sqrt(fresh_repeats) / den)
    rep["deploy"] = {"n_mols": deploy_mols, "box_angstrom": float(box[0] * 0.529177210903),
                     "surrogate_cmd_ms_per_step": t_cmd * 1e3, "surrogate_cmd_ns_day": ns_per_day(t_cmd, 0.25),
                     "pimd_ms_per_step": t_pimd * 1e3, "pimd_beads": deploy_beads,
                     "pimd_ns_day": ns_per_day(t_pimd, 0.25), "speedup_over_pimd": t_pimd / t_cmd,
                     "fresh_constrained_pimd": dict(model.evaluate(fresh), steps=fresh_steps, beads=deploy_beads,
                                                    repeats=fresh_repeats, target_noise_floor=noise)}
    ev = rep["deploy"]["fresh_constrained_pimd"]
    if noise is not None:
        # the error left once the targets' own noise is taken out (independent errors add in squares)
        ev["rms_rel_err_corrected_noise_removed"] = float(np.sqrt(max(ev["rms_rel_err_corrected"] ** 2 - noise ** 2,
                                                                      0.0)))
    return rep


def headline(steps=200, seed=2024):
    st = seeded_start(512, 32, 298.0, seed=seed)
    d = system_desc(512, 32, st.box_bohr, dt_fs=0.25, propagator=TROTTER, thermostat=PILE_G, seed=seed)
    ctx, _ = make_ctx([d], [st], MIXED)
    ctx.run_steps(5, is_nvt=True)
    ctx.sync()
    t0 = time.perf_counter()
    ctx.run_steps(steps, is_nvt=True)
    ctx.sync()
    t = time.perf_counter() - t0
    ctx.close()
    return {"workload": "headline", "steps": steps, "ms_per_step": t / steps * 1e3, "ns_day": ns_per_day(t / steps, 0.25)}


WORKLOADS = {"headline": headline, "classical216": classical216, "trotter216": trotter216, "sc512": sc512,
             "replicas48": replicas48, "cmd": cmd, "large4096": large4096}


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("name", choices=sorted(WORKLOADS))
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--seed", type=int, default=None)
    ap.add_argument("--arg", action="append", default=[], metavar="KEY=VALUE",
                    help="any other keyword of the workload function (numbers)")
    a = ap.parse_args(argv)
    kw = {}
    for item in a.arg:
        k, v = item.split("=", 1)
        kw[k] = float(v) if any(ch in v for ch in ".e") else int(v)
    if a.steps is not None:
        kw["steps"] = a.steps
    if a.seed is not None:
        kw["seed"] = a.seed
    print(json.dumps(WORKLOADS[a.name](**kw)), flush=True)


if __name__ == "__main__":
    main()
