"""Benchmark: ns/day of 512-water, 32-bead PIMD on one GB300.

Workload (the headline): 512 flexible qTIP4P/F waters in a cubic box of
24.85 A (0.997 g/cm^3), P = 32 beads, 298 K, dt = 0.25 fs, second-order
(Trotter) ring-polymer propagation with the sqrt-Cayley free-ring-polymer
step and the PILE-G thermostat, Ewald eps = 1e-6. The start is the seeded
synthetic lattice of qtip4pf_water_gb300.start (synthetic data: the reference
names no dataset).

value  : ns/day of the mixed-precision form (FP32 Ewald with FP64 accumulation,
         FP64 LJ / intramolecular / integration / normal modes / thermostat),
         device-resident, one CUDA-graph replay per MD step, the L2 cache
         flushed (256 MiB write) before every timed step, flush not timed.
e2e    : the same workload driven through the reference-facing C-ABI call
         qtg_update_pimd (the update_sc_nospline drop-in) with pinned host
         buffers: every step copies the full state host->device and back.
Also reported: the plain-FP64 GPU form and the Suzuki-Chin propagator (mixed),
the mixed-vs-FP64 per-atom force RMS error, the roofline of the dominant
kernel and a CPU baseline (the C oracle, OpenMP over beads) on the host cores.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_MOLS, N_BEADS, TEMP, DT_FS, SEED = 512, 32, 298.0, 0.25, 2024
METRIC = "ns/day, 512 H2O P=32 PIMD: plain FP64 vs mixed/surrogate-CMD at stated error"
REF_SECONDS = 60.0
WORKLOAD = "512 H2O (L=24.85 A), P=32 PIMD, Trotter + PILE-G, 298 K, dt=0.25 fs, eps_ewald=1e-6"
# algorithmic work per force evaluation (fixed convention): real-space pair within
# r_c 60 flop, LJ pair within 9 A 30 flop, (site, k-vector) 20 flop (S(k) 8 +
# force 12), molecule intramolecular 150 flop
FLOP_REAL, FLOP_LJ, FLOP_SK, FLOP_KF, FLOP_INTRA = 60.0, 30.0, 8.0, 12.0, 150.0


def ns_per_day(step_seconds: float, dt_fs: float = DT_FS) -> float:
    return dt_fs * 1e-6 / step_seconds * 86400.0


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms while active."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.samples = []
        self._stop = threading.Event()
        self._proc = None
        self._thr = None

    def start(self):
        try:
            self._proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self._proc = None
            return
        self._thr = threading.Thread(target=self._read, daemon=True)
        self._thr.start()
        t0 = time.time()  # nvidia-smi takes a moment to start: let the samples cover the timed region
        while not self.samples and time.time() - t0 < 5.0:
            time.sleep(0.02)

    def _read(self):
        for line in self._proc.stdout:
            if self._stop.is_set():
                break
            self.samples.append([x.strip() for x in line.split(",")])

    def stop(self):
        self._stop.set()
        if self._proc:
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()
        if self._thr:
            self._thr.join(timeout=2)

    def summary(self):
        sm = [float(s[0]) for s in self.samples if s and s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if len(s) > 1 and s[1].replace(".", "").isdigit()]
        reasons = set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for s in self.samples:
            for k, n in enumerate(names):
                if len(s) > 4 + k and s[4 + k].lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.samples)}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def count_pairs(q, box, rc2, n_mols):
    """Site pairs of different molecules within rc (per bead, averaged) and O-O pairs within 9 A."""
    from qtip4pf_water_gb300.start import ANGS2BOHR

    P = q.shape[0]
    nreal = nlj = 0
    for b in range(0, P, max(1, P // 4)):
        x = q[b].reshape(n_mols, 3, 3)
        g = 0.73612
        s = x.copy()
        s[:, 0] = g * x[:, 0] + 0.5 * (1 - g) * (x[:, 1] + x[:, 2])
        s = s.reshape(-1, 3)
        mol = np.repeat(np.arange(n_mols), 3)
        for i0 in range(0, len(s), 256):
            d = s[i0:i0 + 256, None, :] - s[None, :, :]
            d -= box * np.round(d / box)
            r2 = (d * d).sum(-1)
            same = mol[i0:i0 + 256, None] == mol[None, :]
            nreal += int(((r2 < rc2) & ~same).sum())
        o = x[:, 0]
        d = o[:, None, :] - o[None, :, :]
        d -= box * np.round(d / box)
        r2 = (d * d).sum(-1)
        nlj += int(((r2 < (9.0 * ANGS2BOHR) ** 2).sum() - n_mols) // 2)
    nb = len(range(0, P, max(1, P // 4)))
    return nreal / 2.0 / nb, nlj / nb


def make_system(q_mod, precision, propagator, st, autotune=False):
    s = q_mod.System.create(N_MOLS, N_BEADS, st.box_bohr, precision=precision, temp_K=TEMP, dt_fs=DT_FS,
                            propagator=propagator, thermostat=q_mod.PILE_G, seed=SEED)
    s.set_state(st.q, st.p)
    if autotune:
        s.ctx.autotune(10)  # the library's launch-shape autotuner (chunk counts of the force kernels)
    s.ctx.init_forces()
    return s


def time_device_steps(s, steps, warmup, flush):
    """Per-step CUDA-event timing of graph replays; L2 flushed before each step (not timed)."""
    import torch

    # a dedicated stream: torch's default stream is the legacy NULL stream, which the
    # library would replace by its own non-blocking stream
    stream = torch.cuda.Stream()
    s.ctx.set_stream(stream.cuda_stream)
    s.ctx.run_steps(warmup, is_nvt=True)
    torch.cuda.synchronize()
    launches0 = s.ctx.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with torch.cuda.stream(stream):
        for k in range(steps):
            flush.zero_()
            ev[k][0].record(stream)
            s.ctx.run_steps(1, is_nvt=True)
            ev[k][1].record(stream)
    torch.cuda.synchronize()
    s.ctx.sync()
    ms = [a.elapsed_time(b) for a, b in ev]
    return sum(ms) / 1e3, s.ctx.kernel_launches() - launches0


def replica_timing(t_local, steps, world, dist=None, device="cpu"):
    """Replicas only: every rank times its own system; the job's time is the
    maximum over ranks, and its throughput is the world replicas' aggregate
    ns/day at that time. Returns (time, value)."""
    t = t_local
    if dist is not None and world > 1:
        import torch

        x = torch.tensor([t_local], dtype=torch.float64, device=device)
        dist.all_reduce(x, op=dist.ReduceOp.MAX)
        t = float(x.item())
    return t, ns_per_day(t / steps) * world


def run_gpu(args):
    import torch

    import qtip4pf_water_gb300 as q

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    st = q.seeded_start(N_MOLS, N_BEADS, TEMP, seed=SEED + rank)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    # ---- headline: mixed precision, Trotter -----------------------------------------------
    mix = make_system(q, q.MIXED, q.TROTTER, st, autotune=True)
    tuned = mix.ctx.tuning()
    sampler = ClockSampler(local)
    sampler.start()
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    t_mix, launches = time_device_steps(mix, args.steps, args.warmup, flush)
    torch.cuda.synchronize()
    sampler.stop()
    t_tot, value = replica_timing(t_mix, args.steps, world, dist, "cuda")
    ms_step = t_tot / args.steps * 1e3
    est = mix.estimators()
    fin = bool(np.all(np.isfinite(est["conserved"])))

    # ---- plain FP64 form and Suzuki-Chin (mixed) on the same start -------------------------
    k2 = max(3, min(args.steps, 10))
    f64 = make_system(q, q.FP64, q.TROTTER, st)
    f_mix0 = None
    t64, _ = time_device_steps(f64, k2, 3, flush)
    sc = make_system(q, q.MIXED, q.SUZUKI_CHIN, st)
    tsc, _ = time_device_steps(sc, k2, 3, flush)

    # force error of the mixed form against FP64 on one configuration (all beads)
    a = make_system(q, q.MIXED, q.TROTTER, st).get_state()["fphys"]
    b = make_system(q, q.FP64, q.TROTTER, st).get_state()["fphys"]
    f_err = float(np.sqrt(np.mean((a - b) ** 2) / np.mean(b ** 2)))
    del f_mix0

    # ---- end to end through the C-ABI call with host buffers -------------------------------
    e2e_py = run_e2e(q, st, min(args.steps, 200), flush)
    try:
        e2e = run_e2e_cabi(st, steps=min(args.steps, 200))
        e2e["python_binding"] = {k: e2e_py[k] for k in ("value", "ms_per_step", "call")}
    except (subprocess.SubprocessError, OSError, ValueError, IndexError) as exc:
        e2e = dict(e2e_py, cabi_error=str(exc)[-300:])

    try:
        e2e_dropin = run_e2e_dropin(st)
    except (subprocess.SubprocessError, OSError, ValueError, IndexError) as exc:
        e2e_dropin = {"error": str(exc)[-300:]}

    # ---- roofline of the dominant kernel -----------------------------------------------------
    roof = roofline(q, st, mix, t64 / k2)
    line = {
        "metric": METRIC,
        "value": value, "unit": "ns/day", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "fp32 Ewald / fp64 accumulation, integration, normal modes",
        "data": "synthetic (seeded lattice start, 512 waters, 32 beads)",
        "config": {"workload": WORKLOAD, "precision": "mixed", "propagator": "trotter", "thermostat": "pile_g",
                   "n_mols": N_MOLS, "n_beads": N_BEADS, "dt_fs": DT_FS,
                   "l2": "flushed (256 MiB write) before every timed step; flush not timed",
                   "launch_shapes": "autotuned chunks (real, structure factor, k-force) = %d, %d, %d" % tuned,
                   "parallelism": "replicas only" if world > 1 else "single GPU"},
        "bead_steps_per_s": N_BEADS * args.steps / t_mix,
        "fp64_ns_day": ns_per_day(t64 / k2), "fp64_ms_per_step": t64 / k2 * 1e3,
        "mixed_over_fp64": (t64 / k2) / (t_mix / args.steps),
        "sc_mixed_ns_day": ns_per_day(tsc / k2), "sc_mixed_ms_per_step": tsc / k2 * 1e3,
        "force_rms_rel_err_mixed_vs_fp64": f_err,
        "estimators_finite": fin,
        "gpu_launches": launches,
        "e2e": e2e,
        "e2e_dropin_sc": e2e_dropin,
        "roofline": roof["main"], "roofline_secondary": roof["secondary"], "kernel_ms": roof["kernel_ms"],
        "roofline_fp64_form": roof.get("fp64_form"), "fp64_peak_tflops": roof["fp64_peak_tflops"],
        "clocks": sampler.summary(),
    }
    if rank == 0:
        line["cpu_baseline"] = cpu_baseline(st, args.cpu_seconds)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_e2e(q, st, steps, flush, autotune=True):
    import torch

    s = q.System.create(N_MOLS, N_BEADS, st.box_bohr, precision=q.MIXED, temp_K=TEMP, dt_fs=DT_FS,
                        propagator=q.TROTTER, thermostat=q.PILE_G, seed=SEED)

    def pinned(a, dtype=torch.float64):
        t = torch.from_numpy(np.ascontiguousarray(a)).to(dtype).pin_memory()
        return t, t.numpy()

    _, qq = pinned(st.q)
    _, pp = pinned(st.p)
    pt, ls, dsp = s.build_lists(qq)
    _, point = pinned(pt, torch.int32)
    _, lst = pinned(ls, torch.int32)
    _, disp = pinned(dsp)
    _, f = pinned(np.zeros_like(st.q))
    _, fp = pinned(np.zeros_like(st.q))
    mass, charge = s.masses(), s.charges()
    s.set_state(st.q, st.p)  # the autotuner times force evaluations of the device state
    if autotune:  # the library's launch-shape autotuner, once at set-up as a user would
        s.ctx.autotune(10)
    s.force_eval_trotter(qq, f, charge, point, lst)
    fp[:] = f
    heat = 0.0
    nbytes = sum(a.nbytes for a in (qq, pp, f, fp, point, lst, disp)) + mass.nbytes + charge.nbytes
    for _ in range(10):
        _, heat, _ = s.update_sc_nospline(qq, pp, mass, f, fp, charge, point, lst, disp, True, heat)
    tot = 0.0
    b0 = s.ctx.transfer_bytes()
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, heat, _ = s.update_sc_nospline(qq, pp, mass, f, fp, charge, point, lst, disp, True, heat)
        tot += time.perf_counter() - t0
    b1 = s.ctx.transfer_bytes()
    del nbytes
    return {"value": ns_per_day(tot / steps), "unit": "ns/day", "h2d_bytes_per_step": (b1[0] - b0[0]) // steps,
            "d2h_bytes_per_step": (b1[1] - b0[1]) // steps, "ms_per_step": tot / steps * 1e3,
            "bytes_counted_by": "the library's own transfer counters (qtg_transfer_bytes)",
            "call": "qtg_update_pimd (update_sc_nospline drop-in), pinned host buffers, one call per step, "
                    "launch shapes autotuned once at set-up (qtg_autotune)"}


def ring_fp64_flop(P, n_dof):
    """FP64 flops one k_ring launch executes for one system, counted from its
    source: per dof column, four transforms (q and p, forward and back), each
    with the folds (8 (P/4 - 1) + 4 adds for P divisible by 4, else P - 1) and
    P rows of about 2 (P/4) + 0.5 flops (twice-folded) or P + 1 (once-folded);
    per bead and dof 26 flops for the kick, two half sqrt-Cayley steps, the O
    step and its heat."""
    if P % 4 == 0 and P >= 8:
        q4 = P // 4
        tr = 8 * (q4 - 1) + 4 + (2 * q4 + 0.5) * P
    else:
        tr = (P - 1) + (P + 1) * P
    return n_dof * (4 * tr + 26 * P)


def write_start(path, st):
    import struct

    with open(path, "wb") as f:
        f.write(struct.pack("<2i", st.n_mols, st.n_beads))
        f.write(struct.pack("<7d", *st.box_bohr, TEMP, DT_FS, 1e-6, 1e-5))
        f.write(np.ascontiguousarray(st.q, dtype="<f8").tobytes())
        f.write(np.ascontiguousarray(st.p, dtype="<f8").tobytes())


def run_e2e_cabi(st, warmup=10, steps=200):
    """The headline workload through qtg_update_pimd from host C++ (e2e_bench):
    host arrays registered once, moved inside every call's graph; L2 flushed
    before each call (outside the timer)."""
    import tempfile

    from qtip4pf_water_gb300 import build as qb

    qb.build()
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "start.bin")
        write_start(path, st)
        out = subprocess.check_output([qb.E2E_BENCH, path, str(warmup), str(steps), str(SEED)], text=True,
                                      timeout=900).split()
    ms, best, h2d, d2h, launches = float(out[0]), float(out[1]), int(out[2]), int(out[3]), float(out[4])
    return {"value": ns_per_day(ms * 1e-3), "unit": "ns/day", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
            "ms_per_step": ms, "min_ms_per_step": best, "gpu_launches_per_call": launches,
            "bytes_counted_by": "the library's own transfer counters (qtg_transfer_bytes)",
            "call": "qtg_update_pimd (update_sc_nospline entry) from host C++ (qtip4pf_water_gb300/csrc/driver/"
                    "e2e_bench.cpp), host arrays registered once with qtg_register_host, one call per step, launch "
                    "shapes autotuned once at set-up; L2 flushed before each call outside the timer",
            "steps": steps, "warmup": warmup}


def run_e2e_dropin(st, warmup=5, steps=40):
    """The drop-in as simulation.cpp drives it: update_sc_nospline on new[] arrays
    with the caller's std::mt19937 (host draws included), mixed precision."""
    import tempfile

    from qtip4pf_water_gb300 import build as qb

    qb.build()
    with tempfile.TemporaryDirectory() as tmp:
        path = os.path.join(tmp, "start.bin")
        write_start(path, st)
        env = dict(os.environ, QTG_PRECISION="mixed")
        out = subprocess.check_output([qb.DROPIN_BENCH, path, str(warmup), str(steps), str(SEED)], text=True,
                                      env=env, timeout=600).split()
    ms, draw_ms = float(out[0]), float(out[1])
    return {"value": ns_per_day(ms * 1e-3), "unit": "ns/day", "ms_per_step": ms, "host_draw_ms_per_step": draw_ms,
            "call": "update_sc_nospline through libqtip_compat.so (the reference's signature) from a C++ loop as "
                    "simulation.cpp:936-961 runs it: new[] state arrays (registered with the library on the first "
                    "call), PILE-G noise drawn on the host from the caller's std::mt19937 as thermostat.cpp draws it",
            "workload": "512 H2O, P=32, Suzuki-Chin (the reference's PIMD step), mixed precision, 298 K, 0.25 fs",
            "steps": steps, "warmup": warmup}


def roofline(q, st, mix, t64_step=None):
    hbm, which = _peaks()
    fp32 = q.fp32_peak_tflops()
    fp64 = q.fp64_peak_tflops()
    s = make_system(q, q.MIXED, q.TROTTER, st)
    info = s.info
    nreal, nlj = count_pairs(st.q, st.box_bohr, info.rc ** 2, N_MOLS)
    ms = {k: s.ctx.time_kernel(k, 20)
          for k in ("prep", "real", "ksk", "sk_reduce", "kforce", "combine", "lj", "ring", "end_step", "rebuild")}
    P, ns = N_BEADS, 3 * N_MOLS
    # algorithmic work per launch: each site pair within r_c counted once (60 flop),
    # each (site, k-vector) of the half set 8 flop for S(k) and 12 for the force
    flop = {"real": nreal * FLOP_REAL * P,
            "ksk": ns * info.n_kvectors * FLOP_SK * P, "kforce": ns * info.n_kvectors * FLOP_KF * P}
    top = max(("real", "ksk", "kforce"), key=lambda k: ms[k])
    ach = flop[top] / (ms[top] * 1e-3) / 1e12
    traffic = None
    tp = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(tp):
        with open(tp) as f:
            tj = json.load(f)
        traffic = tj.get(top)
    main = {"kernel": "k_" + top, "bound": "fp32", "achieved": ach, "peak": fp32, "unit": "TFLOP/s",
            "frac": ach / fp32, "traffic": traffic,
            "traffic_source": "not measured in this run: dram__bytes_read.sum + dram__bytes_write.sum per launch "
                              "from the ncu capture recorded in profiles/traffic.json (command there)",
            "peak_source": "FP32 FMA throughput measured live by qtg_fp32_peak (MEASURED_PEAKS.json has no FP32 figure)",
            "algorithmic_flop_per_launch": flop[top],
            "work": "site pairs within r_c once each x 60 flop x %d beads (%.0f pairs a bead)" % (P, nreal)}
    nd = 9 * N_MOLS
    ring_bytes = P * nd * 8 * 5  # read q, p, f; write q, p
    ring_bw = ring_bytes / (ms["ring"] * 1e-3) / 1e9
    ring_flop = ring_fp64_flop(P, nd)
    ring_tf = ring_flop / (ms["ring"] * 1e-3) / 1e12
    sec = {"kernel": "k_ring", "bound": "fp64", "achieved": ring_tf, "peak": fp64, "unit": "TFLOP/s",
           "frac": ring_tf / fp64, "peak_source": "FP64 FMA throughput measured live by qtg_fp64_peak",
           "fp64_flop_per_launch": ring_flop,
           "bytes": {"achieved_gbs": ring_bw, "peak_gbs": hbm, "frac": ring_bw / hbm,
                     "algorithmic_bytes_per_launch": ring_bytes, "peak_source": which + " (MEASURED_PEAKS.json hbm_gbs)"}}
    out = {"main": main, "secondary": sec, "kernel_ms": ms, "fp32_peak_tflops": fp32, "fp64_peak_tflops": fp64,
           "pairs_within_rc_per_bead": nreal, "lj_pairs_per_bead": nlj}
    if t64_step:
        per_eval = nreal * FLOP_REAL + nlj * FLOP_LJ + ns * info.n_kvectors * (FLOP_SK + FLOP_KF) + N_MOLS * FLOP_INTRA
        tf = per_eval * P / t64_step / 1e12
        out["fp64_form"] = {"achieved": tf, "peak": fp64, "unit": "TFLOP/s", "frac": tf / fp64,
                            "work": "algorithmic flop of one step (%d force evaluations) / step time" % P}
    return out


def pile_noise(rng, n_dof, n_beads):
    """One PILE-G step's draws in the oracle's layout [R, chi^2(n_dof - 1), xi(beads 1..P-1)]."""
    return np.concatenate(([rng.standard_normal(), rng.chisquare(n_dof - 1)],
                           rng.standard_normal((n_beads - 1) * n_dof)))


def cpu_baseline(st, seconds):
    """The oracle's Trotter step on the host cores (OpenMP over beads), bounded sample."""
    from oracle.binding import Oracle, build

    build()
    threads = os.cpu_count() or 1
    o = Oracle(N_MOLS, N_BEADS, st.box_bohr, TEMP, DT_FS)
    qq, pp = st.q.copy(), st.p.copy()
    point, lst, disp = o.build_lists(qq)
    f = np.zeros_like(qq)
    fp = np.zeros_like(qq)
    o.force_eval_trotter(qq, f, point, lst)
    rng = np.random.default_rng(SEED)
    t0 = time.perf_counter()
    n = 0
    while True:
        o.update_pimd(qq, pp, f, fp, point, lst, disp, is_nvt=True, trotter=True,
                      noise=pile_noise(rng, 9 * N_MOLS, N_BEADS))
        n += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = (time.perf_counter() - t0) / n
    return {"value": ns_per_day(dt), "unit": "ns/day", "cores": threads, "kind": "port",
            "sample": f"{n} Trotter + PILE-G steps of the benchmark workload (512 H2O, P=32) with the C oracle, "
                      f"OpenMP over beads, {threads} threads; {dt:.3f} s/step"}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from oracle.binding import Oracle, build

    from qtip4pf_water_gb300.start import seeded_start

    build()
    threads = os.cpu_count() or 1
    st = seeded_start(N_MOLS, N_BEADS, TEMP, seed=SEED)
    o = Oracle(N_MOLS, N_BEADS, st.box_bohr, TEMP, DT_FS)
    qq, pp = st.q.copy(), st.p.copy()
    point, lst, disp = o.build_lists(qq)
    f = np.zeros_like(qq)
    fp = np.zeros_like(qq)
    o.force_eval_trotter(qq, f, point, lst)
    rng = np.random.default_rng(SEED)
    for _ in range(args.warmup):
        o.update_pimd(qq, pp, f, fp, point, lst, disp, is_nvt=True, trotter=True,
                      noise=pile_noise(rng, 9 * N_MOLS, N_BEADS))
    # each oracle step takes ~0.2 s on 16 cores: time at most REF_SECONDS of the K steps asked for
    t0 = time.perf_counter()
    n = 0
    while n < args.steps:
        o.update_pimd(qq, pp, f, fp, point, lst, disp, is_nvt=True, trotter=True,
                      noise=pile_noise(rng, 9 * N_MOLS, N_BEADS))
        n += 1
        if time.perf_counter() - t0 > REF_SECONDS:
            break
    dt = (time.perf_counter() - t0) / n
    v = ns_per_day(dt)
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "ns/day",
            "n_gpus": 0, "steps": n, "warmup": args.warmup, "ms_per_step": dt * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "fp64",
            "data": "synthetic (seeded lattice start, 512 waters, 32 beads)",
            "config": {"workload": WORKLOAD, "precision": "fp64", "propagator": "trotter"},
            "cpu_baseline": {"value": v, "unit": "ns/day", "cores": threads, "kind": "port",
                             "sample": f"{n} timed Trotter + PILE-G steps (of {args.steps} asked; at most {REF_SECONDS:.0f} s, "
                                       f"after {args.warmup} warm-up) of the benchmark workload with the C oracle, "
                                       f"OpenMP over beads, {threads} threads"},
            "e2e": {"value": v, "unit": "ns/day", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3000)  # ~1.7 s timed: several clock samples
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
