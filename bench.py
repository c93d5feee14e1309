#!/usr/bin/env python3
"""P3M force-and-step throughput (particle-steps/s) on GB300: plain P3M vs the learned closure.

Workload (default, the metric's configuration): the 1,048,576-particle exponential disk +
Plummer bulge, 128^3 mesh, TSC, S2-shaped particles, P3M cutoff 3 mesh cells on the y-sorted
chaining mesh, dt = 0.005 (particlesimulation_gb300.workloads.disk_p3m_1m).  A step is one
iteration of the reference's run loop: drift, force (cell lists, deposit, FFT Poisson solve,
interpolation, short-range pair pass), kick.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

ours:       the learned closure (pair cutoff 1.5 mesh cells + MLP residual) is trained on residuals
            of the plain P3M (untimed set-up), then K judged steps run: every 10th step the plain
            full-cutoff P3M judges the closure (median relative force difference over every 16th
            particle) and the rest of the run falls back to plain P3M when it exceeds the bound
            (default 1e-3, the target force error).  `value` is that judged run, judge and
            fallback included: W warm-up steps, then K steps each timed with CUDA events on the
            handle's stream, L2 flushed (256 MB write) before every step.  Replicas only for N > 1.
            e2e: the same judged steps through the C ABI with host buffers (state copied
            host->device from pinned memory every step, state and accelerations read back).
            The line also reports both modes alone, their force errors against an FP64 direct
            sum on 8,192 particles (at the training positions and again after the judged run
            is continued to 200 steps), the roofline of the dominant kernel (the learned step's
            reduced-cutoff pair pass; plain P3M's full-cutoff pass beside it), and the other
            workloads (disk_p3m, pm_hbm, ensemble).
reference:  the reference's CPU P3M path (the oracle port of it: oracle/port.cpp, float, all
            host threads) on the same workload; each step a bounded sample (see cpu_sample()).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s on 1 GB300: plain P3M vs learned closure at equal force error"
UNIT = "particle-steps/s"
L2_FLUSH_BYTES = 256 << 20
# CPU samples per workload: (pair stride S: every S-th particle is an i-particle of the pair pass,
# j loops complete, time x S; fill stride F: the y-sorting insertion sort on every F-th particle,
# time x F^2)
CPU_SAMPLE = {"disk_p3m_1m": (1024, 32), "disk_p3m": (64, 1)}
JUDGE_INTERVAL, JUDGE_STRIDE, ERR_TARGETS = 10, 16, 8192


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="disk_p3m_1m")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-closure", action="store_true",
                    help="skip the plain-P3M vs learned-closure comparison")
    ap.add_argument("--no-ensemble", action="store_true",
                    help="skip the 64-system ensemble measurement")
    ap.add_argument("--no-reference-scenarios", action="store_true",
                    help="skip the reference's own timing scenarios (run by the scenario CLI)")
    ap.add_argument("--no-pm-hbm", action="store_true",
                    help="skip the HBM-roofline measurement of the PM path on the 256^3 workload")
    ap.add_argument("--closure-epochs", type=int, default=60)
    ap.add_argument("--closure-bound", type=float, default=1e-3,
                    help="judge bound: median relative deviation from plain P3M (the target force "
                         "error)")
    ap.add_argument("--no-reference-table", action="store_true",
                    help="skip the closure comparison with the reference's 500-entry table")
    ap.add_argument("--no-disk-p3m", action="store_true",
                    help="skip the plain P3M measurement on the 262,144-particle disk")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--profile-closure", type=int, default=0, metavar="K",
                    help="only run K learned-closure steps on the 1,048,576-particle disk (untrained "
                         "weights: same work) and print the stage times (the command profiled "
                         "with ncu)")
    ap.add_argument("--profile-forces", type=int, default=0, metavar="K",
                    help="only run K force evaluations of the workload and print the stage "
                         "times (the command profiled with ncu)")
    return ap.parse_args()


def run_profile_forces(args):
    from particlesimulation_gb300 import workloads as W
    w = W.WORKLOADS[args.workload]()
    pm, p3m = make_system(w)
    for _ in range(args.profile_forces):
        (p3m.force() if p3m else pm.pmMethodStep())
    out = {"stage_ms": pm.stageTimes()}
    if p3m:
        p3m.setPairCounting(True)
        p3m.force()
        out["ordered_pairs"] = p3m.pairCount()
        p3m.close()
    pm.close()
    print(json.dumps(out))


def run_profile_closure(args):
    import particlesimulation_gb300 as P
    from particlesimulation_gb300 import workloads as W
    w = W.disk_p3m_1m()
    pm, _ = make_system(W.Workload(**{**w.__dict__, "p3m": None}))
    q = w.p3m
    cl = P.LearnedClosure(pm, q["comp_box"], q["cutoff"], q["diameter"], q["softening"],
                          P.CloudShape(q["cloud_shape"]), 0.5 * q["cutoff"], seed=args.seed,
                          useSRForceTable=bool(q["table"]))
    cl.setMode(cl.LEARNED)
    pm.run(0)
    _, _, ms = pm.advance(args.profile_closure)
    print(json.dumps({"learned_ms_per_step": ms / max(args.profile_closure, 1)}))
    cl.close()
    pm.close()


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def config_of(w):
    d = dict(workload=f"{w.name}: {w.n:,} particles, {w.grid[0]}^3 mesh, "
                      f"{['NGP', 'CIC', 'TSC'][w.interpolation]}, "
                      + (f"P3M cutoff {w.p3m['cutoff'] / w.H:g} mesh cells" if w.p3m else "PM"),
             particles=w.n, mesh=list(w.grid), dt=w.DT, method="P3M" if w.p3m else "PM",
             parallelism="replicas")
    return d


def load_peaks():
    for p in (os.path.join(ROOT, "MEASURED_PEAKS.json"),):
        if os.path.exists(p):
            with open(p) as f:
                return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms while running."""

    def __init__(self, gpu_id: str):
        self.gpu_id = gpu_id
        self.proc = None
        self.f = None

    def start(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", self.gpu_id, f"--query-gpu={q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.1)

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        self.proc.wait()
        self.f.close()
        rows = []
        with open(self.f.name) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) == 7 and parts[0].replace(".", "").isdigit():
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(float(r[0]) for r in rows),
                "sm_max_mhz": max(float(r[1]) for r in rows),
                "power_w_max": max(float(r[2]) for r in rows if r[2].replace(".", "").isdigit()),
                "reasons": reasons, "samples": len(rows)}


def cpu_sample(w, threads, steps=1):
    """The reference's CPU P3M step on the full workload, sampled (CPU_SAMPLE): the PM part runs
    on all particles; the y-sorted chaining-mesh build (the reference's insertion sort) on every
    F-th particle, its time scaled by F^2; the short-range pair pass on every S-th particle by
    index (complete j loops), its time scaled by S.  Returns (particle-steps/s, estimated seconds
    per full step, breakdown incl. the wall time the sampled steps took per step)."""
    from oracle import oracle as O
    cfg = O.PMConfig(grid=w.grid, box=w.box, H=w.H, DT=w.DT, G=w.G, interpolation=w.interpolation,
                     finite_diff=w.finite_diff, greens=w.greens, diameter=w.diameter,
                     periodic=int(w.periodic))
    q = None
    if w.p3m:
        q = O.P3MConfig(comp_box=w.p3m["comp_box"], cutoff=w.p3m["cutoff"],
                        diameter=w.p3m["diameter"], softening=w.p3m["softening"],
                        cloud_shape=w.p3m["cloud_shape"], use_table=w.p3m["table"],
                        y_sorting=w.p3m["ysort"])
    ps, fs = CPU_SAMPLE.get(w.name, (1, 1)) if q else (1, 1)
    r = O.port_time_steps(cfg, q, w.pos, w.vel, w.mass, steps, threads, ps, fs)
    return w.n / r["est"], r["est"], r


def sample_text(w):
    if not w.p3m:
        return f"{w.name}, all {w.n:,} particles, full PM steps; oracle port of the reference's CPU PM in float"
    ps, fs = CPU_SAMPLE.get(w.name, (1, 1))
    return (f"{w.name}, all {w.n:,} particles: PM step in full; y-sorted chaining-mesh build "
            f"(the reference's insertion sort) on every {fs}th particle, time x {fs}^2; short-range "
            f"pair pass for every {ps}th particle by index (complete j loops), time x {ps}; "
            "oracle port of the reference's CPU P3M in float")


def make_system(w):
    import particlesimulation_gb300 as P
    pm = P.PMMethod(w.state, w.mass, w.box, None, w.H, w.DT, w.G,
                    P.InterpolationScheme(w.interpolation), P.FiniteDiffScheme(w.finite_diff),
                    P.GreensFunction(w.greens), w.diameter, w.grid, periodic=w.periodic)
    p3m = None
    if w.p3m:
        q = w.p3m
        p3m = P.P3MMethod(pm, q["comp_box"], q["cutoff"], q["diameter"], w.H, q["softening"],
                          P.CloudShape(q["cloud_shape"]), bool(q["table"]), bool(q["ysort"]))
    return pm, p3m


class StreamTimer:
    """CUDA events recorded on a handle's own stream (torch.cuda.Event on the current torch
    stream would not see the library's work)."""

    def __init__(self, stream_ptr):
        import torch
        self.torch = torch
        self.stream = torch.cuda.ExternalStream(stream_ptr)
        self.pairs = []

    def start(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        self.pairs.append([e, None])

    def stop(self):
        e = self.torch.cuda.Event(enable_timing=True)
        e.record(self.stream)
        self.pairs[-1][1] = e

    def total_ms(self):
        self.torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in self.pairs)


def med_err(a, ref):
    """Per-particle relative force errors |a - ref| / |ref|: median, 90th percentile, max, and the
    RMS-normalised figure sqrt(mean |a - ref|^2 / mean |ref|^2)."""
    import numpy as np
    a = np.asarray(a, np.float64)
    d = np.linalg.norm(a - ref, axis=1)
    r = np.linalg.norm(ref, axis=1)
    e = d / np.maximum(r, 1e-300)
    return {"median": float(np.median(e)), "p90": float(np.percentile(e, 90)), "max": float(e.max()),
            "rms_normalised": float(np.sqrt((d * d).mean() / (r * r).mean()))}


def pair_roofline(pm, p3m, flush_l2, fp32_peak):
    """Roofline of the short-range pair pass: 20 FLOP per unordered pair within the cutoff (the
    exact count from one counting evaluation) over the pass's CUDA-event time (median of 3
    evaluations, L2 flushed before each), against the FP32 FMA peak measured in this run."""
    import statistics
    p3m.setPairCounting(True)
    p3m.force()
    pairs = p3m.pairCount() / 2.0
    p3m.setPairCounting(False)
    ms, stage = [], None
    for _ in range(3):
        flush_l2()
        p3m.force()
        stage = pm.stageTimes()
        ms.append(stage["pair"])
    t = statistics.median(ms)
    flop = 20.0 * pairs
    achieved = flop / (t * 1e-3) / 1e12
    return {"kernel": "pair_slot_kernel + pair_epilogue_kernel", "bound": "fp32",
            "achieved": round(achieved, 3), "peak": round(fp32_peak, 3), "unit": "TFLOP/s",
            "frac": round(achieved / fp32_peak, 4), "traffic": None,
            "traffic_note": "DRAM bytes are read by ncu, not in this run (profiles/)",
            "peak_source": "FP32 FMA probe measured in this run (pmgb_fp32_peak_probe); the pair "
                           "pass is CUDA-core FP32 bound, not HBM or tensor",
            "flop_per_launch": flop, "pairs_in_range_unordered": pairs,
            "launch_ms": round(t, 4)}, stage


def run_ours(args):
    import torch

    from particlesimulation_gb300 import workloads as W

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")

    def flush_l2():
        flush.random_(0, 255)
        torch.cuda.synchronize()

    props = torch.cuda.get_device_properties(local)
    uuid = getattr(props, "uuid", None)
    clocks = ClockSampler(f"GPU-{uuid}" if uuid is not None else str(local))
    w = W.WORKLOADS[args.workload]()
    if w.name == "disk_p3m_1m":
        line = closure_headline(args, w, flush_l2, clocks, rank, world)
    else:
        line = plain_headline(args, w, flush_l2, clocks, rank, world)
    default = args.workload == "disk_p3m_1m"
    if default and not args.no_disk_p3m:
        line["disk_p3m"] = plain_headline(args, W.disk_p3m(), flush_l2, None, rank, world,
                                          brief=True)
    if default and not args.no_ensemble:
        line["ensemble"] = ensemble_bench(args, rank, world)
    if default and not args.no_pm_hbm:
        line["pm_hbm"] = pm_hbm_bench(args, rank, world)
    if rank == 0 and world == 1 and default and not args.no_reference_scenarios:
        line["reference_scenarios"] = reference_scenarios()
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        torch.distributed.destroy_process_group()


def max_over_ranks(x, world):
    import torch
    if world == 1:
        return x
    t = torch.tensor([x], device="cuda", dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    torch.distributed.barrier()
    return float(t.item())


def e2e_steps(pm, steps, step_fn, world, n):
    """Steps through the C ABI with host buffers: per step the state is copied from pinned host
    memory to the device (pmgb_pm_set_particles), stepped, and positions, velocities and
    accelerations are read back (pmgb_pm_get_particles).  Host wall clock, synchronised."""
    import torch
    pos_h = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    vel_h = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    acc_h = torch.empty((n, 3), dtype=torch.float32, pin_memory=True).numpy()
    pm.getParticles(units="original", pos=pos_h, vel=vel_h, acc=acc_h)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(steps):
        pm.setParticles(pos_h, vel_h, units="original")
        step_fn(s)
        pm.getParticles(units="original", pos=pos_h, vel=vel_h, acc=acc_h)
    torch.cuda.synchronize()
    sec = max_over_ranks(time.perf_counter() - t0, world)
    return {"value": world * n * steps / sec, "unit": UNIT,
            "h2d_bytes_per_step": int(pos_h.nbytes + vel_h.nbytes),
            "d2h_bytes_per_step": int(pos_h.nbytes + vel_h.nbytes + acc_h.nbytes)}


def cpu_baseline_obj(w, args, rank, world):
    if rank != 0 or world != 1 or args.no_cpu_baseline:
        return None
    threads = os.cpu_count()
    v, sec, r = cpu_sample(w, threads)
    return {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample_text(w),
            "seconds_per_step_estimated": sec, "sample_wall_s": round(float(r["wall"]), 3),
            "breakdown_s": {k: round(float(x), 4) for k, x in r.items()}}


def plain_headline(args, w, flush_l2, clocks, rank, world, brief=False):
    """Plain PM / P3M on one workload: W warm-up steps, K steps each timed with CUDA events on
    the handle's stream (pmgb_pm_advance) after an L2 flush; the pair-pass roofline (P3M) and the
    HBM roofline of the PM stages; e2e through the C ABI; the CPU baseline."""
    import numpy as np

    import particlesimulation_gb300 as P
    pm, p3m = make_system(w)
    escaped, _ = pm.run(0)  # initial force, half kick, first iteration (state ready for advance)
    if escaped:
        raise RuntimeError("a particle left the box during set-up")
    for _ in range(args.warmup):
        flush_l2()
        pm.advance(1)
    max_over_ranks(0.0, world)
    launches0 = pm.kernelLaunches()
    if clocks:
        clocks.start()
    total_ms = 0.0
    for _ in range(args.steps):
        flush_l2()
        esc, _, ms = pm.advance(1)
        if esc:
            raise RuntimeError("a particle left the box during the timed steps")
        total_ms += ms
    clk = clocks.stop() if clocks else None
    launches = pm.kernelLaunches() - launches0
    total_ms = max_over_ranks(total_ms, world)
    ms_step = total_ms / args.steps
    value = world * w.n * args.steps / (total_ms * 1e-3)
    peaks, peak_src = load_peaks()
    roofline = None
    if p3m:
        roofline, stage = pair_roofline(pm, p3m, flush_l2, P.methods.fp32_peak_tflops())
    else:
        flush_l2()
        pm.pmMethodStep()
        stage = pm.stageTimes()
    pm_ms = stage["deposit"] + stage["poisson"] + stage["interpolation"]
    pm_bytes = 60.0 * w.n + 26.0 * float(np.prod(w.grid))
    roofline_pm = {"bound": "hbm", "achieved": round(pm_bytes / (pm_ms * 1e-3) / 1e9, 1),
                   "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                   "frac": round(pm_bytes / (pm_ms * 1e-3) / 1e9 / peaks.get("hbm_gbs"), 4),
                   "bytes_per_step": pm_bytes, "stage_ms": {k: round(v, 4) for k, v in stage.items()},
                   "peak_source": peak_src}
    e2e = e2e_steps(pm, args.steps, lambda s: pm.advance(1), world, w.n)
    cpu = cpu_baseline_obj(w, args, rank, world)
    if p3m:
        p3m.close()
    pm.close()
    if brief:
        return {"value": value, "unit": UNIT, "ms_per_step": ms_step, "steps": args.steps,
                "config": config_of(w), "e2e": e2e, "roofline": roofline,
                "roofline_pm": roofline_pm, "cpu_baseline": cpu}
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, particlesimulation_gb300/workloads.py)",
            "config": {**config_of(w), "l2": "256 MB L2 flush before every timed step"},
            "e2e": e2e, "roofline": roofline, "roofline_pm": roofline_pm, "cpu_baseline": cpu,
            "clocks": clk, "gpu_launches": launches, "impl": "ours"}


def closure_config(w, bound=1e-3):
    """config of the metric's workload, the same in both arms."""
    return {**config_of(w), "method": "P3M; learned short-range closure judged by plain P3M",
            "short_range_force": "500-entry table" if w.p3m["table"] else
            "exact formula (useSRForceTable = false)",
            "closure_pair_cutoff_cells": 0.5 * w.p3m["cutoff"] / w.H, "closure_bound": bound,
            "l2": "256 MB L2 flush before every timed step"}


def closure_errors(pm, cl, w):
    """At the current positions: the forces of plain P3M, the learned closure and the reduced
    cutoff alone against an FP64 direct sum on ERR_TARGETS particles (median / p90 / max
    relative error), the two reduced modes against plain P3M, and the judge's median relative
    difference (learned vs plain, every JUDGE_STRIDE-th slice).  Leaves the learned mode set."""
    import numpy as np

    from particlesimulation_gb300 import methods as M
    acc = {}
    for name, mode in (("plain_p3m", cl.FULL), ("learned_closure", cl.LEARNED),
                       ("reduced_cutoff_alone", cl.REDUCED_ONLY)):
        cl.setMode(mode)
        cl.force()
        x, _, a = pm.getParticles(units="original")
        acc[name] = a
    rng = np.random.default_rng(12345)
    idx = np.sort(rng.choice(w.n, ERR_TARGETS, replace=False)).astype(np.int32)
    a_pp = M.direct_sum_fp64(x, w.mass, w.G, idx)
    errors = {k: med_err(a[idx], a_pp) for k, a in acc.items()}
    vs_plain = {k: med_err(acc[k][idx], acc["plain_p3m"][idx].astype(np.float64))
                for k in ("learned_closure", "reduced_cutoff_alone")}
    cl.setMode(cl.LEARNED)
    judge = cl.judge(stride=JUDGE_STRIDE)
    return errors, vs_plain, judge


def closure_setup(args, w, flush_l2):
    """PM + learned closure on the workload, trained (untimed): training rows from the plain P3M
    at t = 0 and after 50 steps (2 x N rows), GPU training.  Then, at the same positions, the
    force errors of plain P3M, the learned closure and the reduced cutoff alone against an FP64
    direct sum on ERR_TARGETS particles, the judge's median relative difference (learned vs
    plain), and each mode's own step time (CUDA events on the handle's stream, L2 flushed)."""
    import numpy as np

    import particlesimulation_gb300 as P
    from particlesimulation_gb300 import methods as M
    pm = P.PMMethod(w.state, w.mass, w.box, None, w.H, w.DT, w.G,
                    P.InterpolationScheme(w.interpolation), P.FiniteDiffScheme(w.finite_diff),
                    P.GreensFunction(w.greens), w.diameter, w.grid)
    q = w.p3m
    cl = P.LearnedClosure(pm, q["comp_box"], q["cutoff"], q["diameter"], q["softening"],
                          P.CloudShape(q["cloud_shape"]), 0.5 * q["cutoff"], capacity=2 * w.n,
                          seed=args.seed, useSRForceTable=bool(q["table"]))
    t0 = time.perf_counter()
    cl.collect()
    pm.run(0)
    pm.advance(50)
    rows = cl.collect()
    t1 = time.perf_counter()
    loss = cl.train(epochs=args.closure_epochs, batch=2048, lr=2e-3)
    t2 = time.perf_counter()
    t3 = time.perf_counter()
    errors, vs_plain, judge = closure_errors(pm, cl, w)
    t4 = time.perf_counter()
    stream = pm.stream()

    def mode_ms(mode, steps):
        cl.setMode(mode)
        for _ in range(2):
            pm.advance(1)
        tm = StreamTimer(stream)
        for _ in range(steps):
            flush_l2()
            tm.start()
            esc, _, _ = pm.advance(1)
            tm.stop()
            if esc:
                raise RuntimeError("a particle left the box")
        return tm.total_ms() / steps

    ms_plain = mode_ms(cl.FULL, min(args.steps, 10))
    ms_learned = mode_ms(cl.LEARNED, min(args.steps, 10))
    summary = {
        "short_range_force": "500-entry table" if q["table"] else "exact formula (useSRForceTable = false)",
        "judge_median_rel_diff_learned_vs_plain": judge,
        "plain_p3m": {"value": w.n / (ms_plain * 1e-3), "ms_per_step": ms_plain,
                      "force_err_vs_fp64_direct": errors["plain_p3m"]},
        "learned_closure": {"value": w.n / (ms_learned * 1e-3), "ms_per_step": ms_learned,
                            "force_err_vs_fp64_direct": errors["learned_closure"],
                            "force_diff_vs_plain_p3m": vs_plain["learned_closure"]},
        "reduced_cutoff_alone": {"force_err_vs_fp64_direct": errors["reduced_cutoff_alone"],
                                 "force_diff_vs_plain_p3m": vs_plain["reduced_cutoff_alone"]},
        "learned_speedup_unjudged": ms_plain / ms_learned,
        "training": {"rows": rows, "epochs": args.closure_epochs, "final_mse": loss,
                     "collect_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2)},
        "direct_sum": {"targets": ERR_TARGETS, "sources": w.n, "seconds": round(t4 - t3, 3),
                       "precision": "fp64", "device": "gpu (pmgb_direct_sum_fp64)"}}
    return pm, cl, summary


def closure_headline(args, w, flush_l2, clocks, rank, world):
    """The metric's configuration: plain P3M vs the learned closure on the 1,048,576-particle
    disk (closure_setup), then the headline: K steps of the judged run (the closure checked by
    plain P3M every JUDGE_INTERVAL steps, fallback to plain P3M above args.closure_bound), CUDA
    events on the handle's stream around each step, judge and fallback included; e2e through the
    C ABI; the roofline of the learned step's reduced-cutoff pair pass (the headline's dominant
    kernel) and of plain P3M's full-cutoff pass; the same comparison with the reference's 500-entry
    table (closure.reference_table)."""
    import particlesimulation_gb300 as P
    from particlesimulation_gb300 import methods as M
    from particlesimulation_gb300 import workloads as W
    pm, cl, summary = closure_setup(args, w, flush_l2)
    stream = pm.stream()
    q = w.p3m

    def judged_step(s):
        iv = 1 if s % JUDGE_INTERVAL == 0 else 0  # judge this step after it ran (learned mode only)
        esc, _, fb, _ = cl.run(1, args.closure_bound, iv, JUDGE_STRIDE)
        if esc:
            raise RuntimeError("a particle left the box")
        return fb

    cl.setMode(cl.LEARNED)
    for s in range(args.warmup):
        flush_l2()
        judged_step(s)
    cl.setMode(cl.LEARNED)
    max_over_ranks(0.0, world)
    tm = StreamTimer(stream)
    launches0 = pm.kernelLaunches()
    clocks.start()
    fallback = -1
    for s in range(args.steps):
        flush_l2()
        tm.start()
        fb = judged_step(s)
        tm.stop()
        if fb >= 0 and fallback < 0:
            fallback = s
    total_ms = tm.total_ms()
    clk = clocks.stop()
    launches = pm.kernelLaunches() - launches0
    total_ms = max_over_ranks(total_ms, world)
    ms_step = total_ms / args.steps
    value = world * w.n * args.steps / (total_ms * 1e-3)
    final_mode = ["plain_p3m", "learned_closure", "reduced_only"][cl.mode()]
    cl.setMode(cl.LEARNED)
    e2e = e2e_steps(pm, args.steps, judged_step, world, w.n)
    # the configuration's evaluation over 200 steps: the judged run continued to 200 steps
    # after the training positions (t = 50), then the three modes against the direct sum there
    done = 2 * (2 + min(args.steps, 10)) + args.warmup + 2 * args.steps  # mode timings, runs
    fallback200 = fallback
    for s in range(max(0, 200 - done)):
        fb = judged_step(done + s)
        if fb >= 0 and fallback200 < 0:
            fallback200 = done + s
    err200, vs_plain200, judge200 = closure_errors(pm, cl, w)
    after200 = {"steps_after_training_positions": max(200, done), "fallback_step": fallback200,
                "judge_median_rel_diff_learned_vs_plain": judge200,
                "force_err_vs_fp64_direct": err200, "force_diff_vs_plain_p3m": vs_plain200}
    cl.close()
    # roofline of the headline's dominant kernel, the learned step's reduced-cutoff pair pass,
    # and of plain P3M's, the full-cutoff pass: plain P3M handles over the same positions
    rooflines = {}
    for name, cut in (("reduced", 0.5 * q["cutoff"]), ("full", q["cutoff"])):
        p3m = P.P3MMethod(pm, q["comp_box"], cut, q["diameter"], w.H, q["softening"],
                          P.CloudShape(q["cloud_shape"]), bool(q["table"]), bool(q["ysort"]))
        rooflines[name] = pair_roofline(pm, p3m, flush_l2, M.fp32_peak_tflops())
        p3m.close()
    pm.close()
    roofline = {**rooflines["reduced"][0], "pass": "reduced cutoff (1.5 mesh cells): the learned step's pair pass"}
    roofline_full = {**rooflines["full"][0], "pass": "full cutoff (3 mesh cells): plain P3M's pair pass"}
    stage = rooflines["full"][1]
    ms_plain = summary["plain_p3m"]["ms_per_step"]
    closure = {"bound": args.closure_bound, "judge_interval": JUDGE_INTERVAL,
               "judge_stride": JUDGE_STRIDE, "fallback_step": fallback,
               "mode_after_run": final_mode, **summary, "after_200_steps": after200,
               "judged_speedup_vs_plain": ms_plain / ms_step,
               "target_met": bool(summary["learned_closure"]["force_err_vs_fp64_direct"]["median"]
                                  <= args.closure_bound and ms_plain / ms_step >= 2.0)}
    if not args.no_reference_table:  # the same comparison with the reference's table
        wt = W.disk_p3m_1m(table=1)
        pmt, clt, st = closure_setup(args, wt, flush_l2)
        clt.close()
        pmt.close()
        closure["reference_table"] = st
    cpu = cpu_baseline_obj(w, args, rank, world)
    return {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, particlesimulation_gb300/workloads.py)",
            "config": closure_config(w, args.closure_bound), "e2e": e2e, "roofline": roofline,
            "roofline_full_cutoff": roofline_full,
            "stage_ms_plain": {k: round(v, 4) for k, v in stage.items()}, "cpu_baseline": cpu,
            "clocks": clk, "gpu_launches": launches, "closure": closure, "impl": "ours"}


def ensemble_bench(args, rank=0, world=1):
    """64 independent Plummer systems (N log-uniform in [4,096, 131,072], 32^3-128^3 meshes, CIC)
    advanced together for `steps` steps, one launch per stage, one CUDA graph per step; systems
    sharded across ranks (no collective on the data path).  particle-steps/s over all ranks."""
    import numpy as np
    import torch

    from particlesimulation_gb300 import methods, sharding
    from particlesimulation_gb300 import workloads as W

    ws = W.plummer_ensemble()
    costs = [sharding.system_cost(w.n, int(np.prod(w.grid))) for w in ws]
    mine = sharding.shard(costs, world)[rank]
    ens = methods.Ensemble([W.as_system(ws[i]) for i in mine])
    ens.run(0)
    ens.advance(args.warmup)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    ms = ens.advance(ws[0].steps)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    total = sum(w.n for w in ws)
    out = {"workload": f"plummer_ensemble: {len(ws)} systems, {total:,} particles, meshes "
                       f"{sorted(set(w.grid[0] for w in ws))}, CIC, {ws[0].steps} steps",
           "value": total * ws[0].steps / (ms * 1e-3), "unit": UNIT, "ms_per_step": ms / ws[0].steps,
           "systems_per_rank": len(mine), "scaling": "strong", "tuning": ens.tuning(),
           "launches_per_step": 7, "cuda_graph": True}
    ens.close()
    return out


def pm_hbm_bench(args, rank=0, world=1):
    """The PM path where it is HBM-sized: 4,194,304 particles (uniform + Gaussian blobs) in the
    periodic unit cube, 256^3 mesh, CIC, 2-point FD (workloads.blobs_periodic).  The working set
    (~0.7 GB) is larger than L2, so no flush is needed.  Algorithmic bytes per step
    60 N + 26 Ng^3 (particle read/write and the mesh passes of deposit, FFTs and
    interpolation), against the measured HBM copy bandwidth."""
    import torch

    from particlesimulation_gb300 import workloads as W
    w = W.blobs_periodic()
    pm, _ = make_system(w)
    pm.run(0)
    pm.advance(max(args.warmup, 3))
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    steps = 20
    _, _, ms = pm.advance(steps)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())
    pm.pmMethodStep()
    stage = pm.stageTimes()
    forces = pm_force_errors(w, pm) if rank == 0 else None
    pm.close()
    peaks, src = load_peaks()
    ms_step = ms / steps
    byts = 60.0 * w.n + 26.0 * float(w.grid[0] * w.grid[1] * w.grid[2])
    gbs = byts / (ms_step * 1e-3) / 1e9
    return {"workload": f"{w.name}: {w.n:,} particles, periodic {w.grid[0]}^3, CIC, 2-point FD, PM",
            "value": world * w.n / (ms_step * 1e-3), "unit": UNIT, "ms_per_step": ms_step,
            "steps": steps, "roofline": {"bound": "hbm", "achieved": round(gbs, 1),
                                         "peak": peaks.get("hbm_gbs"), "unit": "GB/s",
                                         "frac": round(gbs / peaks.get("hbm_gbs"), 4),
                                         "bytes_per_step": byts, "peak_source": src},
            "stage_ms": {k: round(v, 4) for k, v in stage.items() if k not in ("pair",)},
            "l2": "working set larger than L2", "force_error": forces}


def pm_force_errors(w, pm, targets=4096):
    """Forces of the periodic PM on `targets` sampled particles at the current positions against
    (a) the same PM method in FP64 (the oracle port: deposit, FFT, Green's function, gradient,
    interpolation in double; the parity measure) and (b) an FP64 direct sum with minimum-image
    separations (the Newtonian force of the nearest images only: an approximation of the
    periodic force, so the figure includes the difference between the two)."""
    import numpy as np

    from oracle import oracle as O
    from particlesimulation_gb300 import methods as M
    pos, vel, _ = pm.getParticles(units="original")
    _, _, acc = pm.getParticles(units="code")
    rng = np.random.default_rng(4096)
    idx = np.sort(rng.choice(w.n, targets, replace=False)).astype(np.int32)
    cfg = O.PMConfig(grid=w.grid, box=w.box, H=w.H, DT=w.DT, G=w.G, interpolation=w.interpolation,
                     finite_diff=w.finite_diff, greens=w.greens, diameter=w.diameter,
                     periodic=int(w.periodic))
    t0 = time.perf_counter()
    ref = O.port_pm_accel(cfg, pos, vel, w.mass, prec=1)
    ref = ref[0] if isinstance(ref, tuple) else ref
    t1 = time.perf_counter()
    a_pp = M.direct_sum_fp64(pos, w.mass, w.G, idx, periodic_L=float(w.box[0]))
    t2 = time.perf_counter()
    to_orig = w.H / (w.DT * w.DT)
    return {"targets": targets,
            "vs_fp64_pm": med_err(acc[idx], ref[idx]),
            "vs_fp64_direct_min_image": med_err(acc[idx] * to_orig, a_pp),
            "fp64_pm_seconds": round(t1 - t0, 2), "direct_sum_seconds": round(t2 - t1, 3)}


# The reference's own published timings of its timing scenarios (whole run of
# galaxySimulationPMTiming / galaxySimulationP3MTiming, source/demos.cpp:779-836, 953-1016:
# disk + bulge, 128x128x64, TSC, 101 resp. 26 iterations with diagnostics and StateRecorder
# output), seconds per N, from its timing/pm_time_cpu.txt, timing/pm_time_gpu.txt and
# timing/p3m_time.txt (hardware not stated there).
REF_TIMING = {
    "galaxy-sim-pm-timing": {
        "published_gpu_s": [0.931208, 1.03497, 1.15184, 1.32805, 1.44811, 1.48474, 1.60336, 1.75799, 1.82338],
        "published_cpu_s": [5.54486, 5.76422, 5.96315, 6.15246, 6.3574, 6.58436, 6.89709, 7.05142, 7.10521],
    },
    "galaxy-sim-p3m-timing": {
        "published_cpu_s": [10.8499, 12.9906, 17.6909, 20.7594, 26.9943, 34.7315, 40.1174, 48.9757, 60.7412],
    },
}


def reference_scenarios():
    """The reference's timing scenarios run by the scenario command line on this GPU (same
    samplers, seeds, settings, diagnostics and output files), wall-clock seconds of each run as
    the reference measures them, next to its published seconds."""
    from particlesimulation_gb300 import build as B
    exe = B.build_demos()
    out = {}
    for opt, ref in REF_TIMING.items():
        with tempfile.TemporaryDirectory() as d:
            r = subprocess.run([exe, opt, d], capture_output=True, text=True, timeout=900)
        if r.returncode != 0:
            out[opt] = {"error": r.stderr.strip()[-300:]}
            continue
        rows = [line.split() for line in r.stdout.splitlines() if len(line.split()) == 2
                and line.split()[0].isdigit()]
        ns = [int(a) for a, _ in rows]
        secs = [float(b) for _, b in rows]
        entry = {"n": ns, "seconds": secs, **ref,
                 "published_hardware": "not stated by the reference: not a same-box comparison",
                 "escaped": "outside the computational box" in r.stdout}
        for k, v in ref.items():
            if len(v) == len(secs):
                entry["ratio_to_" + k[:-2]] = [round(a / b, 1) for a, b in zip(v, secs)]
        out[opt] = entry
    return out


def run_reference(args):
    """The reference's CPU P3M step (the oracle port of it, float, every host thread) on the
    ours arm's workload: W warm-up steps, then K timed steps, each a bounded sample (cpu_sample).
    The line's ms_per_step is the wall time a sampled step took; value is particle-steps/s of the
    estimated full step."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from particlesimulation_gb300 import workloads as W
    w = W.WORKLOADS[args.workload]()
    threads = os.cpu_count()
    if args.warmup:
        cpu_sample(w, threads, steps=args.warmup)
    _, est, r = cpu_sample(w, threads, steps=args.steps)  # per-step figures over the K steps
    value = w.n / est
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * float(r["wall"]),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded generator, particlesimulation_gb300/workloads.py)",
            "config": closure_config(w) if w.name == "disk_p3m_1m" else
            {**config_of(w), "l2": "256 MB L2 flush before every timed step"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": sample_text(w), "estimated_full_step_s": est,
                             "breakdown_s": {k: round(float(x), 4) for k, x in r.items()}},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def main():
    args = parse()
    if args.profile_closure:
        run_profile_closure(args)
    elif args.profile_forces:
        run_profile_forces(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
