#!/usr/bin/env python3
"""Benchmark of the GB300 kD-tree Barnes-Hut step.

Workload (one line of JSON on rank 0): the 10,000,000-body ring (body 0: mass 1 at the
origin; bodies 1..N-1: mass 1e-14, r ~ U[0.8, 1.2], phi ~ U[0, 2 pi), z ~ Normal(0, 1e-4),
circular velocities), theta = 0.3, leaf size 7, dt = 1e-3, mixed precision.  A "step" is one
simulation step: tree build, centre-of-mass pass, force walk, kick-drift.

* ``value``: body-steps/s of the mixed path with the bodies resident in HBM (640 MB of
  bodies > 129 MB L2, so no L2 flush is needed between steps).
* ``e2e``: the same metric through the reference-shaped C-ABI call with host buffers: every
  step copies the bodies from pinned host memory (kd_set_bodies), runs one step
  (kd_simple_sim), and copies them back (kd_get_bodies).
* ``fp64``: the plain FP64 path on the same bodies (the reference's arithmetic), and the
  mixed/FP64 speed ratio.
* ``accuracy``: max / RMS relative acceleration error of the mixed walk against an FP64
  direct sum on 4,096 seeded bodies, body 0 (the central mass) among them.
* ``roofline``: the force walk (the dominant kernel) on the algorithmic flops of the
  reference walk (18 per pair, 10 per opening test, 9 per accepted node, counted by the
  oracle's instrumented walk on 20,000 seeded sinks) against the measured FP32 rate;
  ``roofline_build``: the build against measured HBM bandwidth.
* ``adjoint``: forward and reverse sweep over two checkpoint segments (recompute included).
* ``plummer``: the 20,000,000-body Plummer stress case (theta 0.5, dt 1e-4, 20 steps, mixed
  forward + adjoint, rooflines, error on 4,096 samples).
* ``adjoint_check``: the 100,000-body ring gradient check (1,000 steps, checkpoints every 32,
  central differences on 64 coordinates, and the 2,000-body FP64 direct-sum CPU adjoint).
* ``cpu_baseline``: the CPU oracle's step (the reference's algorithm: fork-join PAR4 build,
  parallel walk, all host threads) on sampled steps of the same workload.

``--impl reference`` times the reference's CPU algorithm (the oracle port, all host
threads) on the same workload -- each step the whole build and kick-drift, the walk on a
seeded sample of sinks scaled to all bodies -- and prints the same line with
``"impl": "reference"``.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import tempfile
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "body-steps/s @N=10M mixed vs FP64 plain, accel err<=1e-4; adjoint/forward time"
UNIT = "body-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=10_000_000)
    ap.add_argument("--theta", type=float, default=0.3)
    ap.add_argument("--leaf", type=int, default=7)
    ap.add_argument("--dt", type=float, default=1e-3)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--fp64-steps", type=int, default=2)
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--err-samples", type=int, default=4096)
    ap.add_argument("--cpu-steps", type=int, default=3,
                    help="sampled steps of the cpu_baseline leg")
    ap.add_argument("--ref-sample", type=float, default=0.02,
                    help="fraction of the sinks the CPU walks in each sampled step")
    ap.add_argument("--adjoint-steps", type=int, default=16)
    ap.add_argument("--adjoint-ckpt", type=int, default=8,
                    help="checkpoint interval of the headline adjoint (two segments)")
    ap.add_argument("--flop-sinks", type=int, default=20_000,
                    help="sinks of the oracle walk that counts the algorithmic flops")
    ap.add_argument("--fd-threads", type=int, default=8,
                    help="contexts stepping the finite-difference runs concurrently")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the Plummer and gradient-check blocks of the default line")
    ap.add_argument("--build-n", type=int, default=10_000_000,
                    help="bodies of the build-only measurement (circular_orbits, leaf 8, PAR4)")
    ap.add_argument("--select-n", type=int, default=100_000_000,
                    help="values of the selection measurement (bench_quickstat: 1e8 uniform)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="only the headline timing (used for profiling captures)")
    ap.add_argument("--workload", default="ring", choices=["ring", "plummer", "adjoint-check"],
                    help="ring: the headline line; plummer: the 2e7-body Plummer stress case; "
                         "adjoint-check: the 1e5-body, 1000-step gradient check")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"],
                    help="arithmetic of the headline step (the extras always measure both)")
    ap.add_argument("--adjoint-only", action="store_true",
                    help="only one forward + reverse sweep of --adjoint-steps steps (profiling)")
    return ap.parse_args()


# ------------------------------------------------------------------ distributed (replicas)

def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("nccl")
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(ws, v: float) -> float:
    """The slowest replica's time: every rank gets the maximum."""
    if ws == 1:
        return v
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([v], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def l2_note(n):
    """How the timed steps stand against the 129 MB L2 (64-byte body records)."""
    mb = 64.0 * n / 1e6
    if mb > 129.0:
        return f"inputs ({mb:.0f} MB of bodies, more with the tree) exceed the 129 MB L2; no flush"
    return f"inputs ({mb:.1f} MB of bodies) fit in the 129 MB L2; no flush (small case)"


def replica_value(ws: int, bodies_per_rank: int, steps: int, t_max_s: float) -> float:
    """Whole-job body-steps/s of N independent replicas (weak scaling): every rank advances
    its own bodies, the job's time is the slowest rank's."""
    return ws * bodies_per_rank * steps / t_max_s


# ------------------------------------------------------------------ clocks

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"kd_bench_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.15)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "samples": len(sm),
                "reasons": sorted(reasons)}


# ------------------------------------------------------------------ CPU reference arm

def sampled_cpu_rate(bodies, steps: int, warmup: int, leaf: int, theta: float, dt: float,
                     frac: float, seed: int):
    """The oracle's step (reference algorithm: fork-join PAR4 build, parallel walk, parallel
    kick-drift) on all host threads, `warmup` untimed and `steps` timed sampled steps.  Each
    sampled step builds the whole tree and kick-drifts every body, but walks only a seeded
    `frac` of the sinks; its walk time is scaled by n / sinks.  Returns (body-steps/s,
    threads, timed CPU seconds, per-part seconds of one full step)."""
    from oracle import Oracle
    orc = Oracle()
    b = bodies.copy()
    n = len(b)
    ns = max(1, min(n, int(round(frac * n))))
    rng = np.random.default_rng(seed)
    total, cpu_s, parts = 0.0, 0.0, np.zeros(3)
    for k in range(warmup + steps):
        sinks = np.sort(rng.choice(n, ns, replace=False))
        tb, tw, tk = orc.sampled_step(b, dt, sinks, leaf=leaf, theta=theta, seed=k + 1)
        if k >= warmup:
            full = np.array([tb, tw * n / ns, tk])
            parts += full
            total += full.sum()
            cpu_s += tb + tw + tk
    return n * steps / total, orc.threads(), cpu_s, parts / steps, ns


def run_reference(a, ws, rank):
    if rank != 0:
        return
    import multilanguagekdtree_gb300.array_particle as ap
    bodies = ap.ring(a.n, seed=a.seed)
    rate, threads, cpu_s, parts, ns = sampled_cpu_rate(bodies, a.steps, a.warmup, a.leaf,
                                                       a.theta, a.dt, a.ref_sample, a.seed)
    sample = (f"{a.steps} sampled steps of the {a.n}-body ring ({cpu_s:.1f} s of CPU time): "
              f"whole PAR4 build and kick-drift, walk of {ns} seeded sinks scaled by "
              f"{a.n / ns:.0f}")
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": a.gpus,
        "steps": a.steps, "warmup": a.warmup, "ms_per_step": 1e3 * a.n / rate,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"ring N={a.n} theta={a.theta} leaf={a.leaf} dt={a.dt} "
                               "(reference algorithm: FP64, fork-join median build, "
                               "recursive walk)", "n_bodies": a.n},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": sample},
        "step_parts_s": {"build": parts[0], "walk": parts[1], "kick_drift": parts[2]},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ GPU arm

ROT_Z1 = np.array([[np.cos(1.0), -np.sin(1.0), 0.0], [np.sin(1.0), np.cos(1.0), 0.0],
                   [0.0, 0.0, 1.0]])


def read_peaks():
    try:
        return json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        return {}


def adjoint_timing(kd, bodies, dt, theta, leaf, steps, every, dev):
    """Forward sweep with checkpoints every `every` steps and the reverse sweep of the loss
    mean |x_T - R_z(1 rad) x_0|^2, timed by the library's events.  With steps > every the
    reverse sweep recomputes every segment but the last."""
    n = len(bodies)
    adj = kd.KDTreeSim(n, leaf_size=leaf, layout="dfs", precision="mixed", theta=theta,
                       dt=dt, device=dev)
    adj.set_bodies(bodies)
    adj.simple_sim(dt, 1)
    adj.set_bodies(bodies)
    with adj.forward(dt, steps, every) as tape:
        fwd_ms = adj.stats()["total_ms"]
        xT = adj.get_bodies()["p"]
        tgt = bodies["p"] @ ROT_Z1.T
        tape.backward(2.0 * (xT - tgt) / n)
        bwd_ms = adj.stats()["total_ms"]
    adj.close()
    return {"steps": steps, "ckpt_every": every, "segments": -(-steps // every),
            "forward_ms_per_step": fwd_ms / steps, "backward_ms_per_step": bwd_ms / steps,
            "adjoint_over_forward": bwd_ms / fwd_ms,
            "note": "backward = recompute of every checkpoint segment but the last (whose "
                    "positions the forward keeps) + rebuild + transpose-Jacobian walk per "
                    "step; loss = mean |x_T - R_z(1) x_0|^2"}


def pinned_bodies(n):
    import torch
    from multilanguagekdtree_gb300 import PARTICLE_DTYPE
    t = torch.empty(n * 64, dtype=torch.uint8, pin_memory=True)
    return t, t.numpy().view(PARTICLE_DTYPE)


def reference_walk_flops(state, leaf, theta, sinks):
    """Algorithmic flops per body-step of the reference walk (18 per pair, 10 per opening
    test at an internal node, 9 per accepted node), from the oracle's instrumented walk
    (array_kd_tree.rs:585-617) over a PAR4 tree of the same bodies on seeded sinks."""
    from oracle import Oracle
    orc = Oracle()
    nodes = orc.build_tree_par4(state, leaf=leaf)
    c = orc.walk_counts(state, nodes, sinks, theta)
    k = len(sinks)
    per = {key: c[key] / k for key in ("p2p", "opened", "m2p", "visits")}
    return 18 * per["p2p"] + 10 * per["opened"] + 9 * per["m2p"], per


def grouped_walk_flops(cnt):
    """FP32 work the grouped walk itself does, from its device counts: 18 per interaction
    (pair or accepted node) + 20 per group node test."""
    return 18 * (cnt["p2p"] + cnt["m2p"]) + 20 * cnt["opened"]


def walk_roofline(n, walk_s, alg_per_body, grouped_total, peak, peak_note):
    achieved = alg_per_body * n / walk_s / 1e12
    return {
        "kernel": "k_walk_group", "bound": "fp32", "achieved": achieved, "peak": peak,
        "unit": "TFLOP/s", "frac": achieved / peak,
        "flops_per_body": alg_per_body, "launch_s": walk_s,
        "grouped_set": {"achieved": grouped_total / walk_s / 1e12,
                        "frac": grouped_total / walk_s / 1e12 / peak,
                        "flops_per_body": grouped_total / n},
        "note": "achieved = algorithmic flops of the reference walk (18 per pair, 10 per "
                "opening test, 9 per accepted node; counts from the oracle's instrumented "
                "walk on seeded sinks) x N / device time of the walk phase (CUDA events); "
                "grouped_set = the flops of the grouped walk's own (larger) interaction set; "
                + peak_note}


def build_roofline(n, leaf, build_s, hbm, hbm_src):
    levels = tree_levels(n, leaf)
    build_bytes = n * (40 * levels + 32)
    achieved = build_bytes / build_s / 1e9
    traffic = BUILD_TRAFFIC_PER_BODY * n if BUILD_TRAFFIC_PER_BODY else None
    return {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "traffic": traffic, "launch_s": build_s,
            "note": f"algorithmic bytes N*(40 L + 32), L = {levels} internal levels; traffic "
                    f"= {BUILD_TRAFFIC_NOTE}", "peak_source": hbm_src}


def fp32_peak_tflops(kd, dev):
    try:
        r = kd.fp32_peak(dev)
        return max(r["scalar"], r["packed"]), r
    except Exception as e:  # measured figure unavailable: nominal rate instead, said so
        import torch
        sms = torch.cuda.get_device_properties(dev).multi_processor_count
        return sms * 128 * 2 * 2070e6 / 1e12, {"error": str(e), "nominal_sms": sms}


def run_ours(a, ws, rank, local):
    import torch

    import multilanguagekdtree_gb300 as kd
    dev = local
    torch.cuda.set_device(dev)
    bodies = kd.ring(a.n, seed=a.seed + rank)
    n = a.n

    if a.adjoint_only:
        line = {"metric": METRIC, "config": {"workload": f"adjoint ring N={n}"},
                "adjoint": adjoint_timing(kd, bodies, a.dt, a.theta, a.leaf, a.adjoint_steps,
                                          a.adjoint_ckpt, dev)}
        print(json.dumps(line))
        return

    # ---- headline: mixed precision (or --precision fp64), bodies resident
    sim = kd.KDTreeSim(n, leaf_size=a.leaf, layout="dfs", precision=a.precision,
                       theta=a.theta, dt=a.dt, device=dev)
    sim.set_bodies(bodies)
    sim.simple_sim(a.dt, a.warmup)
    clocks = ClockSampler(dev)
    clocks.start()
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    sim.simple_sim(a.dt, a.steps)
    torch.cuda.synchronize()
    host_s = time.perf_counter() - t0
    barrier(ws)
    clk = clocks.stop()
    st = sim.stats()
    dev_s = st["total_ms"] / 1e3
    launches = int(st["launches"])
    t_max = max_over_ranks(ws, dev_s)
    value = replica_value(ws, n, a.steps, t_max)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": a.steps,
        "warmup": a.warmup, "ms_per_step": 1e3 * t_max / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f32+f64 (mixed)" if a.precision == "mixed" else "f64", "data": "synthetic",
        "config": {"workload": f"ring N={n} theta={a.theta} leaf={a.leaf} dt={a.dt} "
                               f"{a.precision}",
                   "n_bodies": n, "leaf_size": a.leaf, "theta": a.theta, "dt": a.dt,
                   "precision": a.precision, "parallelism": f"replicas x{ws}",
                   "l2": l2_note(n)},
        "gpu_launches": launches, "clocks": clk, "host_wall_s": host_s,
    }
    if a.no_extras or rank != 0:
        if rank == 0:
            print(json.dumps(line))
        return

    peaks = read_peaks()
    hbm = peaks.get("hbm_gbs", 6800.0)
    hbm_src = "MEASURED_PEAKS.json" if "hbm_gbs" in peaks else "fallback 6800 GB/s"
    fp32, fp32_detail = fp32_peak_tflops(kd, dev)
    peak_note = ("peak = the larger of the measured scalar and packed (f32x2) FP32 "
                 "multiply-add rates (kd_fp32_peak: every SM, a few ms)")

    # ---- per-phase device times (events around every phase) and interaction counts
    sim.set_bodies(bodies)
    sim.set_timing(True)
    sim.simple_sim(a.dt, 2)
    ph = sim.stats()
    sim.set_timing(False)
    sim.set_bodies(bodies)
    sim.build_tree()
    sim.set_counting(True)
    sim.calc_accel()
    cnt = sim.counts()
    sim.set_precision("fp64")  # the reference walk itself, every body, counted on the device
    sim.calc_accel()
    cnt64 = sim.counts()
    sim.set_precision("mixed")
    sim.set_counting(False)
    rng = np.random.default_rng(a.seed + 101)
    flop_sinks = np.sort(rng.choice(n, min(n, a.flop_sinks), replace=False))
    alg, per = reference_walk_flops(bodies, a.leaf, a.theta, flop_sinks)
    walk_s = ph["walk_ms"] / 2 / 1e3
    line["phases_ms_per_step"] = {k: ph[k] / 2 for k in ("build_ms", "moments_ms", "walk_ms",
                                                         "kick_ms")}
    line["interactions_per_body"] = {
        "grouped_walk": {k: v / n for k, v in cnt.items()},
        "reference_walk_oracle": dict(per, sinks=len(flop_sinks)),
        "reference_walk_device_fp64": {k: v / n for k, v in cnt64.items()}}
    line["roofline"] = walk_roofline(n, walk_s, alg, grouped_walk_flops(cnt), fp32, peak_note)
    line["roofline"]["traffic"] = WALK_TRAFFIC_PER_BODY * n
    line["roofline"]["traffic_unit"] = ("bytes per launch (ncu dram read + write of the 10M "
                                        "ring walk, scaled by N)")
    line["fp32_peak_tflops"] = fp32_detail
    line["roofline_build"] = build_roofline(n, a.leaf, ph["build_ms"] / 2 / 1e3, hbm, hbm_src)

    # ---- energy drift over the timed run length
    sim.set_bodies(bodies)
    e0 = sim.energy()
    sim.simple_sim(a.dt, a.steps)
    e1 = sim.energy()
    line["energy"] = {"steps": a.steps, "start": e0, "end": e1,
                      "relative_drift": (sum(e1) - sum(e0)) / abs(sum(e0)),
                      "potential": "mixed tree walk (theta as above), FP64 heavy-body terms"}

    # ---- accuracy of the mixed walk against the FP64 direct sum, body 0 included
    rng = np.random.default_rng(12345)
    sinks = np.sort(np.concatenate([[0], rng.choice(np.arange(1, n), a.err_samples - 1,
                                                    replace=False)]))
    sim.set_bodies(bodies)
    sim.build_tree()
    macc = sim.calc_accel()
    direct = sim.direct_accel(sinks)
    sim.set_precision("fp64")
    facc = sim.calc_accel()
    sim.set_precision("mixed")
    e_mixed = rel_rows(macc[sinks], direct)
    e_fp64 = rel_rows(facc[sinks], direct)
    line["accuracy"] = {
        "samples": int(len(sinks)), "reference": "FP64 direct sum (GPU kernel, all N)",
        "mixed_max_rel": float(e_mixed.max()),
        "mixed_rms_rel": float(np.sqrt(np.mean(e_mixed ** 2))),
        "fp64_tree_max_rel": float(e_fp64[1:].max()),
        "body0_mixed_rel": float(e_mixed[0]), "body0_fp64_tree_rel": float(e_fp64[0]),
        "note": "body 0 (the central mass) is among the samples; the mixed path takes its "
                "acceleration as an FP64 direct sum, the FP64 tree keeps the reference's "
                "theta truncation of its cancelling sum (excluded from fp64_tree_max_rel)"}
    sim.close()

    # ---- FP64 plain path, same bodies
    f64 = kd.KDTreeSim(n, leaf_size=a.leaf, layout="dfs", precision="fp64", theta=a.theta,
                       dt=a.dt, device=dev)
    f64.set_bodies(bodies)
    f64.simple_sim(a.dt, 1)
    torch.cuda.synchronize()
    f64.simple_sim(a.dt, a.fp64_steps)
    fst = f64.stats()
    fp64_rate = n * a.fp64_steps / (fst["total_ms"] / 1e3)
    line["fp64"] = {"value": fp64_rate, "unit": UNIT, "steps": a.fp64_steps,
                    "ms_per_step": fst["total_ms"] / a.fp64_steps}
    line["mixed_over_fp64"] = value / ws / fp64_rate
    f64.close()

    # ---- adjoint: two checkpoint segments, so the reverse sweep includes a recompute
    line["adjoint"] = adjoint_timing(kd, bodies, a.dt, a.theta, a.leaf, a.adjoint_steps,
                                     a.adjoint_ckpt, dev)

    # ---- build only: the reference's bench_build_tree input (circular_orbits, leaf 8, PAR4)
    cb = kd.circular_orbits(a.build_n - 1, seed=a.seed)
    bo = kd.KDTreeSim(len(cb), leaf_size=8, layout="par4", precision="fp64", device=dev)
    bo.set_bodies(cb)
    bo.build_tree()
    times = []
    for _ in range(3):
        bo.build_tree()
        times.append(bo.stats()["build_ms"])
    bo.close()
    line["build_only"] = {"n_bodies": len(cb), "input": "circular_orbits, leaf 8, PAR4 numbering",
                          "gpu_ms": min(times), "note": "tree + FP64 moments + walk records"}

    # ---- selection only: the reference's bench_quickstat input (1e8 uniform doubles)
    rng = np.random.default_rng(a.seed)
    sv = rng.random(a.select_n)
    goal = int(rng.integers(0, a.select_n))
    kd.quickstat_index(sv[:1000], 10)  # load / warm the path
    t0 = time.perf_counter()
    sidx, sel_ms = kd.quickstat_index(sv, goal, timing=True)
    sel_e2e = time.perf_counter() - t0
    line["select_only"] = {"n": a.select_n, "input": "uniform [0,1) doubles, random goal",
                           "gpu_ms": sel_ms, "e2e_ms": 1e3 * sel_e2e,
                           "note": "device time of select + partition; e2e adds the host "
                                   "transfers of values and indices"}
    del sidx

    # ---- end to end through the C ABI with host buffers
    keep, host = pinned_bodies(n)
    host[:] = bodies
    e2e = kd.KDTreeSim(n, leaf_size=a.leaf, layout="dfs", precision="mixed", theta=a.theta,
                       dt=a.dt, device=dev)
    e2e.set_bodies(host)
    e2e.simple_sim(a.dt, 1)
    e2e.get_bodies(out=host)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(a.e2e_steps):
        e2e.set_bodies(host)
        e2e.simple_sim(a.dt, 1)
        e2e.get_bodies(out=host)
    e2e_s = time.perf_counter() - t0
    e2e.close()
    line["e2e"] = {"value": n * a.e2e_steps / e2e_s, "unit": UNIT,
                   "h2d_bytes_per_step": 64 * n, "d2h_bytes_per_step": 64 * n,
                   "steps": a.e2e_steps,
                   "call": "kd_set_bodies(pinned host) + kd_simple_sim(1) + kd_get_bodies"}
    del keep

    # ---- the Plummer stress case and the gradient check (the other GPU configurations)
    if not a.no_configs:
        line["plummer"] = plummer_block(kd, a, dev, fp32, peak_note, hbm, hbm_src)
        line["adjoint_check"] = adjoint_check_block(kd, a, dev)

    # ---- CPU baseline (oracle port of the reference algorithm)
    if not a.no_cpu_baseline:
        from oracle import Oracle
        orc = Oracle()
        t0 = time.perf_counter()
        orc.build_tree_par4(cb, leaf=8)
        line["build_only"]["cpu_ms"] = 1e3 * (time.perf_counter() - t0)
        line["build_only"]["cpu_threads"] = orc.threads()
        t0 = time.perf_counter()
        orc.quickstat_index(sv, goal)
        line["select_only"]["cpu_ms"] = 1e3 * (time.perf_counter() - t0)
        line["select_only"]["cpu_kind"] = "oracle quickstat_index (sequential, as quickstat.rs)"
        rate, threads, cpu_s, parts, ns = sampled_cpu_rate(bodies, a.cpu_steps, 1, a.leaf,
                                                           a.theta, a.dt, a.ref_sample,
                                                           a.seed)
        line["cpu_baseline"] = {
            "value": rate, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{a.cpu_steps} sampled FP64 steps of the {n}-body ring ({cpu_s:.1f} s "
                      f"of CPU time): whole PAR4 build and kick-drift, walk of {ns} seeded "
                      f"sinks scaled by {n / ns:.0f}",
            "step_parts_s": {"build": parts[0], "walk": parts[1], "kick_drift": parts[2]}}
    print(json.dumps(line))


# DRAM bytes per body of one launch, from one-pass ncu captures of the 10M-body step (the
# launch list in profiles/): the grouped walk (4.79 GB), and the build's kernels summed over
# the step (10.94 GB, every kernel starting with cold caches), both scaled by the number of
# bodies
WALK_TRAFFIC_PER_BODY = 479.0
BUILD_TRAFFIC_PER_BODY = 1094.0
BUILD_TRAFFIC_NOTE = ("ncu dram read + write of the build's kernels in one 10M-ring step "
                      "(1,094 B/body, cold caches per kernel), scaled by N; captured while the "
                      "first pass still copied the positions (~23 B/body more than now)")


def tree_levels(n: int, leaf: int) -> int:
    """Internal levels of the median-split tree of n bodies (halvings until <= leaf)."""
    levels, c = 0, n
    while c > leaf:
        c = c - c // 2
        levels += 1
    return levels


def rel_rows(x, y):
    return np.linalg.norm(x - y, axis=1) / np.linalg.norm(y, axis=1)


def plummer_block(kd, a, dev, fp32, peak_note, hbm, hbm_src, n=20_000_000):
    """Clustered stress case: Plummer sphere (G = M = a = 1, equal masses, radii <= 20),
    theta 0.5, leaf 7, dt 1e-4, 20 mixed-precision steps, then a reverse sweep over the same
    20 steps in checkpoint segments of 8; error of the mixed walk against the FP64 direct sum
    on 4,096 bodies; walk and build rooflines."""
    import torch
    theta, dt, steps, every = 0.5, 1e-4, 20, 8
    s = kd.KDTreeSim(n, leaf_size=a.leaf, precision="mixed", theta=theta, dt=dt, device=dev)
    s.generate("plummer", a.seed)
    e0 = s.energy()
    s.simple_sim(dt, 1)
    s.generate("plummer", a.seed)
    clocks = ClockSampler(dev)
    clocks.start()
    torch.cuda.synchronize()
    s.simple_sim(dt, steps)
    torch.cuda.synchronize()
    clk = clocks.stop()
    fwd = s.stats()
    e1 = s.energy()
    out = {"workload": f"plummer N={n} theta={theta} leaf={a.leaf} dt={dt} mixed",
           "steps": steps, "value": n * steps / (fwd["total_ms"] / 1e3), "unit": UNIT,
           "ms_per_step": fwd["total_ms"] / steps,
           "energy": {"start": e0, "end": e1,
                      "relative_drift": (sum(e1) - sum(e0)) / abs(sum(e0))},
           "gpu_launches": int(fwd["launches"]), "clocks": clk}
    s.generate("plummer", a.seed)
    state = s.get_bodies().copy()
    s.set_timing(True)
    s.simple_sim(dt, 2)
    ph = s.stats()
    s.set_timing(False)
    out["phases_ms_per_step"] = {k: ph[k] / 2 for k in ("build_ms", "walk_ms", "kick_ms")}
    s.set_bodies(state)
    s.build_tree()
    s.set_counting(True)
    acc = s.calc_accel()
    cnt = s.counts()
    s.set_counting(False)
    rng = np.random.default_rng(a.seed + 202)
    flop_sinks = np.sort(rng.choice(n, a.flop_sinks, replace=False))
    alg, per = reference_walk_flops(state, a.leaf, theta, flop_sinks)
    out["interactions_per_body"] = {"grouped_walk": {k: v / n for k, v in cnt.items()},
                                    "reference_walk_oracle": dict(per, sinks=len(flop_sinks))}
    out["roofline_walk"] = walk_roofline(n, ph["walk_ms"] / 2 / 1e3, alg,
                                         grouped_walk_flops(cnt), fp32, peak_note)
    out["roofline_build"] = build_roofline(n, a.leaf, ph["build_ms"] / 2 / 1e3, hbm, hbm_src)
    rng = np.random.default_rng(12345)
    sinks = np.sort(rng.choice(n, a.err_samples, replace=False))
    ref = s.direct_accel(sinks)
    e = rel_rows(acc[sinks], ref)
    out["accuracy"] = {"samples": int(a.err_samples), "reference": "FP64 direct sum",
                       "mixed_max_rel": float(e.max()),
                       "mixed_rms_rel": float(np.sqrt(np.mean(e ** 2))),
                       "mixed_median_rel": float(np.median(e)),
                       "note": "theta = 0.5 truncation dominates (the FP64 tree has the same)"}
    s.set_bodies(state)
    with s.forward(dt, steps, every) as tape:
        f_ms = s.stats()["total_ms"]
        xT = s.get_bodies()["p"]
        tape.backward(np.zeros_like(xT), np.ones_like(xT) / n)
        b_ms = s.stats()["total_ms"]
    out["adjoint"] = {"steps": steps, "ckpt_every": every, "segments": -(-steps // every),
                      "forward_ms": f_ms, "backward_ms": b_ms, "adjoint_over_forward": b_ms / f_ms,
                      "loss": "sum of final velocities / n (dL/dv_T = 1/n)"}
    s.close()
    return out


def adjoint_check_block(kd, a, dev, n=100_000):
    """Gradient check: 100,000-body ring, theta 0.3, dt 1e-3, 1,000 steps, checkpoints every
    32 steps, loss = mean |x_T - R_z(1 rad) x_0|^2.  dL/dv0 from the reverse sweep against
    central differences (h = 1e-6) of the forward on 64 seeded coordinates (the forward runs
    of the differences step concurrently, one context per thread); and the 2,000-body,
    1,000-step sweep against the oracle's FP64 direct-sum adjoint."""
    from concurrent.futures import ThreadPoolExecutor
    steps, dt, h, every = 1000, 1e-3, 1e-6, 32

    def sweep(bodies):
        m = len(bodies)
        tgt = bodies["p"] @ ROT_Z1.T
        with kd.KDTreeSim(m, leaf_size=a.leaf, precision="mixed", theta=a.theta,
                          device=dev) as s:
            s.set_bodies(bodies)
            s.simple_sim(dt, 1)
            s.set_bodies(bodies)
            with s.forward(dt, steps, every) as tape:
                fms = s.stats()["total_ms"]
                xT = s.get_bodies()["p"]
                gx, gv = tape.backward(2.0 * (xT - tgt) / m)
                bms = s.stats()["total_ms"]
        return gx, gv, fms, bms, tgt

    t0 = time.perf_counter()
    b = kd.ring(n, seed=a.seed)
    gx, gv, fms, bms, tgt = sweep(b)
    rng = np.random.default_rng(77)
    coords = list(zip(rng.choice(np.arange(1, n), 64, replace=False).tolist(),
                      rng.integers(0, 2, 64).tolist()))

    def fd_share(share):
        import torch
        torch.cuda.set_device(dev)
        res = []
        with kd.KDTreeSim(n, leaf_size=a.leaf, precision="mixed", theta=a.theta,
                          device=dev) as s:
            def final(bb):
                s.set_bodies(bb)
                s.simple_sim(dt, steps)
                return s.get_bodies()["p"].copy()
            for i, d in share:
                bp = b.copy(); bp["v"][i, d] += h
                bm = b.copy(); bm["v"][i, d] -= h
                lp = np.sum((final(bp) - tgt) ** 2, axis=1)
                lm = np.sum((final(bm) - tgt) ** 2, axis=1)
                fd = np.sum(lp - lm) / n / (2 * h)
                res.append(abs(fd - gv[i, d]) / abs(gv[i, d]))
        return res

    k = max(1, a.fd_threads)
    with ThreadPoolExecutor(k) as ex:
        errs = [e for part in ex.map(fd_share, [coords[j::k] for j in range(k)]) for e in part]
    fd_s = time.perf_counter() - t0
    # the 2,000-body sweep against the FP64 direct-sum CPU adjoint
    from oracle import Oracle
    small = kd.ring(2000, seed=a.seed + 5)
    sgx, sgv, _, _, stgt = sweep(small)
    ref = Oracle().adjoint_direct(small, dt, steps, target=stgt)
    ev = rel_rows(sgv, ref["g_v0"])
    ex_ = rel_rows(sgx, ref["g_x0"])
    return {"workload": f"ring N={n} theta={a.theta} dt={dt} steps={steps} ckpt={every}",
            "forward_ms": fms, "backward_ms": bms, "adjoint_over_forward": bms / fms,
            "fd": {"coords": 64, "h": h, "max_rel_err": float(max(errs)),
                   "median_rel_err": float(np.median(errs)), "wall_s": fd_s},
            "cpu_direct_adjoint": {"n": 2000, "steps": steps,
                                   "dL_dv0_max_rel_err": float(ev.max()),
                                   "dL_dv0_median_rel_err": float(np.median(ev)),
                                   "dL_dx0_max_rel_err": float(ex_.max())}}


def run_plummer(a, dev):
    import multilanguagekdtree_gb300 as kd
    fp32, _ = fp32_peak_tflops(kd, dev)
    peaks = read_peaks()
    line = plummer_block(kd, a, dev, fp32, "peak = measured FP32 multiply-add rate",
                         peaks.get("hbm_gbs", 6800.0),
                         "MEASURED_PEAKS.json" if "hbm_gbs" in peaks else "fallback 6800 GB/s",
                         n=a.n if a.n != 10_000_000 else 20_000_000)
    print(json.dumps(line))


def run_adjoint_check(a, dev):
    import multilanguagekdtree_gb300 as kd
    print(json.dumps(adjoint_check_block(kd, a, dev,
                                         n=a.n if a.n != 10_000_000 else 100_000)))


def main():
    a = parse()
    ws, rank, local = dist_setup()
    if a.impl == "reference":
        run_reference(a, ws, rank)
    elif a.workload == "plummer":
        run_plummer(a, local)
    elif a.workload == "adjoint-check":
        run_adjoint_check(a, local)
    else:
        run_ours(a, ws, rank, local)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
