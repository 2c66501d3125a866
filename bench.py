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
  direct sum on 4,096 seeded bodies (body 0, whose acceleration is a near-cancelling
  residual, is reported separately).
* ``roofline``: the force walk (the dominant kernel) against the FP32 rate of the GPU;
  ``roofline_build``: the build against measured HBM bandwidth.
* ``cpu_baseline``: the CPU oracle's step loop (the reference's algorithm, OpenMP,
  fork-join build) on one step of the same workload.

``--impl reference`` times the reference's CPU algorithm (the oracle port, all host
threads) on the same workload and prints the same line with ``"impl": "reference"``.
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
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--adjoint-steps", type=int, default=4)
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

def cpu_step_rate(bodies, steps: int, leaf: int, theta: float, dt: float):
    """The oracle's step loop (reference algorithm: fork-join PAR4 build, parallel walk)
    on all host threads.  Returns (body-steps/s, threads, seconds)."""
    from oracle import Oracle
    orc = Oracle()
    threads = orc.threads()
    b = bodies.copy()
    t0 = time.perf_counter()
    orc.simple_sim(b, dt, steps, leaf=leaf, layout="par4", theta=theta)
    t = time.perf_counter() - t0
    return len(b) * steps / t, threads, t


def run_reference(a, ws, rank):
    if rank != 0:
        return
    import multilanguagekdtree_gb300.array_particle as ap
    bodies = ap.ring(a.n, seed=a.seed)
    # one untimed step warms caches and page tables; each timed step is one full step of
    # the same 10M-body workload, capped so the run stays within a few minutes
    rate_w, threads, tw = cpu_step_rate(bodies, 1, a.leaf, a.theta, a.dt)
    steps = max(1, min(a.steps, int(150.0 / max(tw, 1e-3))))
    rate, threads, t = cpu_step_rate(bodies, steps, a.leaf, a.theta, a.dt)
    line = {
        "impl": "reference", "metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": a.gpus,
        "steps": steps, "warmup": 1, "ms_per_step": 1e3 * t / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"ring N={a.n} theta={a.theta} leaf={a.leaf} dt={a.dt} "
                               "(reference algorithm: FP64, fork-join median build, "
                               "recursive walk)", "n_bodies": a.n},
        "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} full step(s) of the {a.n}-body ring"},
        "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ------------------------------------------------------------------ GPU arm

def adjoint_timing(kd, bodies, a, dev):
    """Forward sweep with checkpoints (every 32 steps) and the reverse sweep of the loss
    mean |x_T - R_z(1 rad) x_0|^2, timed by the library's events."""
    n = len(bodies)
    adj = kd.KDTreeSim(n, leaf_size=a.leaf, layout="dfs", precision="mixed", theta=a.theta,
                       dt=a.dt, device=dev)
    adj.set_bodies(bodies)
    adj.simple_sim(a.dt, 1)
    adj.set_bodies(bodies)
    with adj.forward(a.dt, a.adjoint_steps, 32) as tape:
        fwd_ms = adj.stats()["total_ms"]
        xT = adj.get_bodies()["p"]
        tgt = bodies["p"] @ np.array([[np.cos(1.0), -np.sin(1.0), 0.0],
                                      [np.sin(1.0), np.cos(1.0), 0.0], [0.0, 0.0, 1.0]]).T
        tape.backward(2.0 * (xT - tgt) / n)
        bwd_ms = adj.stats()["total_ms"]
    adj.close()
    return {"steps": a.adjoint_steps, "forward_ms_per_step": fwd_ms / a.adjoint_steps,
            "backward_ms_per_step": bwd_ms / a.adjoint_steps,
            "adjoint_over_forward": bwd_ms / fwd_ms,
            "note": "backward = recompute of each checkpoint segment but the last (whose "
                    "positions the forward keeps) + rebuild + transpose-Jacobian walk per "
                    "step; loss = mean |x_T - R_z(1) x_0|^2"}


def pinned_bodies(n):
    import torch
    from multilanguagekdtree_gb300 import PARTICLE_DTYPE
    t = torch.empty(n * 64, dtype=torch.uint8, pin_memory=True)
    return t, t.numpy().view(PARTICLE_DTYPE)


def run_ours(a, ws, rank, local):
    import torch

    import multilanguagekdtree_gb300 as kd
    dev = local
    torch.cuda.set_device(dev)
    bodies = kd.ring(a.n, seed=a.seed + rank)
    n = a.n

    if a.adjoint_only:
        line = {"metric": METRIC, "config": {"workload": f"adjoint ring N={n}"},
                "adjoint": adjoint_timing(kd, bodies, a, dev)}
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
    sim.set_counting(False)
    flops = walk_flops(cnt)
    walk_s = ph["walk_ms"] / 2 / 1e3
    sm_mhz = clk.get("sm_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s at the sampled clock
    achieved = flops / walk_s / 1e12
    line["phases_ms_per_step"] = {k: ph[k] / 2 for k in ("build_ms", "moments_ms", "walk_ms",
                                                         "kick_ms")}
    line["interactions_per_body"] = {k: v / n for k, v in cnt.items()}
    # DRAM bytes per launch: one-pass ncu capture of the 10M-body walk (4.31 GB read +
    # 0.475 GB written, 479 B per body), scaled by the number of bodies
    walk_traffic = 479.0 * n
    line["roofline"] = {
        "kernel": "k_walk_group", "bound": "fp32", "achieved": achieved, "peak": fp32_peak,
        "unit": "TFLOP/s", "frac": achieved / fp32_peak, "traffic": walk_traffic,
        "traffic_unit": "bytes per launch (ncu dram read + write of the 10M ring walk, scaled "
                        "by N)",
        "note": WALK_FLOPS_NOTE}
    # build: algorithmic bytes per build = N*(40 L + 32), L = internal levels of the tree
    # (each level reads x, y, z for the box, the split key and the index; a final gather of
    # the leaves)
    peaks = {}
    try:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text())
    except (OSError, ValueError):
        pass
    hbm = peaks.get("hbm_gbs", 6800.0)
    levels = tree_levels(n, a.leaf)
    build_bytes = n * (40 * levels + 32)
    build_s = ph["build_ms"] / 2 / 1e3
    line["roofline_build"] = {
        "bound": "hbm", "achieved": build_bytes / build_s / 1e9, "peak": hbm, "unit": "GB/s",
        "frac": build_bytes / build_s / 1e9 / hbm, "traffic": None,
        "note": f"algorithmic bytes N*(40 L + 32), L = {levels} internal levels",
        "peak_source": "MEASURED_PEAKS.json" if "hbm_gbs" in peaks else "fallback 6800 GB/s"}

    # ---- energy drift over the timed run length
    sim.set_bodies(bodies)
    e0 = sim.energy()
    sim.simple_sim(a.dt, a.steps)
    e1 = sim.energy()
    line["energy"] = {"steps": a.steps, "start": e0, "end": e1,
                      "relative_drift": (sum(e1) - sum(e0)) / abs(sum(e0)),
                      "potential": "mixed tree walk (theta as above), FP64 central-mass term"}

    # ---- accuracy of the mixed walk against the FP64 direct sum
    rng = np.random.default_rng(12345)
    sinks = np.sort(rng.choice(np.arange(1, n), a.err_samples, replace=False))
    sim.set_bodies(bodies)
    sim.build_tree()
    macc = sim.calc_accel()
    direct = sim.direct_accel(np.concatenate([[0], sinks]))
    sim.set_precision("fp64")
    facc = sim.calc_accel()
    sim.set_precision("mixed")

    def rel(x, y):
        return np.linalg.norm(x - y, axis=1) / np.linalg.norm(y, axis=1)

    e_mixed = rel(macc[sinks], direct[1:])
    e_fp64 = rel(facc[sinks], direct[1:])
    e_mix_vs_fp64 = rel(macc[sinks], facc[sinks])
    line["accuracy"] = {
        "samples": int(a.err_samples), "reference": "FP64 direct sum (GPU kernel, all N)",
        "mixed_max_rel": float(e_mixed.max()), "mixed_rms_rel": float(np.sqrt(np.mean(e_mixed ** 2))),
        "fp64_tree_max_rel": float(e_fp64.max()),
        "mixed_vs_fp64_tree_max_rel": float(e_mix_vs_fp64.max()),
        "body0_mixed_rel": float(rel(macc[:1], direct[:1])[0]),
        "body0_fp64_tree_rel": float(rel(facc[:1], direct[:1])[0]),
    }
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

    # ---- adjoint: forward sweep with checkpoints, then the reverse sweep, same bodies
    line["adjoint"] = adjoint_timing(kd, bodies, a, dev)

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
        rate, threads, t = cpu_step_rate(bodies, a.cpu_steps, a.leaf, a.theta, a.dt)
        line["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                                "sample": f"{a.cpu_steps} full FP64 step(s) of the {n}-body "
                                          f"ring ({t:.1f} s)"}
    print(json.dumps(line))


WALK_FLOPS_NOTE = ("walk flops = 18 per body interaction (P2P or accepted node, the "
                   "reference's pair count) + 20 per group node test, counted on the device; "
                   "peak = 152 SMs x 128 FP32 lanes x 2 x sampled SM clock (nominal rate; no "
                   "measured FP32 figure exists)")


def tree_levels(n: int, leaf: int) -> int:
    """Internal levels of the median-split tree of n bodies (halvings until <= leaf)."""
    levels, c = 0, n
    while c > leaf:
        c = c - c // 2
        levels += 1
    return levels


def walk_flops(cnt):
    """Algorithmic FP32 work of one grouped walk from its device counts."""
    return 18 * (cnt["p2p"] + cnt["m2p"]) + 20 * cnt["opened"]


def rel_rows(x, y):
    return np.linalg.norm(x - y, axis=1) / np.linalg.norm(y, axis=1)


def run_plummer(a, dev):
    """Clustered stress case: Plummer sphere (G = M = a = 1, equal masses, radii <= 20),
    theta 0.5, leaf 7, dt 1e-4, 20 mixed-precision steps, then a reverse sweep over the same
    20 steps; error of the mixed walk against the FP64 direct sum on 4,096 bodies."""
    import torch

    import multilanguagekdtree_gb300 as kd
    n = a.n if a.n != 10_000_000 else 20_000_000
    theta, dt, steps = 0.5, 1e-4, 20
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
    line = {"workload": f"plummer N={n} theta={theta} leaf={a.leaf} dt={dt} mixed",
            "steps": steps, "value": n * steps / (fwd["total_ms"] / 1e3), "unit": UNIT,
            "ms_per_step": fwd["total_ms"] / steps,
            "energy": {"start": e0, "end": e1,
                       "relative_drift": (sum(e1) - sum(e0)) / abs(sum(e0))},
            "gpu_launches": int(fwd["launches"]), "clocks": clk}
    s.set_timing(True)
    s.simple_sim(dt, 2)
    ph = s.stats()
    s.set_timing(False)
    line["phases_ms_per_step"] = {k: ph[k] / 2 for k in ("build_ms", "walk_ms", "kick_ms")}
    s.build_tree()
    s.set_counting(True)
    s.calc_accel()
    cnt = s.counts()
    s.set_counting(False)
    flops = walk_flops(cnt)
    peak = 152 * 128 * 2 * (clk.get("sm_mhz") or 2070.0) * 1e6 / 1e12
    walk_s = ph["walk_ms"] / 2 / 1e3
    line["interactions_per_body"] = {k: v / n for k, v in cnt.items()}
    line["roofline_walk"] = {"bound": "fp32", "achieved": flops / walk_s / 1e12, "peak": peak,
                             "unit": "TFLOP/s", "frac": flops / walk_s / 1e12 / peak}
    try:
        hbm = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()).get("hbm_gbs", 6800.0)
    except (OSError, ValueError):
        hbm = 6800.0
    levels = tree_levels(n, a.leaf)
    bb = n * (40 * levels + 32) / (ph["build_ms"] / 2 / 1e3) / 1e9
    line["roofline_build"] = {"bound": "hbm", "achieved": bb, "peak": hbm, "unit": "GB/s",
                              "frac": bb / hbm}
    rng = np.random.default_rng(12345)
    sinks = np.sort(rng.choice(n, a.err_samples, replace=False))
    acc = s.calc_accel()
    ref = s.direct_accel(sinks)
    e = rel_rows(acc[sinks], ref)
    line["accuracy"] = {"samples": int(a.err_samples), "reference": "FP64 direct sum",
                        "mixed_max_rel": float(e.max()),
                        "mixed_rms_rel": float(np.sqrt(np.mean(e ** 2))),
                        "mixed_median_rel": float(np.median(e))}
    s.generate("plummer", a.seed)
    with s.forward(dt, steps, 32) as tape:
        f_ms = s.stats()["total_ms"]
        xT = s.get_bodies()["p"]
        tape.backward(np.zeros_like(xT), np.ones_like(xT) / n)
        b_ms = s.stats()["total_ms"]
    line["adjoint"] = {"steps": steps, "forward_ms": f_ms, "backward_ms": b_ms,
                       "adjoint_over_forward": b_ms / f_ms,
                       "loss": "sum of final velocities / n (dL/dv_T = 1/n)"}
    s.close()
    print(json.dumps(line))


def run_adjoint_check(a, dev):
    """Gradient check: 100,000-body ring, theta 0.3, dt 1e-3, 1,000 steps, checkpoints every
    32 steps, loss = mean |x_T - R_z(1 rad) x_0|^2.  dL/dv0 from the reverse sweep against
    central differences (h = 1e-6) of the forward on 64 seeded coordinates."""
    import multilanguagekdtree_gb300 as kd
    n = a.n if a.n != 10_000_000 else 100_000
    steps, dt, h = 1000, 1e-3, 1e-6
    R = np.array([[np.cos(1.0), -np.sin(1.0), 0.0], [np.sin(1.0), np.cos(1.0), 0.0],
                  [0.0, 0.0, 1.0]])

    def grad(bodies):
        m = len(bodies)
        tgt = bodies["p"] @ R.T
        with kd.KDTreeSim(m, leaf_size=a.leaf, precision="mixed", theta=a.theta,
                          device=dev) as s:
            s.set_bodies(bodies)
            with s.forward(dt, steps, 32) as tape:
                fms = s.stats()["total_ms"]
                xT = s.get_bodies()["p"]
                gx, gv = tape.backward(2.0 * (xT - tgt) / m)
                bms = s.stats()["total_ms"]
        return gx, gv, fms, bms, tgt

    b = kd.ring(n, seed=a.seed)
    gx, gv, fms, bms, tgt = grad(b)
    rng = np.random.default_rng(77)
    coords = list(zip(rng.choice(np.arange(1, n), 64, replace=False).tolist(),
                      rng.integers(0, 2, 64).tolist()))
    errs = []
    with kd.KDTreeSim(n, leaf_size=a.leaf, precision="mixed", theta=a.theta, device=dev) as s:
        def final(bb):
            s.set_bodies(bb)
            s.simple_sim(dt, steps)
            return s.get_bodies()["p"].copy()
        for i, d in coords:
            bp = b.copy(); bp["v"][i, d] += h
            bm = b.copy(); bm["v"][i, d] -= h
            lp = np.sum((final(bp) - tgt) ** 2, axis=1)
            lm = np.sum((final(bm) - tgt) ** 2, axis=1)
            fd = np.sum(lp - lm) / n / (2 * h)
            errs.append(abs(fd - gv[i, d]) / abs(gv[i, d]))
    line = {"workload": f"adjoint-check ring N={n} theta={a.theta} dt={dt} steps={steps} ckpt=32",
            "forward_ms": fms, "backward_ms": bms, "adjoint_over_forward": bms / fms,
            "fd": {"coords": 64, "h": h, "max_rel_err": float(max(errs)),
                   "median_rel_err": float(np.median(errs))},
            "cpu_direct_adjoint": "2,000-body, 1,000-step comparison with the FP64 direct-sum "
                                  "adjoint: tests/test_gpu_adjoint.py"}
    print(json.dumps(line))


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
