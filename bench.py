#!/usr/bin/env python3
"""Benchmark of the GB300 midpoint Lennard-Jones path (one JSON line on stdout).

Workload: 1,048,576 atoms (FCC 64^3 x 4) at rho* = 0.8442, melted at T* = 1.0,
LJ eps = sigma = m = 1, rc = 2.5 sigma truncated and unshifted, dt = 0.005,
velocity-Verlet with re-binning every step.  A step = one velocity-Verlet step
over all atoms (kick + drift + wrap + binning + midpoint pair forces).
Synthetic, seeded inputs; no dataset is involved.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl examd|reference]

value: atom-steps/s of the mixed form with all state resident in HBM, device
time (CUDA events on the library's stream), max over ranks.  e2e: the same
metric through the drop-in force call with host buffers (pinned positions in,
forces out, every step).  --impl reference times the CPU restatement of the
reference's force routine (oracle/) with all host threads on the same
workload.  With N > 1 (torchrun) each rank runs an independent replica on its
own GPU (the path has no inter-GPU exchange): scaling "weak".
"""
from __future__ import annotations

import argparse
import json
import os
import re
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

NC, RHO, RC, DT, T_MELT = 64, 0.8442, 2.5, 0.005, 1.0
WORKLOAD = "lj-liquid-fcc64-1048576-rc2.5"
METRIC = "atom-steps/s on 1 GB300: mixed-FP32 vs FP64 path at <=1e-5 RMS force rel. error"
FP32_PEAK_TFLOPS = 73.84  # FFMA probe (python -m examd_gb300.peaks) on a GB300; used if the live probe fails


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rk = int(os.environ.get("RANK", "0"))
    lr = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rk, lr


def init_pg(ws):
    if ws <= 1:
        return None
    import torch.distributed as dist
    dist.init_process_group("gloo")
    return dist


def barrier(dist):
    if dist is not None:
        dist.barrier()


def allmax(dist, x):
    if dist is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def build_liquid(ex, seed=1):
    pos, L = ex.gen_fcc(NC, RHO)
    vel = ex.gen_velocities(len(pos), 2.0 * T_MELT, seed)
    return pos, vel, L


def melt(sysm, n, steps=300, every=50):
    """Melt the lattice: hot start, velocity rescaling to T_MELT every `every` steps."""
    for _ in range(steps // every):
        sysm.run(every, DT)
        ek = sysm.kinetic()[0]
        T = 2.0 * ek / (3.0 * (n - 1))
        sysm.scale_velocities(np.sqrt(T_MELT / T))


class ClockSampler:
    """nvidia-smi clock/throttle samples during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "100"],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        time.sleep(0.2)
        self.out = ""
        if self.p is not None:
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()
                self.out = ""

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def read_traffic():
    """dram bytes per pair-kernel launch from the committed ncu summary, if any."""
    p = os.path.join(ROOT, "profiles", "pair_mixed_fcc64_1048576.md")
    if not os.path.exists(p):
        return None
    m = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", open(p).read())
    return float(m.group(1)) if m else None


def fp32_peak():
    """FP32 FMA peak in TFLOP/s, measured now on this GPU by the pipe-rate probe."""
    try:
        from examd_gb300 import peaks
        r = peaks.measure()
        return float(r["fp32_tflops"]), (f"of measured: FFMA issue rate {r['ffma_per_clk_sm']:.1f}/clk/SM at "
                                          f"{r['clock_mhz']:.0f} MHz, python -m examd_gb300.peaks, this run "
                                          "(the driver-measured peaks have no FP32 figure)")
    except Exception as e:  # the probe is a measurement aid; the committed figure stands in
        return FP32_PEAK_TFLOPS, f"of measured earlier (profiles/gb300_pipe_rates.txt); live probe failed: {e}"


def drift_per_1000(e):
    """Least-squares slope of (E - E0)/|E0| per 1000 steps."""
    e = np.asarray(e, dtype=np.float64)
    s = np.arange(len(e))
    y = (e - e[0]) / abs(e[0])
    return float(np.polyfit(s, y, 1)[0] * 1000.0)


def cpu_baseline(pos, L, reps=2):
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    O.forces_typed(pos[: min(len(pos), 20000)], np.full(3, L), RC, threads=cores)  # warm
    t0 = time.perf_counter()
    for _ in range(reps):
        O.forces_typed(pos, np.full(3, L), RC, threads=cores)
    t = (time.perf_counter() - t0) / reps
    return {"value": len(pos) / t, "unit": "atom-steps/s", "cores": cores, "kind": "port",
            "sample": f"{reps} force evaluations of the {len(pos)}-atom workload by the C restatement of "
                      f"exaMD_forces_midpoint_all (OpenMP over home blocks, {cores} threads); "
                      f"{t:.3f} s each; integration O(N) neglected"}


def run_reference(args, ws, rk):
    """CPU restatement of the reference path, all host threads, same workload."""
    if rk != 0:
        return
    import examd_gb300 as ex
    from oracle import oracle as O
    O.build()
    pos, vel, L = build_liquid(ex)
    rng = np.random.default_rng(7)
    pos = (pos + rng.uniform(-0.15, 0.15, pos.shape)) % L  # liquid-like disorder without a GPU melt
    cores = os.cpu_count() or 1
    box = np.full(3, L)
    O.vv_run(pos, vel, box, RC, DT, max(args.warmup, 1), threads=cores)
    t0 = time.perf_counter()
    out = O.vv_run(pos, vel, box, RC, DT, args.steps, threads=cores)
    t = time.perf_counter() - t0
    v = len(pos) * args.steps / t
    line = {"metric": METRIC, "value": v, "unit": "atom-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "atoms": len(pos), "rc": RC, "dt": DT, "precision": "fp64",
                       "l2": "working set > L2"},
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "atom-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{args.steps} velocity-Verlet steps (force evaluation by the C restatement "
                                       f"of exaMD_forces_midpoint_all, OpenMP {cores} threads) of the "
                                       f"{len(pos)}-atom workload"},
            "e2e": {"value": v, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "final_epot": float(out["epot"][-1])}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="examd", choices=["examd", "reference"])
    ap.add_argument("--chunk", type=int, default=20, help="steps per captured CUDA graph")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 / drift side measurements")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    ws, rk, lr = dist_info()
    dist = init_pg(ws)
    if args.impl == "reference":
        run_reference(args, ws, rk)
        barrier(dist)
        return

    import examd_gb300 as ex
    from examd_gb300 import build as B
    B.build()
    pos, vel, L = build_liquid(ex, seed=1 + rk)
    n = len(pos)
    box = np.full(3, L)
    sysm = ex.MidpointLJ(box, [n], precision="mixed", rc=RC, device=lr)
    sysm.set_atoms(pos, vel=vel)
    melt(sysm, n)
    chunk = max(2, args.chunk // 2 * 2)
    wsteps = max(args.warmup, chunk + 2)
    wsteps += wsteps % 2
    sysm.run(wsteps, DT, graph_chunk=chunk)  # warm-up; captures the graph (even count keeps buffer parity)

    barrier(dist)
    with ClockSampler(lr) as clk:
        out = sysm.run(args.steps, DT, graph_chunk=chunk)
    barrier(dist)
    t_ms = allmax(dist, out["ms"])
    value = n * args.steps * ws / (t_ms * 1e-3)

    # pair-kernel roofline: algorithmic FLOPs per launch / event-timed duration
    cnt = sysm.counters()
    flops = 8.0 * cnt["candidates"] + 22.0 * cnt["accepted"]
    peak, peak_src = fp32_peak()
    reps = 20
    _, k_ms = sysm.time_forces(reps)
    achieved = flops / (k_ms * 1e-3) / 1e12
    traffic = read_traffic()

    # end to end through the drop-in force call with pinned host buffers
    melted, _ = sysm.state()
    hp = ex.pinned_empty((n, 3))
    hp[:] = melted
    hf = ex.pinned_empty((n, 3))
    sysm.forces_at(hp, out=hf)
    e2e_steps = max(args.steps // 2, 10)
    barrier(dist)
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        sysm.forces_at(hp, out=hf)
    t_e2e = allmax(dist, time.perf_counter() - t0)
    e2e = n * e2e_steps * ws / t_e2e

    extra = {}
    if not args.no_accuracy:
        f32, e32, _ = sysm.forces(energy=True)
        _, vmel = sysm.state()
        with ex.MidpointLJ(box, [n], precision="fp64", rc=RC, device=lr) as s64:
            s64.set_atoms(melted, vel=vmel)
            f64, e64, _ = s64.forces(energy=True)
            err = np.sqrt(((f32 - f64) ** 2).sum(1))
            fr = np.sqrt((f64 * f64).sum(1).mean())
            s64.run(4, DT)
            k64 = 10
            o64 = s64.run(k64, DT)
            v64 = n * k64 / (o64["ms"] * 1e-3)
            d64 = s64.run(1000, DT, graph_chunk=50, energies=True)
        dm = sysm.run(1000, DT, graph_chunk=50, energies=True)
        extra = {"fp64": {"value": v64, "ms_per_step": o64["ms"] / k64},
                 "mixed_over_fp64": value / ws / v64,
                 "force_rel_err_vs_fp64": {"rms": float(np.sqrt((err * err).mean()) / fr),
                                           "max": float(err.max() / fr)},
                 "epot_rel_err_vs_fp64": float(abs(e32[0] - e64[0]) / abs(e64[0])),
                 "energy_drift_per_1000_steps": {
                     "mixed": drift_per_1000(dm["ekin"][:, 0] + dm["epot"][:, 0]),
                     "fp64": drift_per_1000(d64["ekin"][:, 0] + d64["epot"][:, 0])}}

    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": wsteps, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "atoms": n, "rc": RC, "dt": DT, "precision": "mixed",
                       "graph_chunk": chunk, "l2": "working set > L2 (per-step HBM traffic ~0.2 GB)",
                       "parallelism": f"replicas{ws}"},
            "clocks": clk.summary(),
            "e2e": {"value": e2e, "unit": "atom-steps/s", "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 24 * n},
            "gpu_launches": 7 * args.steps + 1,
            "roofline": {"bound": "fp32", "kernel": "k_pair (mixed)", "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": traffic, "kernel_ms": k_ms, "flops_per_launch": flops,
                         "candidates": cnt["candidates"], "accepted": cnt["accepted"],
                         "peak_source": peak_src},
            **extra}
    if rk == 0 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(melted, L)
    if rk == 0:
        print(json.dumps(line), flush=True)
    sysm.close()
    barrier(dist)


if __name__ == "__main__":
    main()
