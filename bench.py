#!/usr/bin/env python3
"""Benchmark of the GB300 midpoint Lennard-Jones path (one JSON line on stdout).

Default workload: 1,048,576 atoms (FCC 64^3 x 4) at rho* = 0.8442, melted at
T* = 1.0, LJ eps = sigma = m = 1, rc = 2.5 sigma truncated and unshifted,
dt = 0.005, velocity-Verlet with re-binning every step.  A step = one
velocity-Verlet step over all atoms (kick + drift + wrap + binning + midpoint
pair forces).  Synthetic, seeded inputs; no dataset is involved.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl examd|reference]
                    [--workload liquid|liquid-rc3|slab|ensemble|mixture|fcc32k]

value: atom-steps/s of the mixed form with all state resident in HBM, device
time (CUDA events on the library's stream), max over ranks.  e2e: the same
metric through the drop-in force call with host buffers (pinned positions in,
forces out, every step).  The line also carries the FP64 form's rate on the
same atoms, the mixed form's force error against it and both forms' energy
drift per 1000 steps.  --impl reference times the CPU restatement of the
reference's force routine (oracle/) with all host threads on the same
workload.  With N > 1 (torchrun) each rank runs an independent replica on its
own GPU (the path has no inter-GPU exchange): scaling "weak".

Other workloads (--workload) are the remaining configurations of the same
metric: rc = 3.0; an uneven liquid slab in vapour; a batched ensemble of 512
boxes; a 16.8M-atom binary mixture; the 32,000-atom FCC fluid at T* = 0.72.
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
METRIC = "atom-steps/s on 1 GB300: mixed-FP32 vs FP64 path at <=1e-5 RMS force rel. error"
FP32_PEAK_TFLOPS = 73.84  # FFMA probe (python -m examd_gb300.peaks) on a GB300; used if the live probe fails

# name -> (workload label, dt, equilibration steps, rescale interval, drift steps)
WORKLOADS = {
    "liquid": ("lj-liquid-fcc64-1048576-rc2.5", 0.005, 300, 50, 1000),
    "liquid-rc3": ("lj-liquid-fcc64-1048576-rc3.0", 0.005, 300, 50, 1000),
    "slab": ("lj-slab-524288-rho0.75-in-vapour0.02-Lz4Lx-rc3.0", 0.005, 200, 20, 500),
    "ensemble": ("lj-ensemble-512-boxes-256-16384-rc2.5", 0.005, 200, 20, 1000),
    "mixture": ("lj-binary-mixture-16777216-80-20-rho1.2-rc2.5sigma", 0.003, 200, 20, 1000),
    "fcc32k": ("lj-fcc-32000-rho0.8442-T0.72-rc2.5", 0.005, 0, 0, 1000),
}


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


def make_case(name, seed):
    """Atoms, boxes and LJ parameters of a workload, plus each box's target temperature."""
    import examd_gb300 as ex
    from examd_gb300 import workloads as W
    if name in ("liquid", "liquid-rc3"):
        pos, vel, L = build_liquid(ex, seed)  # hot start at 2 T*, melted by the equilibration
        case = {"pos": pos, "vel": vel, "types": None, "boxes": np.full((1, 3), L), "natoms": np.array([len(pos)]),
                "lj": {"rc": 3.0 if name == "liquid-rc3" else RC}}
        return case, np.array([T_MELT])
    if name == "slab":
        return W.slab(seed=seed + 2), np.array([0.85])
    if name == "ensemble":
        c = W.ensemble(seed=seed + 3)
        return c, c["temperatures"]
    if name == "mixture":
        return W.binary_mixture(seed=seed + 4), np.array([1.0])
    if name == "fcc32k":
        pos, L = ex.gen_fcc(20, RHO)
        vel = ex.gen_velocities(len(pos), 0.72, seed)
        case = {"pos": pos, "vel": vel, "types": None, "boxes": np.full((1, 3), L), "natoms": np.array([len(pos)]),
                "lj": {"rc": RC}}
        return case, np.array([0.72])
    raise ValueError(name)


def equilibrate(sysm, natoms, temps, steps, every, dt):
    """steps velocity-Verlet steps, rescaling each box to its target temperature every `every` steps."""
    dof = 3.0 * np.maximum(np.asarray(natoms, dtype=np.float64) - 1.0, 1.0)
    for _ in range(steps // every if every else 0):
        sysm.run(every, dt)
        T = 2.0 * sysm.kinetic() / dof
        sysm.scale_velocities(np.sqrt(temps / np.maximum(T, 1e-12)))


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
                                          "(MEASURED_PEAKS.json holds no FP32 figure)")
    except Exception as e:  # the probe is a measurement aid; the committed figure stands in
        return FP32_PEAK_TFLOPS, f"of measured earlier (profiles/gb300_pipe_rates.txt); live probe failed: {e}"


def drift_per_1000(e, scale=None):
    """Least-squares slope of (E - E0)/|E0| per 1000 steps (or of (E - E0)/scale)."""
    e = np.asarray(e, dtype=np.float64)
    s = np.arange(len(e))
    y = (e - e[0]) / (abs(e[0]) if scale is None else scale)
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
    t1 = time.perf_counter()
    O.forces_typed(pos, np.full(3, L), RC, threads=1)  # one core, as one reference MPI rank runs
    t1 = time.perf_counter() - t1
    return {"value": len(pos) / t, "unit": "atom-steps/s", "cores": cores, "kind": "port",
            "sample": f"{reps} force evaluations of the {len(pos)}-atom workload by the C restatement of "
                      f"exaMD_forces_midpoint_all (OpenMP over home blocks, {cores} threads); "
                      f"{t:.3f} s each; integration O(N) neglected",
            "single_core": {"value": len(pos) / t1, "cores": 1,
                            "sample": f"1 force evaluation on one thread, {t1:.3f} s"}}


def run_reference(args, ws, rk):
    """CPU restatement of the reference path, all host threads, same workload."""
    if rk != 0:
        return
    if args.workload != "liquid":
        print(json.dumps({"impl": "reference", "unavailable": f"the CPU arm covers the default workload only, "
                                                              f"not {args.workload}"}), flush=True)
        return
    import examd_gb300 as ex
    from oracle import oracle as O
    O.build()
    pos, vel, L = build_liquid(ex)
    rng = np.random.default_rng(7)
    pos = (pos + rng.uniform(-0.15, 0.15, pos.shape)) % L  # liquid-like disorder without a GPU melt
    cores = os.cpu_count() or 1
    box = np.full(3, L)
    w = O.vv_run(pos, vel, box, RC, DT, max(args.warmup, 1), threads=cores)
    # the timed steps continue the warm-up trajectory from its forces: exactly `steps` force evaluations
    t0 = time.perf_counter()
    out = O.vv_run(w["pos"], w["vel"], box, RC, DT, args.steps, threads=cores, forces=w["forces"])
    t = time.perf_counter() - t0
    v = len(pos) * args.steps / t
    line = {"metric": METRIC, "value": v, "unit": "atom-steps/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOADS["liquid"][0], "atoms": len(pos), "rc": RC, "dt": DT,
                       "precision": "fp64", "l2": "working set > L2"},
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
    ap.add_argument("--workload", default="liquid", choices=sorted(WORKLOADS))
    ap.add_argument("--chunk", type=int, default=20, help="steps per captured CUDA graph")
    ap.add_argument("--drift-steps", type=int, default=None, help="steps of the energy-drift runs")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 / drift side measurements")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-tune", action="store_true", help="default tile shape instead of the autotuner's")
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
    label, dt, eq_steps, eq_every, drift_steps = WORKLOADS[args.workload]
    if args.drift_steps is not None:
        drift_steps = args.drift_steps
    case, temps = make_case(args.workload, 1 + rk)
    n = int(case["natoms"].sum())
    nboxes = len(case["natoms"])
    lj = dict(case["lj"])
    sysm = ex.MidpointLJ(case["boxes"], case["natoms"], precision="mixed", device=lr, **lj)
    sysm.set_atoms(case["pos"], case["types"], case["vel"])
    equilibrate(sysm, case["natoms"], temps, eq_steps, eq_every, dt)
    tuning = {"tile": "default", "warps": "default", "tile_balance": 0}
    if not args.no_tune:
        # tile shape, warps per CTA and tile split for the equilibrated atoms (examd_autotune)
        pos_eq, vel_eq = sysm.state()
        tuning = ex.autotune(case["boxes"], case["natoms"], pos_eq, case["types"], precision="mixed", device=lr,
                             **lj)
        sysm.close()
        sysm = ex.MidpointLJ(case["boxes"], case["natoms"], precision="mixed", device=lr, tile=tuning["tile"],
                             warps=tuning["warps"], tile_balance=tuning["tile_balance"], **lj)
        sysm.set_atoms(pos_eq, case["types"], vel_eq)
    chunk = max(2, args.chunk // 2 * 2)
    wsteps = max(args.warmup, chunk + 2)
    wsteps += wsteps % 2
    sysm.run(wsteps, dt, graph_chunk=chunk)  # warm-up; captures the graph (even count keeps buffer parity)

    barrier(dist)
    with ClockSampler(lr) as clk:
        out = sysm.run(args.steps, dt, graph_chunk=chunk)
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
    traffic = read_traffic() if args.workload == "liquid" else None

    # end to end through the drop-in force call with pinned host buffers
    state, _ = sysm.state()
    hp = ex.pinned_empty((n, 3))
    hp[:] = state
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
        pos_now, vel_now = sysm.state()
        with ex.MidpointLJ(case["boxes"], case["natoms"], precision="fp64", device=lr, **lj) as s64:
            s64.set_atoms(pos_now, case["types"], vel_now)
            f64, e64, _ = s64.forces(energy=True)
            err = np.sqrt(((f32 - f64) ** 2).sum(1))
            fr = np.sqrt((f64 * f64).sum(1).mean())
            s64.run(4, dt)
            k64 = 10
            o64 = s64.run(k64, dt)
            v64 = n * k64 / (o64["ms"] * 1e-3)
            d64 = s64.run(drift_steps, dt, graph_chunk=50, energies=True)
        dm = sysm.run(drift_steps, dt, graph_chunk=50, energies=True)
        em = dm["ekin"] + dm["epot"]
        e6 = d64["ekin"] + d64["epot"]
        drift_m = [drift_per_1000(em[:, b]) for b in range(nboxes)]
        drift_d = [drift_per_1000(e6[:, b]) for b in range(nboxes)]
        extra = {"fp64": {"value": v64, "ms_per_step": o64["ms"] / k64},
                 "mixed_over_fp64": value / ws / v64,
                 "force_rel_err_vs_fp64": {"rms": float(np.sqrt((err * err).mean()) / fr),
                                           "max": float(err.max() / fr)},
                 "epot_rel_err_vs_fp64": float(np.abs(e32.sum() - e64.sum()) / abs(e64.sum())),
                 "energy_drift_per_1000_steps": {"mixed": drift_m[0], "fp64": drift_d[0], "steps": drift_steps}}
        if nboxes > 1:
            # a box's total energy can be near zero (gas-like boxes), which makes
            # (E - E0)/|E0| meaningless there: also report (E - E0)/<Ekin>
            km, k6 = dm["ekin"].mean(0), d64["ekin"].mean(0)
            am, ad = np.abs(drift_m), np.abs(drift_d)
            bm = np.abs([drift_per_1000(em[:, b], km[b]) for b in range(nboxes)])
            bd = np.abs([drift_per_1000(e6[:, b], k6[b]) for b in range(nboxes)])
            extra["energy_drift_per_1000_steps"] = {
                "mixed": {"median_abs": float(np.median(am)), "max_abs": float(am.max()),
                          "median_abs_vs_ekin": float(np.median(bm)), "max_abs_vs_ekin": float(bm.max())},
                "fp64": {"median_abs": float(np.median(ad)), "max_abs": float(ad.max()),
                         "median_abs_vs_ekin": float(np.median(bd)), "max_abs_vs_ekin": float(bd.max())},
                "per_box": "per-box drift; median and max of |drift| over the boxes, relative to |E0| and "
                           "to the box's mean kinetic energy", "steps": drift_steps}

    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": wsteps, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": label, "atoms": n, "boxes": nboxes, "rc": lj.get("rc"), "dt": dt,
                       "precision": "mixed", "graph_chunk": chunk,
                       "tile": list(tuning["tile"]) if isinstance(tuning["tile"], tuple) else tuning["tile"],
                       "warps": tuning["warps"], "tile_balance": tuning["tile_balance"],
                       "l2": "working set > L2 (per-step HBM traffic ~0.2 KB per atom)" if n * 200 > 129e6
                       else "working set fits L2 (small configuration)",
                       "parallelism": f"replicas{ws}"},
            "clocks": clk.summary(),
            "e2e": {"value": e2e, "unit": "atom-steps/s", "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 24 * n},
            # per step: kick+drift+bin count, 2 scan kernels, finalize, pair, redo pass
            "gpu_launches": 6 * args.steps + 1,
            # pair rates of the timed run (the counters of one force evaluation x steps / time)
            "pairs": {"interactions_per_s": cnt["accepted"] * args.steps * ws / (t_ms * 1e-3),
                      "candidates_per_s": cnt["candidates"] * args.steps * ws / (t_ms * 1e-3),
                      "kernel_interactions_per_s": cnt["accepted"] / (k_ms * 1e-3)},
            "roofline": {"bound": "fp32", "kernel": "k_pair (mixed)", "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": traffic, "kernel_ms": k_ms, "flops_per_launch": flops,
                         "candidates": cnt["candidates"], "accepted": cnt["accepted"],
                         "peak_source": peak_src},
            **extra}
    if rk == 0 and not args.no_cpu and args.workload == "liquid":
        line["cpu_baseline"] = cpu_baseline(state, case["boxes"][0, 0])
    if rk == 0:
        print(json.dumps(line), flush=True)
    sysm.close()
    barrier(dist)


if __name__ == "__main__":
    main()
