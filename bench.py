#!/usr/bin/env python3
"""Benchmark of the GB300 midpoint Lennard-Jones path (one JSON line on stdout).

Default workload: the largest configuration that fits one GPU, 16,777,216
atoms of an 80:20 two-species LJ mixture (Kob-Andersen-type table eps_AA = 1,
sigma_AA = 1, eps_AB = 1.5, sigma_AB = 0.8, eps_BB = 0.5, sigma_BB = 0.88,
cutoff 2.5 sigma_ab per pair) on a jittered simple-cubic lattice at rho* =
1.2, T* = 1.0, dt = 0.003.  A step = one velocity-Verlet step over all atoms
(kick + drift + wrap + binning + midpoint pair forces).  Synthetic, seeded
inputs built by examd_gb300/workloads.py (plain numpy); no dataset is
involved.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl examd|reference]
                    [--workload mixture|liquid|liquid-rc3|slab|ensemble|fcc32k]

Both arms time the same state: the workload's seeded atoms after W warm-up
steps, then K timed steps.

value: atom-steps/s of the mixed form with all state resident in HBM, device
time (CUDA events on the library's stream, the step loop replayed as CUDA
graphs captured before the timed region), max over ranks.  The mixed form
runs with per-tile pair lists (skin 0.3 sigma, --pair-skin; 0 for cells and
candidates at every step): a step computes its forces from the lists, and
the cells and lists are rebuilt at the steps whose atoms moved more than half
the skin, inside the timed steps.  e2e: the same metric through the drop-in
force call with host buffers (pinned positions in, forces out, every call;
the positions of consecutive steps in turn).  The line also carries the pair
kernel's roofline,
per-phase times, the CPU baseline (the oracle on the machine's host cores), and,
on a separately equilibrated state, the FP64 form's rate at its own tuned
tiles, the mixed form's force error against it and both forms' energy drift.
--impl reference times the CPU restatement of the reference's force routine
(oracle/) with all host threads on the same workload and state, loading no
library of the product.  With N > 1 (torchrun) each rank runs an independent
replica on its own GPU (the path has no inter-GPU exchange): scaling "weak".

Other workloads (--workload) are the remaining configurations of the same
metric: the 1,048,576-atom liquid at rc 2.5 and 3.0; an uneven liquid slab in
vapour; a batched ensemble of 512 boxes; the 32,000-atom FCC crystal at T* =
0.72.
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import os
import re
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "atom-steps/s on 1 GB300: mixed-FP32 vs FP64 path at <=1e-5 RMS force rel. error"
FP32_PEAK_TFLOPS = 73.84  # FFMA probe (python -m examd_gb300.peaks) on a GB300; used if the live probe fails

# name -> workload label, generator name and arguments, dt, equilibration steps (velocity rescaling every
# `every` steps), steps of NVE before the drift window, drift window
WORKLOADS = {
    "mixture": dict(label="lj-binary-mixture-16777216-80-20-rho1.2-rc2.5sigma", gen="binary_mixture",
                    args={"m": 256, "seed": 5}, dt=0.003, eq=2000, every=20, settle=200, drift=1000),
    "liquid": dict(label="lj-liquid-fcc64-1048576-rc2.5", gen="liquid_fcc", args={"nc": 64, "rc": 2.5, "seed": 1},
                   dt=0.005, eq=2000, every=20, settle=200, drift=1000),
    "liquid-rc3": dict(label="lj-liquid-fcc64-1048576-rc3.0", gen="liquid_fcc",
                       args={"nc": 64, "rc": 3.0, "seed": 1}, dt=0.005, eq=2000, every=20, settle=200, drift=1000),
    "slab": dict(label="lj-slab-524288-rho0.75-in-vapour0.02-Lz4Lx-rc3.0", gen="slab", args={"seed": 3},
                 dt=0.005, eq=2000, every=20, settle=200, drift=500),
    "ensemble": dict(label="lj-ensemble-512-boxes-256-16384-rc2.5", gen="ensemble", args={"seed": 4},
                     dt=0.005, eq=2000, every=20, settle=200, drift=1000),
    # the perfect lattice has zero forces: 100 NVE steps move the atoms off their sites before the force
    # comparison (a relative error against F_rms = 0 would mean nothing)
    "fcc32k": dict(label="lj-fcc-32000-rho0.8442-T0.72-rc2.5", gen="fcc_lattice", args={"nc": 20, "seed": 1},
                   dt=0.005, eq=0, every=0, settle=100, drift=1000),
}
DEFAULT_WORKLOAD = "mixture"
# the mixed form's pair lists: the skin (pairs within rc + skin, rebuilt when
# an atom has moved skin/2 since the last build; 0: no lists, cells and
# candidates at every step) is picked among these by short untimed runs of
# the workload's own dynamics (a larger skin rebuilds less often and tests
# more pairs per step), among those whose cell edge (rc + skin)/2 leaves
# every box at least 5 cells per axis
PAIR_SKINS = (0.0, 0.3, 0.4, 0.5)


def skins_allowed(case):
    """The candidate skins whose cells of edge (rc + skin)/2 leave 5 per axis in every box."""
    rc = np.max(case["lj"]["rc"])
    lmin = float(np.min(case["boxes"]))
    return [sk for sk in PAIR_SKINS if (rc + sk) / 2.0 * 1.001 * 5.0 <= lmin]


def load_workloads():
    """examd_gb300/workloads.py by its path: the generators are plain numpy,
    and loading the file alone keeps the package (and its CUDA library) out
    of the reference arm's process."""
    spec = importlib.util.spec_from_file_location("examd_workloads", os.path.join(ROOT, "examd_gb300", "workloads.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def make_case(name):
    w = WORKLOADS[name]
    return getattr(load_workloads(), w["gen"])(**w["args"])


def config_of(name, case):
    """The `config` object both arms print (no implementation-specific keys)."""
    w = WORKLOADS[name]
    n = int(case["natoms"].sum())
    lj = case["lj"]
    rc = lj.get("rc")
    return {"workload": w["label"], "atoms": n, "boxes": int(len(case["natoms"])),
            "rc": rc if np.ndim(rc) == 0 else np.asarray(rc).tolist(), "dt": w["dt"],
            "state": f"{w['gen']}({', '.join(f'{k}={v}' for k, v in w['args'].items())}) then the warm-up steps",
            "l2": ("working set > L2 (per-step HBM traffic ~0.2 KB per atom)" if n * 200 > 129e6
                   else "working set fits L2 (small configuration)")}


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


def read_traffic(workload, lists=False):
    """DRAM bytes per pair-kernel launch from the committed ncu summary of this workload, if any."""
    names = {"mixture": ("pair_mixed_mixture_2097152.md", "traffic_bytes_per_launch_16777216"),
             "liquid": ("pair_mixed_fcc64_1048576.md", "traffic_bytes_per_launch")}
    if lists:
        names = {"mixture": ("pair_list_mixture_2097152.md", "traffic_bytes_per_launch_16777216"),
                 "liquid": ("pair_list_liquid_1048576.md", "traffic_bytes_per_launch")}
    if workload not in names:
        return None, None
    fname, key = names[workload]
    p = os.path.join(ROOT, "profiles", fname)
    if not os.path.exists(p):
        return None, None
    m = re.search(key + r":\s*([0-9.eE+]+)", open(p).read())
    return (float(m.group(1)), f"profiles/{fname} ({key})") if m else (None, None)


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


def _oracle_boxes(case):
    """(pos, types, box) per box of a case, for the oracle (one box at a time)."""
    a0 = np.concatenate([[0], np.cumsum(case["natoms"])])
    t = case["types"]
    for b in range(len(case["natoms"])):
        yield (case["pos"][a0[b]:a0[b + 1]], None if t is None else t[a0[b]:a0[b + 1]], case["boxes"][b],
               case["vel"][a0[b]:a0[b + 1]])


def _oracle_lj(case):
    lj = case["lj"]
    return dict(rc=lj["rc"], eps=lj.get("eps", 1.0), sigma=lj.get("sigma", 1.0), ntypes=lj.get("ntypes", 1))


def cpu_baseline(case, budget_s=30.0):
    """Force evaluations of the oracle (the C restatement of
    exaMD_forces_midpoint_all) on the given atoms, all host threads: the
    reference's timed call (exaMD.f90:241-253) turned into atom-steps/s."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    lj = _oracle_lj(case)
    n = int(case["natoms"].sum())

    def one(threads):
        t0 = time.perf_counter()
        for p, t, L, _ in _oracle_boxes(case):
            O.forces_typed(p, L, types=t, threads=threads, **lj)
        return time.perf_counter() - t0

    t_first = one(cores)
    reps = int(max(1, min(3, budget_s // max(t_first, 1e-3))))
    ts = [one(cores) for _ in range(reps)]
    t = float(np.mean(ts))
    out = {"value": n / t, "unit": "atom-steps/s", "cores": cores, "kind": "port",
           "sample": f"{reps} force evaluations (after one untimed) of the {n}-atom workload on its generated "
                     f"state by the C restatement of exaMD_forces_midpoint_all (OpenMP over home blocks, "
                     f"{cores} threads), {t:.3f} s each; integration O(N) neglected"}
    if t * cores < budget_s:
        t1 = one(1)
        out["single_core"] = {"value": n / t1, "cores": 1, "sample": f"1 force evaluation on one thread, {t1:.3f} s"}
    return out


def run_reference(args, ws, rk):
    """The CPU restatement of the reference path, all host threads, on the
    workload's generated state: W warm-up steps, then timed steps of
    velocity-Verlet whose forces come from the restated
    exaMD_forces_midpoint_all.  Loads no library of the product."""
    if rk != 0:
        return
    from oracle import oracle as O
    O.build()
    case = make_case(args.workload)
    w = WORKLOADS[args.workload]
    dt = w["dt"]
    cores = os.cpu_count() or 1
    lj = _oracle_lj(case)
    mass = case["lj"].get("mass")
    boxes = list(_oracle_boxes(case))
    n = int(case["natoms"].sum())
    states = []
    t0 = time.perf_counter()
    for p, t, L, v in boxes:
        r = O.vv_run(p, v, L, dt=dt, nsteps=args.warmup, types=t, mass=mass, threads=cores, **lj)
        states.append((r["pos"], r["vel"], r["forces"], t, L))
    t_warm = (time.perf_counter() - t0) / max(args.warmup, 1)
    # the timed steps continue the warm-up trajectory from its forces: exactly K force evaluations; a step
    # that would take the run past about 150 s is not started (a bounded sample of the K steps)
    k_run = int(max(1, min(args.steps, 150.0 // max(t_warm, 1e-6))))
    t0 = time.perf_counter()
    for p, v, f, t, L in states:
        O.vv_run(p, v, L, dt=dt, nsteps=k_run, types=t, mass=mass, threads=cores, forces=f, **lj)
    t = time.perf_counter() - t0
    val = n * k_run / t
    sample = (f"{k_run} velocity-Verlet steps (forces by the C restatement of exaMD_forces_midpoint_all, OpenMP "
              f"{cores} threads) of the {n}-atom workload after {args.warmup} warm-up steps"
              + (f"; {k_run} of the {args.steps} requested steps timed, to bound the run" if k_run < args.steps
                 else ""))
    line = {"metric": METRIC, "value": val, "unit": "atom-steps/s", "n_gpus": args.gpus, "steps": k_run,
            "warmup": args.warmup, "ms_per_step": 1e3 * t / k_run, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_of(args.workload, case),
            "impl": "reference",
            "cpu_baseline": {"value": val, "unit": "atom-steps/s", "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "atom-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def equilibrate(sysm, natoms, temps, steps, every, dt):
    """steps velocity-Verlet steps, rescaling each box to its target temperature every `every` steps."""
    dof = 3.0 * np.maximum(np.asarray(natoms, dtype=np.float64) - 1.0, 1.0)
    for _ in range(steps // every if every else 0):
        sysm.run(every, dt, graph_chunk=every)
        T = 2.0 * sysm.kinetic() / dof
        sysm.scale_velocities(np.sqrt(temps / np.maximum(T, 1e-12)))


def accuracy_and_drift(ex, case, w, lj, tuning, lr, dt):
    """On an equilibrated state (rescaled, then NVE): the mixed form's force
    error against the FP64 form, the FP64 form's rate at its own tuned tiles
    (graph-captured as the mixed form), and both forms' energy drift."""
    natoms, boxes, types = case["natoms"], case["boxes"], case["types"]
    nboxes = len(natoms)
    n = int(natoms.sum())
    with ex.MidpointLJ(boxes, natoms, precision="mixed", device=lr, **tuning, **lj) as s:
        s.set_atoms(case["pos"], types, case["vel"])
        equilibrate(s, natoms, case["temperatures"], w["eq"], w["every"], dt)
        if w["settle"]:
            s.run(w["settle"], dt, graph_chunk=20)
        pos_eq, vel_eq = s.state()
        f32, e32, _ = s.forces(energy=True)
        dm = s.run(w["drift"], dt, graph_chunk=50, energies=True)
        s.set_atoms(pos_eq, types, vel_eq)
        s.run(4, dt)
        s.prepare_run(dt, 10)
        o32 = s.run(20, dt, graph_chunk=10)
    t64 = ex.autotune(boxes, natoms, pos_eq, types, precision="fp64", device=lr, **lj)
    tune64 = {"tile": t64["tile"], "warps": t64["warps"], "tile_balance": t64["tile_balance"],
              "block_length": t64["block_length"]}
    with ex.MidpointLJ(boxes, natoms, precision="fp64", device=lr, **tune64, **lj) as s64:
        s64.set_atoms(pos_eq, types, vel_eq)
        f64, e64, _ = s64.forces(energy=True)
        d64 = s64.run(w["drift"], dt, graph_chunk=50, energies=True)
        s64.set_atoms(pos_eq, types, vel_eq)
        s64.run(4, dt)
        k64 = 20
        s64.prepare_run(dt, 10)
        o64 = s64.run(k64, dt, graph_chunk=10)
    err = np.sqrt(((f32 - f64) ** 2).sum(1))
    fr = np.sqrt((f64 * f64).sum(1).mean())
    v64 = n * k64 / (o64["ms"] * 1e-3)
    v32 = n * 20 / (o32["ms"] * 1e-3)
    em = dm["ekin"] + dm["epot"]
    e6 = d64["ekin"] + d64["epot"]
    drift_m = [drift_per_1000(em[:, b]) for b in range(nboxes)]
    drift_d = [drift_per_1000(e6[:, b]) for b in range(nboxes)]
    out = {"fp64": {"value": v64, "ms_per_step": o64["ms"] / k64, "tile": list(tune64["tile"]),
                    "warps": tune64["warps"], "tile_balance": tune64["tile_balance"],
                    "cell_edge": tune64["block_length"] or "rc/2 (the reference's)", "graph_chunk": 10,
                    "state": "equilibrated"},
           "mixed_equilibrated": {"value": v32, "ms_per_step": o32["ms"] / 20, "graph_chunk": 10},
           "mixed_over_fp64": v32 / v64,
           "force_rel_err_vs_fp64": {"rms": float(np.sqrt((err * err).mean()) / fr), "max": float(err.max() / fr),
                                     "state": "equilibrated"},
           "epot_rel_err_vs_fp64": float(np.abs(e32.sum() - e64.sum()) / abs(e64.sum())),
           "equilibration": {"steps": w["eq"], "rescale_every": w["every"], "nve_steps": w["settle"]}}
    if nboxes == 1:
        out["energy_drift_per_1000_steps"] = {"mixed": drift_m[0], "fp64": drift_d[0], "steps": w["drift"]}
    else:
        # a box's total energy can be near zero (gas-like boxes), which makes
        # (E - E0)/|E0| meaningless there: also report (E - E0)/<Ekin>
        km, k6 = dm["ekin"].mean(0), d64["ekin"].mean(0)
        am, ad = np.abs(drift_m), np.abs(drift_d)
        bm = np.abs([drift_per_1000(em[:, b], km[b]) for b in range(nboxes)])
        bd = np.abs([drift_per_1000(e6[:, b], k6[b]) for b in range(nboxes)])
        out["energy_drift_per_1000_steps"] = {
            "mixed": {"median_abs": float(np.median(am)), "max_abs": float(am.max()),
                      "median_abs_vs_ekin": float(np.median(bm)), "max_abs_vs_ekin": float(bm.max())},
            "fp64": {"median_abs": float(np.median(ad)), "max_abs": float(ad.max()),
                     "median_abs_vs_ekin": float(np.median(bd)), "max_abs_vs_ekin": float(bd.max())},
            "per_box": "per-box drift; median and max of |drift| over the boxes, relative to |E0| and "
                       "to the box's mean kinetic energy", "steps": w["drift"]}
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="examd", choices=["examd", "reference"])
    ap.add_argument("--workload", default=DEFAULT_WORKLOAD, choices=sorted(WORKLOADS))
    ap.add_argument("--chunk", type=int, default=20, help="steps per captured CUDA graph")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 / drift side measurements")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    ap.add_argument("--no-tune", action="store_true", help="default tile shape instead of the autotuner's")
    ap.add_argument("--pair-skin", type=float, default=None,
                    help="mixed form's pair-list skin in sigma (0: cells and candidates at every step; "
                         "default: picked among 0.3, 0.4, 0.5)")
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
    w = WORKLOADS[args.workload]
    dt = w["dt"]
    case = make_case(args.workload)  # every replica times the same seeded state
    n = int(case["natoms"].sum())
    nboxes = len(case["natoms"])
    lj = dict(case["lj"])
    cands = skins_allowed(case)
    # the tiles are tuned at the middle candidate skin
    skin = float(args.pair_skin) if args.pair_skin is not None else cands[(len(cands) - 1) // 2 + (len(cands) > 2)]
    tuning = {"pair_skin": skin}
    edge0 = "(rc + skin)/2" if skin > 0 else "rc/2 (the reference's)"
    tune_info = {"tile": "default", "warps": "default", "tile_balance": 0, "pair_skin": skin}
    if not args.no_tune:
        # tile shape, warps per CTA, tile split and cell edge for these atoms (examd_autotune)
        t = ex.autotune(case["boxes"], case["natoms"], case["pos"], case["types"], precision="mixed", device=lr,
                        pair_skin=skin, **lj)
        tuning = {"tile": t["tile"], "warps": t["warps"], "tile_balance": t["tile_balance"],
                  "block_length": t["block_length"], "pair_skin": skin}
        tune_info = {"tile": list(t["tile"]), "warps": t["warps"], "tile_balance": t["tile_balance"],
                     "cell_edge": t["block_length"] or edge0, "pair_skin": skin}
    if args.pair_skin is None and len(cands) > 1:
        # the skin: a short run from the workload's state at each candidate, the tiles above (long enough to
        # hold several rebuilds: 20 steps for millions of atoms, 100 for smaller systems)
        ntrial = 20 if n > 4_000_000 else 100
        trial = {}
        for sk in cands:
            with ex.MidpointLJ(case["boxes"], case["natoms"], precision="mixed", device=lr,
                               **dict(tuning, pair_skin=sk), **lj) as s:
                s.set_atoms(case["pos"], case["types"], case["vel"])
                s.run(args.warmup, dt)
                s.prepare_run(dt, 20)
                trial[sk] = s.run(ntrial, dt, graph_chunk=20)["ms"] / ntrial
        tuned_at = skin
        skin = min(trial, key=trial.get)
        tuning["pair_skin"] = skin
        tune_info["pair_skin"] = skin
        tune_info["pair_skin_trials_ms_per_step"] = {str(k): v for k, v in trial.items()}
        if skin != tuned_at and not args.no_tune:  # the tiles again, for the skin picked
            t = ex.autotune(case["boxes"], case["natoms"], case["pos"], case["types"], precision="mixed",
                            device=lr, pair_skin=skin, **lj)
            tuning.update(tile=t["tile"], warps=t["warps"], tile_balance=t["tile_balance"],
                          block_length=t["block_length"])
            tune_info.update(tile=list(t["tile"]), warps=t["warps"], tile_balance=t["tile_balance"],
                             cell_edge=t["block_length"] or ("(rc + skin)/2" if skin > 0 else "rc/2 (the reference's)"))
    sysm = ex.MidpointLJ(case["boxes"], case["natoms"], precision="mixed", device=lr, **tuning, **lj)
    # the end-to-end leg's page-locked host buffers, allocated before the run's large host arrays
    hp = ex.pinned_empty((n, 3))
    hf = ex.pinned_empty((n, 3))
    sysm.set_atoms(case["pos"], case["types"], case["vel"])
    sysm.run(args.warmup, dt)  # exactly W untimed steps
    chunk = max(2, args.chunk // 2 * 2)
    sysm.prepare_run(dt, chunk)  # capture the step-loop graph outside the timed region

    b0 = sysm.list_info()["builds"]
    barrier(dist)
    with ClockSampler(lr) as clk:
        out = sysm.run(args.steps, dt, graph_chunk=chunk)
    barrier(dist)
    t_ms = allmax(dist, out["ms"])
    value = n * args.steps * ws / (t_ms * 1e-3)
    builds = sysm.list_info()["builds"] - b0  # rebuilds of the cells and pair lists in the timed steps

    # pair-kernel roofline: algorithmic FLOPs per launch / event-timed duration.  The candidates are the
    # reference's pair calls at its own cell edge rc/2 (exaMD.f90:56), whatever edge the run uses
    cnt = sysm.counters()
    if tuning.get("block_length") or skin > 0:
        pos_now, _ = sysm.state()
        with ex.MidpointLJ(case["boxes"], case["natoms"], precision="mixed", device=lr, **lj) as s0:
            s0.set_atoms(pos_now, case["types"])
            cnt["candidates"] = s0.counters()["candidates"]
    flops = 8.0 * cnt["candidates"] + 22.0 * cnt["accepted"]
    peak, peak_src = fp32_peak()
    _, k_ms = sysm.time_forces(20)
    achieved = flops / (k_ms * 1e-3) / 1e12
    traffic, traffic_src = read_traffic(args.workload, skin > 0)
    rebuild_ms = sysm.time_rebuild(2) if skin > 0 else 0.0

    # end to end through the drop-in force call with pinned host buffers: the caller's positions of
    # consecutive steps (a pair-list context rebuilds when they have moved far enough since its build),
    # each call timed from the host with the host->device and device->host copies inside
    nstate = min(max(args.steps // 2, 10), 10 if n <= 4_000_000 else 4)
    states = []
    for _ in range(nstate):
        sysm.run(1, dt)
        states.append(sysm.state()[0])
    hp[:] = states[-1]
    sysm.forces_at(hp, out=hf)
    sysm.forces_at(hp, out=hf)  # the captured call, at both parities of the sort's double buffer
    e2e_steps = max(args.steps // 2, 10)
    t_e2e = 0.0
    builds0 = sysm.list_info()["builds"] if skin > 0 else 0
    for k in range(e2e_steps):
        hp[:] = states[k % nstate]
        barrier(dist)
        t0 = time.perf_counter()
        sysm.forces_at(hp, out=hf)
        t_e2e += time.perf_counter() - t0
    t_e2e = allmax(dist, t_e2e)
    e2e = n * e2e_steps * ws / t_e2e
    e2e_rebuilds = sysm.list_info()["builds"] - builds0 if skin > 0 else 0
    phases = sysm.time_phases(10, dt)  # advances the state: last
    sysm.close()

    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": t_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic", "config": config_of(args.workload, case),
            "precision": "mixed", "tuning": {**tune_info, "graph_chunk": chunk},
            "clocks": clk.summary(),
            "e2e": {"value": e2e, "unit": "atom-steps/s", "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 24 * n,
                    "call": "examd_gpu_forces_at (positions in, forces out, pinned host buffers), "
                            f"positions of {nstate} consecutive steps in turn, each call timed",
                    "calls": e2e_steps, "list_rebuilds_in_calls": e2e_rebuilds},
            # per step: kick+drift+bin count, 2 scan kernels, finalize, pair, redo pass (pair lists: kick, the
            # rebuild decision, bin count, 2 scan kernels, finalize, copy-back and list build, which return at
            # once on a step that does not rebuild, list pass, redo pass); + the closing kick
            "gpu_launches": (10 if skin > 0 else 6) * args.steps + 1,
            "phases_ms_per_step": phases,
            # pair rates of the timed run (the counters of one force evaluation x steps / time)
            "pairs": {"interactions_per_s": cnt["accepted"] * args.steps * ws / (t_ms * 1e-3),
                      "candidates_per_s": cnt["candidates"] * args.steps * ws / (t_ms * 1e-3),
                      "kernel_interactions_per_s": cnt["accepted"] / (k_ms * 1e-3)},
            "roofline": {"bound": "fp32", "kernel": "k_pair_list (mixed, pair lists)" if skin > 0 else "k_pair (mixed)",
                         "achieved": achieved,
                         "peak": peak, "unit": "TFLOP/s", "frac": achieved / peak,
                         "traffic": traffic, "traffic_source": traffic_src, "kernel_ms": k_ms,
                         "flops_per_launch": flops, "candidates": cnt["candidates"], "accepted": cnt["accepted"],
                         "peak_source": peak_src}}
    if skin > 0:
        # the pair work of a step with the rebuilds' share: the list pass plus the timed steps' rebuilds
        per_step_ms = k_ms + rebuild_ms * builds / args.steps
        line["pair_lists"] = {"skin": skin, "rebuilds_in_timed_steps": builds, "steps": args.steps,
                              "list_pass_ms": k_ms, "rebuild_ms": rebuild_ms,
                              "pair_ms_per_step_with_rebuilds": per_step_ms,
                              "achieved_per_step_tflops": flops / (per_step_ms * 1e-3) / 1e12,
                              "frac_per_step": flops / (per_step_ms * 1e-3) / 1e12 / peak}
    if ws == 1 and not args.no_accuracy:
        line.update(accuracy_and_drift(ex, case, w, lj, tuning, lr, dt))
    if rk == 0 and ws == 1 and not args.no_cpu:
        line["cpu_baseline"] = cpu_baseline(case)
    if rk == 0:
        print(json.dumps(line), flush=True)
    barrier(dist)


if __name__ == "__main__":
    main()
