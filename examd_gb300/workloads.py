"""Seeded synthetic workloads of the midpoint LJ path, and a small runner.

Each generator returns a dict with positions (n, 3) in posn(3,n) order (boxes
concatenated), velocities, per-atom types, box edges (nboxes, 3), atoms per
box and the LJ parameters of the case:

  liquid_fcc     FCC lattice (4 nc^3 atoms) at rho* = 0.8442, uniformly
                 jittered (a liquid-like stand-in for a melted lattice),
                 Maxwell-Boltzmann velocities, eps = sigma = m = 1.
  slab           uneven density: liquid slab (rho* 0.75) in the middle quarter
                 of z of an elongated box (Lz = 4 Lx), vapour (rho* 0.02)
                 elsewhere; uniform random placement with a minimum separation
                 enforced by rejection.
  ensemble       many independent cubic boxes, atom counts log-uniform in
                 [256, 16384], rho* and T* uniform, FCC or random placement
                 chosen per box.
  binary_mixture jittered simple-cubic lattice at rho* 1.2 with an 80:20
                 A:B species split and a Kob-Andersen-type parameter table,
                 cutoff 2.5 sigma_ab per pair.

    python -m examd_gb300.workloads --case liquid --nc 64 --precision mixed --evals 3

runs `evals` force evaluations of one case on the GPU, then `--steps`
velocity-Verlet steps (a short, fixed launch sequence for profilers), and
prints the pair counters.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import api as _api


def _case(pos, vel, types, boxes, natoms, **lj):
    return {"pos": np.ascontiguousarray(pos, dtype=np.float64), "vel": np.ascontiguousarray(vel, dtype=np.float64),
            "types": None if types is None else np.ascontiguousarray(types, dtype=np.int32),
            "boxes": np.atleast_2d(np.asarray(boxes, dtype=np.float64)),
            "natoms": np.atleast_1d(np.asarray(natoms, dtype=np.int64)), "lj": lj}


def liquid_fcc(nc=64, rho=0.8442, T=1.0, jitter=0.15, rc=2.5, seed=1):
    pos, L = _api.gen_fcc(nc, rho)
    rng = np.random.default_rng(seed)
    pos = (pos + rng.uniform(-jitter, jitter, pos.shape)) % L
    vel = _api.gen_velocities(len(pos), T, seed)
    return _case(pos, vel, None, [L, L, L], [len(pos)], rc=rc)


def slab(n=524288, rho_liq=0.75, rho_vap=0.02, T=0.85, rc=3.0, dmin=0.8, seed=3):
    """Lx = Ly, Lz = 4 Lx; liquid in z in [3Lz/8, 5Lz/8), vapour elsewhere."""
    # n = Lx^2 Lz (rho_liq/4 + rho_vap 3/4) with Lz = 4 Lx
    lx = (n / (4.0 * (rho_liq / 4.0 + 0.75 * rho_vap))) ** (1.0 / 3.0)
    L = np.array([lx, lx, 4.0 * lx])
    v_liq = lx * lx * L[2] / 4.0
    n_liq = int(round(n * rho_liq * v_liq / (rho_liq * v_liq + rho_vap * 3.0 * v_liq)))
    n_lo = (n - n_liq) // 2
    n_hi = n - n_liq - n_lo
    z0, z1 = 3.0 * L[2] / 8.0, 5.0 * L[2] / 8.0
    pos = _api.gen_random(n_liq, L, dmin, seed, lo=[0, 0, z0], hi=[lx, lx, z1])
    pos = _api.gen_random(n_lo, L, dmin, seed + 1, lo=[0, 0, 0], hi=[lx, lx, z0], fixed=pos)
    pos = _api.gen_random(n_hi, L, dmin, seed + 2, lo=[0, 0, z1], hi=[lx, lx, L[2]], fixed=pos)
    vel = _api.gen_velocities(n, T, seed)
    return _case(pos, vel, None, L, [n], rc=rc)


def ensemble(nboxes=512, nmin=256, nmax=16384, rho=(0.3, 0.9), T=(0.7, 1.5), rc=2.5, dmin=0.8, seed=4):
    """Independent cubic boxes; FCC boxes round the count to 4 k^3."""
    rng = np.random.default_rng(seed)
    pos_all, vel_all, boxes, counts, temps = [], [], [], [], []
    for b in range(nboxes):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        r = float(rng.uniform(*rho))
        t = float(rng.uniform(*T))
        if rng.random() < 0.5:
            k = max(2, int(round((n / 4.0) ** (1.0 / 3.0))))
            p, L = _api.gen_fcc(k, r)
            n = len(p)
        else:
            L = (n / r) ** (1.0 / 3.0)
            p = _api.gen_random(n, [L, L, L], dmin, seed * 100003 + b)
        pos_all.append(p)
        vel_all.append(_api.gen_velocities(n, t, seed * 7919 + b))
        boxes.append([L, L, L])
        counts.append(n)
        temps.append(t)
    c = _case(np.concatenate(pos_all), np.concatenate(vel_all), None, boxes, counts, rc=rc)
    c["temperatures"] = np.array(temps)
    return c


# Kob-Andersen-type table (A = type 0, B = type 1): eps, sigma; rc = 2.5 sigma.
KA_EPS = [[1.0, 1.5], [1.5, 0.5]]
KA_SIGMA = [[1.0, 0.8], [0.8, 0.88]]


def binary_mixture(m=256, rho=1.2, T=1.0, jitter=0.1, frac_b=0.2, seed=5):
    pos, types, L = _api.gen_jittered_sc(m, rho, jitter, frac_b, seed)
    vel = _api.gen_velocities(len(pos), T, seed, types=types, mass=[1.0, 1.0])
    rc = (2.5 * np.asarray(KA_SIGMA)).tolist()
    return _case(pos, vel, types, [L, L, L], [len(pos)], ntypes=2, eps=KA_EPS, sigma=KA_SIGMA, rc=rc)


CASES = {"liquid": liquid_fcc, "slab": slab, "ensemble": ensemble, "binary_mixture": binary_mixture}


def system(case, precision="mixed", **kw):
    """A MidpointLJ holding the case's atoms."""
    lj = dict(case["lj"])
    s = _api.MidpointLJ(case["boxes"], case["natoms"], precision=precision, **lj, **kw)
    s.set_atoms(case["pos"], case["types"], case["vel"])
    return s


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--case", default="liquid", choices=sorted(CASES))
    ap.add_argument("--nc", type=int, default=64, help="liquid: FCC cells per edge")
    ap.add_argument("--m", type=int, default=256, help="binary_mixture: lattice sites per edge")
    ap.add_argument("--n", type=int, default=524288, help="slab: atoms")
    ap.add_argument("--nboxes", type=int, default=512, help="ensemble: boxes")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    ap.add_argument("--evals", type=int, default=3)
    ap.add_argument("--steps", type=int, default=0, help="then this many velocity-Verlet steps (dt 0.005)")
    ap.add_argument("--tile", type=int, nargs="+", default=None, help="tile edge, or edges per axis")
    ap.add_argument("--tile-balance", type=int, default=0, choices=[0, 1],
                    help="split of each axis into tiles: 0 by cell count, 1 by width")
    a = ap.parse_args(argv)
    kw = {"liquid": {"nc": a.nc}, "slab": {"n": a.n}, "ensemble": {"nboxes": a.nboxes},
          "binary_mixture": {"m": a.m}}[a.case]
    case = CASES[a.case](**kw)
    tile = None if a.tile is None else (a.tile * 3 if len(a.tile) == 1 else a.tile)
    if tile is not None and len(tile) != 3:
        ap.error("--tile takes one edge or three")
    with system(case, a.precision, tile=tile, tile_balance=a.tile_balance) as s:
        for _ in range(a.evals):
            s.forces()
        cnt = s.counters()
        if a.steps:
            s.run(a.steps, 0.005)
    print(json.dumps({"case": a.case, "atoms": int(case["natoms"].sum()), "boxes": len(case["natoms"]),
                      "precision": a.precision, "evals": a.evals, **cnt}))


if __name__ == "__main__":
    main()
