"""Seeded synthetic workloads of the midpoint LJ path, in plain numpy.

These generators load no compiled code, so the same module builds the
identical atoms for the GPU path, for the CPU timing of the oracle, and for
the parity tests.  Each case is a dict with positions (n, 3) in posn(3,n)
order (boxes concatenated), velocities, per-atom types (or None), box edges
(nboxes, 3), atoms per box, the LJ parameters and each box's target
temperature:

  liquid          FCC lattice (4 nc^3 atoms) at rho* = 0.8442 with a uniform
                  jitter (liquid-like disorder without a melt), Maxwell-
                  Boltzmann velocities, eps = sigma = m = 1, rc = 2.5 or 3.0.
  fcc             the perfect FCC lattice at T* = 0.72 (4 * 20^3 = 32,000).
  slab            uneven density: a liquid slab (rho* 0.75) in the middle
                  quarter of z of an elongated box (Lz = 4 Lx), vapour
                  (rho* 0.02) elsewhere; uniform random placement with a
                  minimum separation enforced by rejection.
  ensemble        independent cubic boxes, atom counts log-uniform in
                  [256, 16384], rho* and T* uniform, FCC or random placement
                  chosen per box.
  binary_mixture  jittered simple-cubic lattice at rho* 1.2 with an 80:20
                  A:B species split and a Kob-Andersen-type parameter table,
                  cutoff 2.5 sigma_ab per pair.

Every random choice comes from numpy's default generator seeded by the
case's seed, so a (case, size, seed) triple always gives the same atoms.

    python -m examd_gb300.workloads --case liquid --nc 64 --precision mixed --evals 3

runs `evals` force evaluations of one case on the GPU (through the library),
then `--steps` velocity-Verlet steps, and prints the pair counters; a short,
fixed launch sequence for profilers.
"""
from __future__ import annotations

import argparse
import json

import numpy as np

RHO_LIQUID = 0.8442

# Kob-Andersen-type table (A = type 0, B = type 1): eps, sigma; rc = 2.5 sigma.
KA_EPS = [[1.0, 1.5], [1.5, 0.5]]
KA_SIGMA = [[1.0, 0.8], [0.8, 0.88]]


# ---- primitives -------------------------------------------------------------
def fcc(nc, rho):
    """4 nc^3 atoms on an FCC lattice at density rho; returns (pos (n, 3), L)."""
    a = (4.0 / rho) ** (1.0 / 3.0)
    basis = np.array([[0, 0, 0], [0.5, 0.5, 0], [0.5, 0, 0.5], [0, 0.5, 0.5]])
    k, j, i = np.meshgrid(np.arange(nc), np.arange(nc), np.arange(nc), indexing="ij")
    cells = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    pos = ((cells[:, None, :] + basis[None, :, :]) * a).reshape(-1, 3)
    return np.ascontiguousarray(pos), nc * a


def velocities(n, T, rng, mass=None):
    """Maxwell-Boltzmann velocities at temperature T (k_B = 1), zero net
    momentum, kinetic temperature rescaled to exactly T over 3 (n - 1)
    degrees of freedom.  mass: per-atom masses or None (1)."""
    m = np.ones(n) if mass is None else np.asarray(mass, dtype=np.float64)
    v = rng.standard_normal((n, 3)) * np.sqrt(T / m)[:, None]
    if n == 0:
        return v
    v -= (m[:, None] * v).sum(0) / m.sum()
    ke2 = (m[:, None] * v * v).sum()
    if ke2 > 0:
        v *= np.sqrt(T * 3.0 * max(n - 1, 1) / ke2)
    return v


def random_placement(n, L, dmin, rng, lo=None, hi=None, fixed=None, max_rounds=100000):
    """n uniform random positions in [lo, hi) of a periodic box L, no two
    (nor any with the already placed `fixed` atoms) closer than dmin.

    Random sequential addition in batches: a batch of candidates is drawn,
    those within dmin of a placed atom are dropped, and of two surviving
    candidates closer than dmin the later one is dropped.  Distances are
    minimum-image (scipy's periodic k-d tree).  Returns (len(fixed) + n, 3)
    with the fixed atoms first."""
    from scipy.spatial import cKDTree
    L = np.asarray(L, dtype=np.float64).reshape(3)
    lo = np.zeros(3) if lo is None else np.asarray(lo, dtype=np.float64).reshape(3)
    hi = L.copy() if hi is None else np.asarray(hi, dtype=np.float64).reshape(3)
    placed = [np.zeros((0, 3)) if fixed is None else np.asarray(fixed, dtype=np.float64).reshape(-1, 3)]
    have = 0
    accept = 1.0
    for _ in range(max_rounds):
        if have >= n:
            break
        want = n - have
        m = int(min(max(1.5 * want / max(accept, 0.02), 256), 1 << 20))
        cand = lo + rng.random((m, 3)) * (hi - lo)
        cand = np.where(cand >= L, 0.0, cand)
        pts = np.concatenate(placed)
        if len(pts):
            d, _ = cKDTree(pts, boxsize=L).query(cand, k=1, distance_upper_bound=dmin)
            cand = cand[~(d < dmin)]
        if len(cand) > 1:
            pairs = cKDTree(cand, boxsize=L).query_pairs(dmin, output_type="ndarray")
            if len(pairs):
                drop = np.zeros(len(cand), dtype=bool)
                drop[pairs.max(axis=1)] = True  # the later candidate of each close pair
                cand = cand[~drop]
        accept = max(len(cand) / m, 1e-3)
        cand = cand[:want]
        placed.append(cand)
        have += len(cand)
    if have < n:
        raise RuntimeError(f"random placement: {have} of {n} atoms placed")
    return np.ascontiguousarray(np.concatenate(placed))


def jittered_sc(m, rho, jitter, frac_b, rng):
    """m^3 atoms on a simple-cubic lattice at density rho, each coordinate
    displaced uniformly by up to jitter * a; type 1 with probability frac_b.
    Returns (pos, types, L)."""
    a = (1.0 / rho) ** (1.0 / 3.0)
    L = m * a
    k, j, i = np.meshgrid(np.arange(m), np.arange(m), np.arange(m), indexing="ij")
    pos = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    pos = (pos + 0.5) * a + rng.uniform(-jitter * a, jitter * a, pos.shape)
    pos %= L
    types = (rng.random(m ** 3) < frac_b).astype(np.int32)
    return np.ascontiguousarray(pos), types, L


def _case(pos, vel, types, boxes, natoms, temps, **lj):
    return {"pos": np.ascontiguousarray(pos, dtype=np.float64), "vel": np.ascontiguousarray(vel, dtype=np.float64),
            "types": None if types is None else np.ascontiguousarray(types, dtype=np.int32),
            "boxes": np.atleast_2d(np.asarray(boxes, dtype=np.float64)),
            "natoms": np.atleast_1d(np.asarray(natoms, dtype=np.int64)),
            "temperatures": np.atleast_1d(np.asarray(temps, dtype=np.float64)), "lj": lj}


# ---- the configurations -----------------------------------------------------
def liquid_fcc(nc=64, rho=RHO_LIQUID, T=1.0, jitter=0.15, rc=2.5, seed=1):
    rng = np.random.default_rng(seed)
    pos, L = fcc(nc, rho)
    pos = (pos + rng.uniform(-jitter, jitter, pos.shape)) % L
    vel = velocities(len(pos), T, rng)
    return _case(pos, vel, None, [L, L, L], [len(pos)], [T], rc=rc)


def fcc_lattice(nc=20, rho=RHO_LIQUID, T=0.72, rc=2.5, seed=1):
    rng = np.random.default_rng(seed)
    pos, L = fcc(nc, rho)
    vel = velocities(len(pos), T, rng)
    return _case(pos, vel, None, [L, L, L], [len(pos)], [T], rc=rc)


def slab(n=524288, rho_liq=0.75, rho_vap=0.02, T=0.85, rc=3.0, dmin=0.8, seed=3):
    """Lx = Ly, Lz = 4 Lx; liquid in z in [3Lz/8, 5Lz/8), vapour elsewhere."""
    rng = np.random.default_rng(seed)
    # n = Lx^2 Lz (rho_liq/4 + rho_vap 3/4) with Lz = 4 Lx
    lx = (n / (4.0 * (rho_liq / 4.0 + 0.75 * rho_vap))) ** (1.0 / 3.0)
    L = np.array([lx, lx, 4.0 * lx])
    v_liq = lx * lx * L[2] / 4.0
    n_liq = int(round(n * rho_liq * v_liq / (rho_liq * v_liq + rho_vap * 3.0 * v_liq)))
    n_lo = (n - n_liq) // 2
    n_hi = n - n_liq - n_lo
    z0, z1 = 3.0 * L[2] / 8.0, 5.0 * L[2] / 8.0
    pos = random_placement(n_liq, L, dmin, rng, lo=[0, 0, z0], hi=[lx, lx, z1])
    pos = random_placement(n_lo, L, dmin, rng, lo=[0, 0, 0], hi=[lx, lx, z0], fixed=pos)
    pos = random_placement(n_hi, L, dmin, rng, lo=[0, 0, z1], hi=[lx, lx, L[2]], fixed=pos)
    vel = velocities(n, T, rng)
    return _case(pos, vel, None, L, [n], [T], rc=rc)


def ensemble(nboxes=512, nmin=256, nmax=16384, rho=(0.3, 0.9), T=(0.7, 1.5), rc=2.5, dmin=0.8, seed=4):
    """Independent cubic boxes; FCC boxes round the count to 4 k^3."""
    rng = np.random.default_rng(seed)
    pos_all, vel_all, boxes, counts, temps = [], [], [], [], []
    for _ in range(nboxes):
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        r = float(rng.uniform(*rho))
        t = float(rng.uniform(*T))
        if rng.random() < 0.5:
            k = max(2, int(round((n / 4.0) ** (1.0 / 3.0))))
            p, L = fcc(k, r)
            n = len(p)
        else:
            L = (n / r) ** (1.0 / 3.0)
            p = random_placement(n, [L, L, L], dmin, rng)
        pos_all.append(p)
        vel_all.append(velocities(n, t, rng))
        boxes.append([L, L, L])
        counts.append(n)
        temps.append(t)
    return _case(np.concatenate(pos_all), np.concatenate(vel_all), None, boxes, counts, temps, rc=rc)


def binary_mixture(m=256, rho=1.2, T=1.0, jitter=0.1, frac_b=0.2, seed=5):
    rng = np.random.default_rng(seed)
    pos, types, L = jittered_sc(m, rho, jitter, frac_b, rng)
    vel = velocities(len(pos), T, rng)
    rc = (2.5 * np.asarray(KA_SIGMA)).tolist()
    return _case(pos, vel, types, [L, L, L], [len(pos)], [T], ntypes=2, eps=KA_EPS, sigma=KA_SIGMA, rc=rc)


CASES = {"liquid": liquid_fcc, "fcc": fcc_lattice, "slab": slab, "ensemble": ensemble,
         "binary_mixture": binary_mixture}


def system(case, precision="mixed", **kw):
    """A MidpointLJ (the GPU library) holding the case's atoms."""
    from . import api as _api
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
    ap.add_argument("--pair-skin", type=float, default=0.0, help="mixed form's pair-list skin (0: none)")
    a = ap.parse_args(argv)
    kw = {"liquid": {"nc": a.nc}, "fcc": {}, "slab": {"n": a.n}, "ensemble": {"nboxes": a.nboxes},
          "binary_mixture": {"m": a.m}}[a.case]
    case = CASES[a.case](**kw)
    tile = None if a.tile is None else (a.tile * 3 if len(a.tile) == 1 else a.tile)
    if tile is not None and len(tile) != 3:
        ap.error("--tile takes one edge or three")
    with system(case, a.precision, tile=tile, tile_balance=a.tile_balance, pair_skin=a.pair_skin) as s:
        for _ in range(a.evals):
            s.forces()
        cnt = s.counters()
        if a.steps:
            s.run(a.steps, 0.005)
    print(json.dumps({"case": a.case, "atoms": int(case["natoms"].sum()), "boxes": len(case["natoms"]),
                      "precision": a.precision, "evals": a.evals, **cnt}))


if __name__ == "__main__":
    main()
