"""Host-side interface of the GB300 midpoint Lennard-Jones path.

Mirrors the reference's force interface (SRC/exaMD_forces.f90:308-318):
``forces_midpoint_all(pos, box, cutoff, ...)`` is the counterpart of
``Call exaMD_forces_midpoint_all(lennardjones_12, cutoff, noprocs)`` with the
module state (blocks, globalbox, prmvdw) passed explicitly, and, like the
reference, accumulates into a caller-supplied force array.  ``MidpointLJ``
keeps the atoms resident on the GPU for repeated calls, velocity-Verlet runs
and batched ensembles.  Everything goes through the C ABI of
``include/examd_gb300.h``; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
import weakref

import numpy as np

from . import _lib as _L
from ._lib import ExamdError, check

__all__ = ["MidpointLJ", "forces_midpoint_all", "gen_fcc", "gen_velocities", "gen_random", "gen_jittered_sc",
           "pinned_empty", "own_table", "tile_split", "ExamdError", "FP64", "MIXED"]

FP64 = "fp64"
MIXED = "mixed"


def _d(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


def _table(v, nt):
    a = np.asarray(v, dtype=np.float64)
    if a.ndim == 0:
        a = np.full((nt, nt), float(a))
    return np.ascontiguousarray(a.reshape(nt, nt))


POTENTIALS = {"lj": _L.POT_LJ, "lj_shifted": _L.POT_LJ_SHIFTED, "wca": _L.POT_WCA}
PAIR_TABLES = {"auto": 0, "wide": 1, "compact": 2}


def _setup(boxes, natoms, precision=FP64, eps=1.0, sigma=1.0, rc=2.5, ntypes=1, mass=None, block_length=None,
           tile=None, warps=None, strict_box=False, device=0, potential="lj", pair_tables="auto",
           tile_balance=0, pair_skin=0.0, pair_list_capacity=0):
    """examd_params and the examd_box array of a system, from Python arguments."""
    lib = _L.load()
    b = np.atleast_2d(np.asarray(boxes, dtype=np.float64))
    n = np.atleast_1d(np.asarray(natoms, dtype=np.int64))
    if b.shape[1] != 3 or b.shape[0] != n.shape[0]:
        raise ValueError("boxes must be (nboxes, 3) with one natoms per box")
    if precision not in (FP64, MIXED):
        raise ValueError("precision must be 'fp64' or 'mixed'")
    p = _L.Params()
    lib.examd_default_params(C.byref(p))
    p.precision = _L.FP64 if precision == FP64 else _L.MIXED
    p.ntypes = int(ntypes)
    e, s, r = _table(eps, ntypes), _table(sigma, ntypes), _table(rc, ntypes)
    for k in range(ntypes * ntypes):
        p.eps[k] = e.flat[k]
        p.sigma[k] = s.flat[k]
        p.rc[k] = r.flat[k]
    m = np.ones(ntypes) if mass is None else np.broadcast_to(np.asarray(mass, dtype=np.float64), (ntypes,))
    for k in range(ntypes):
        p.mass[k] = m[k]
    p.cell_edge = 0.0 if block_length is None else float(block_length)
    if tile is not None:
        for a in range(3):
            p.tile[a] = int(tile[a] if np.ndim(tile) else tile)
    p.warps = 0 if warps is None else int(warps)
    p.strict_box = 1 if strict_box else 0
    p.device = int(device)
    if potential not in POTENTIALS:
        raise ValueError(f"potential must be one of {sorted(POTENTIALS)}")
    p.potential = POTENTIALS[potential]
    if pair_tables not in PAIR_TABLES:
        raise ValueError(f"pair_tables must be one of {sorted(PAIR_TABLES)}")
    p.pair_tables = PAIR_TABLES[pair_tables]
    if tile_balance not in (0, 1):
        raise ValueError("tile_balance must be 0 (split by cell count) or 1 (by width)")
    p.tile_balance = int(tile_balance)
    p.pair_skin = float(pair_skin)
    p.pair_list_capacity = int(pair_list_capacity)
    arr = (_L.Box * b.shape[0])()
    for k in range(b.shape[0]):
        for a in range(3):
            arr[k].L[a] = b[k, a]
        arr[k].natoms = int(n[k])
    return lib, p, arr, b, n, np.array(m, dtype=np.float64)


def autotune(boxes, natoms, pos, types=None, cache=None, **kw):
    """Cell edge, tile shape, warps per CTA and tile split for this system,
    picked by timing the pair kernel on these atoms (examd_autotune).  cache:
    path of a text cache of earlier choices, or None.  Returns dict(tile,
    warps, tile_balance, block_length (None: the reference's rc/2), ms per
    launch); the first four are MidpointLJ keyword arguments."""
    lib, p, arr, b, n, _ = _setup(boxes, natoms, **kw)
    pp = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
    best = _L.Params()
    ms = C.c_double()
    path = None if cache is None else os.fsencode(cache)
    check(lib.examd_autotune(C.byref(p), len(n), arr, len(pp), _d(pp), _i(t), path, C.byref(best), C.byref(ms)),
          "examd_autotune")
    return {"tile": tuple(int(v) for v in best.tile), "warps": int(best.warps),
            "tile_balance": int(best.tile_balance),
            "block_length": float(best.cell_edge) if best.cell_edge > 0 else None, "ms": ms.value}


class MidpointLJ:
    """Resident GPU state for one box or a batch of independent boxes.

    boxes: (nboxes, 3) box edges (or one 3-vector); natoms: atoms per box.
    precision: "fp64" (FP64 end to end) or "mixed" (FP32 pair forces, FP64
    positions, integration and reductions).  eps/sigma/rc: scalars or
    (ntypes, ntypes) tables; block_length defaults to max(rc)/2 as the
    reference (exaMD.f90:56).  potential: the pair function, "lj" (the
    reference's lennardjones_12), "lj_shifted" or "wca".  pair_tables: the
    mixed form's per-warp tables, "auto" (compact where that fits more CTAs
    on an SM), "wide" or "compact"; the forces are the same bit for bit.
    tile_balance: 0 splits each axis into tiles by cell count, 1 by width (the
    wide last cell that absorbs the box's remainder counts as two).
    pair_skin: 0 (the reference's schedule: cells and candidate pairs at
    every evaluation) or, mixed form, the skin of the per-tile pair lists
    (rebuilt when an atom has moved more than half of it); pair_list_capacity:
    list entries per atom (0: sized by the library)."""

    def __init__(self, boxes, natoms, *, precision=FP64, eps=1.0, sigma=1.0, rc=2.5, ntypes=1, mass=None,
                 block_length=None, tile=None, warps=None, strict_box=False, device=0, potential="lj",
                 pair_tables="auto", tile_balance=0, pair_skin=0.0, pair_list_capacity=0):
        lib, p, arr, b, n, m = _setup(boxes, natoms, precision, eps, sigma, rc, ntypes, mass, block_length, tile,
                                      warps, strict_box, device, potential, pair_tables, tile_balance, pair_skin,
                                      pair_list_capacity)
        self._lib = lib
        self.nboxes = int(b.shape[0])
        self.natoms = n.copy()
        self.n = int(n.sum())
        self.box_edges = b.copy()
        self.precision = precision
        self.mass = m
        self.params = p
        ctx = C.c_void_p()
        check(lib.examd_gpu_create(C.byref(p), self.nboxes, arr, C.byref(ctx)), "examd_gpu_create")
        self._ctx = ctx
        self._fin = weakref.finalize(self, lib.examd_gpu_destroy, ctx)
        self.types = None
        self.tuning = None

    @classmethod
    def tuned(cls, boxes, natoms, pos, types=None, vel=None, cache=None, **kw):
        """A system whose tile shape, CTA width and tile split the autotuner picked for these atoms."""
        r = autotune(boxes, natoms, pos, types, cache, **kw)
        kw = dict(kw, tile=r["tile"], warps=r["warps"], tile_balance=r["tile_balance"],
                  block_length=r["block_length"])
        s = cls(boxes, natoms, **kw)
        s.set_atoms(pos, types, vel)
        s.tuning = r
        return s

    # -- lifecycle -----------------------------------------------------------
    def close(self):
        if self._fin.alive:
            self._fin()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _chk(self, code, where):
        check(code, where, self._ctx)

    # -- atoms ---------------------------------------------------------------
    def set_atoms(self, pos, types=None, vel=None):
        """pos: (n, 3) in posn(3,n) order, boxes concatenated."""
        p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
        if p.shape[0] != self.n:
            raise ValueError(f"expected {self.n} atoms, got {p.shape[0]}")
        t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
        v = None if vel is None else np.ascontiguousarray(vel, dtype=np.float64).reshape(-1, 3)
        self.types = t
        self._chk(self._lib.examd_gpu_set_atoms(self._ctx, self.n, _d(p), _i(t), _d(v)), "examd_gpu_set_atoms")

    def forces(self, out=None, accumulate=False, energy=False):
        """One force evaluation at the resident positions.

        Returns (forces (n,3), epot per box, virial per box); epot/virial are
        None unless energy=True.  With accumulate=True the forces are added to
        ``out`` (the reference's += semantics)."""
        f = out if out is not None else np.zeros((self.n, 3))
        if f.dtype != np.float64 or not f.flags.c_contiguous or f.shape != (self.n, 3):
            raise ValueError("out must be a C-contiguous (n, 3) float64 array")
        ep = np.zeros(self.nboxes) if energy else None
        w = np.zeros(self.nboxes) if energy else None
        self._chk(self._lib.examd_gpu_forces(self._ctx, _d(f), _d(ep), _d(w), 1 if accumulate else 0),
                  "examd_gpu_forces")
        return f, ep, w

    def forces_at(self, pos, out=None, accumulate=False, energy=False):
        """New positions (same atoms, caller order) and one force evaluation.

        With pos and out in pinned memory (pinned_empty) the library replays the
        call as a captured CUDA graph from the second call with the same arrays;
        the energies then land in pinned arrays of this object and are copied."""
        p = pos if (isinstance(pos, np.ndarray) and pos.dtype == np.float64 and pos.flags.c_contiguous) \
            else np.ascontiguousarray(pos, dtype=np.float64)
        f = out if out is not None else np.zeros((self.n, 3))
        ep = w = None
        if energy:
            if getattr(self, "_pinned_ew", None) is None:
                self._pinned_ew = (pinned_empty((self.nboxes,)), pinned_empty((self.nboxes,)))
            ep, w = self._pinned_ew
        self._chk(self._lib.examd_gpu_forces_at(self._ctx, _d(p), _d(f), _d(ep), _d(w), 1 if accumulate else 0),
                  "examd_gpu_forces_at")
        return f, (ep.copy() if energy else None), (w.copy() if energy else None)

    def run(self, nsteps, dt, graph_chunk=0, energies=False):
        """Velocity-Verlet steps.  Returns dict(ms, ekin[steps, boxes], epot[steps, boxes])."""
        en = np.zeros((max(nsteps, 1), self.nboxes, 2)) if energies else None
        st = _L.Stats()
        self._chk(self._lib.examd_gpu_run(self._ctx, int(nsteps), float(dt), int(graph_chunk), _d(en),
                                          C.byref(st)), "examd_gpu_run")
        out = dict(ms=st.ms, steps=st.steps)
        if energies:
            out["ekin"] = en[:nsteps, :, 0].copy()
            out["epot"] = en[:nsteps, :, 1].copy()
        return out

    def prepare_run(self, dt, graph_chunk, energies=False):
        """Capture the step-loop graph that run(nsteps, dt, graph_chunk, energies)
        replays, without running a step (keeps capture out of a timed run)."""
        self._chk(self._lib.examd_gpu_prepare_run(self._ctx, float(dt), int(graph_chunk), 1 if energies else 0),
                  "examd_gpu_prepare_run")

    def time_phases(self, nsteps, dt):
        """Average device ms per step over nsteps eager steps of: the kick with drift (and the binning count,
        or in pair-list mode the offsets and displacement since the build); the binning's scan and scatter
        (pair-list mode: the rebuild decision and the rebuilds of the steps that had one); the pair kernels.
        Advances the state (timing only)."""
        ms = np.zeros(3)
        self._chk(self._lib.examd_gpu_time_phases(self._ctx, int(nsteps), float(dt), _d(ms)), "examd_gpu_time_phases")
        return {"kick": float(ms[0]), "binning": float(ms[1]), "pair": float(ms[2])}

    def time_rebuild(self, reps=3):
        """Pair-list mode: device ms of one rebuild of the cells and lists at the current positions."""
        ms = C.c_double()
        self._chk(self._lib.examd_gpu_time_rebuild(self._ctx, int(reps), C.byref(ms)), "examd_gpu_time_rebuild")
        return ms.value

    def list_info(self):
        """Pair-list mode: builds so far, list entries per atom, the most entries of one atom at the builds
        since the last call and the tiles computed by enumeration (zeros without pair lists)."""
        b = C.c_int64()
        c, l, f = C.c_int(), C.c_int(), C.c_int()
        self._chk(self._lib.examd_gpu_list_info(self._ctx, C.byref(b), C.byref(c), C.byref(l), C.byref(f)),
                  "examd_gpu_list_info")
        return {"builds": b.value, "capacity": c.value, "longest": l.value, "fallback_tiles": f.value}

    def state(self):
        pos = np.zeros((self.n, 3))
        vel = np.zeros((self.n, 3))
        self._chk(self._lib.examd_gpu_get_state(self._ctx, _d(pos), _d(vel)), "examd_gpu_get_state")
        return pos, vel

    def kinetic(self):
        ek = np.zeros(self.nboxes)
        self._chk(self._lib.examd_gpu_kinetic(self._ctx, _d(ek)), "examd_gpu_kinetic")
        return ek

    def scale_velocities(self, factor):
        f = np.ascontiguousarray(np.broadcast_to(np.asarray(factor, dtype=np.float64), (self.nboxes,)))
        self._chk(self._lib.examd_gpu_scale_velocities(self._ctx, _d(f)), "examd_gpu_scale_velocities")

    def time_forces(self, reps):
        """Device time (ms) of `reps` pair-kernel launches on the context stream; returns (total, per launch)."""
        ms = C.c_double()
        kms = C.c_double()
        self._chk(self._lib.examd_gpu_time_forces(self._ctx, int(reps), C.byref(ms), C.byref(kms)),
                  "examd_gpu_time_forces")
        return ms.value, kms.value

    def counters(self):
        c, a, e, t, m = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        self._chk(self._lib.examd_gpu_counters(self._ctx, C.byref(c), C.byref(a), C.byref(e), C.byref(t),
                                               C.byref(m)), "examd_gpu_counters")
        return dict(candidates=c.value, accepted=a.value, evaluated=e.value, tiles=t.value,
                    max_tile_atoms=m.value)


def forces_midpoint_all(pos, box, cutoff, eps=1.0, sigma=1.0, forces=None, precision=FP64, energy=False, **kw):
    """One midpoint LJ force evaluation on the GPU for a single periodic box.

    Counterpart of exaMD_forces_midpoint_all(lennardjones_12, cutoff, noprocs=1)
    (SRC/exaMD_forces.f90:308-390) with prmvdw(1,:) = (eps, sigma, -, -, cutoff)
    (exaMD.f90:199-202).  ``forces`` when given is accumulated into (+=), as the
    reference accumulates into grid%forces.  Returns forces, or
    (forces, epot, virial) when energy=True."""
    p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    with MidpointLJ(np.asarray(box, dtype=np.float64).reshape(1, 3), [p.shape[0]], precision=precision, eps=eps,
                    sigma=sigma, rc=cutoff, **kw) as sysm:
        sysm.set_atoms(p)
        if forces is None:
            f, ep, w = sysm.forces(energy=energy)
        else:
            f, ep, w = sysm.forces(out=forces, accumulate=True, energy=energy)
    return (f, float(ep[0]), float(w[0])) if energy else f


# -- generators (host code in the library) ------------------------------------
def read_particles(path):
    """Atoms of an exaMD_particles.dat file (SRC/exaMD_input_formats.f90:128-192): (pos (n, 3), L (3,))."""
    lib = _L.load()
    n = C.c_int64()
    L = np.zeros(3)
    p = os.fsencode(path)
    check(lib.examd_read_particles(p, C.byref(n), _d(L), None, 0), "examd_read_particles", detail=str(path))
    pos = np.zeros((n.value, 3))
    check(lib.examd_read_particles(p, C.byref(n), _d(L), _d(pos), n.value), "examd_read_particles",
          detail=str(path))
    return pos, L


def write_particles(path, pos, L):
    """Write atoms in the exaMD_particles.dat format (exaMD_write_particles, :211-235)."""
    lib = _L.load()
    p = np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)
    box = np.ascontiguousarray(np.broadcast_to(np.asarray(L, dtype=np.float64), (3,)))
    check(lib.examd_write_particles(os.fsencode(path), len(p), _d(box), _d(p)), "examd_write_particles",
          detail=str(path))


def gen_fcc(nc, rho):
    """4*nc^3 atoms on an FCC lattice at density rho; returns (pos (n,3), L)."""
    lib = _L.load()
    pos = np.zeros((4 * nc ** 3, 3))
    L = C.c_double()
    check(lib.examd_gen_fcc(int(nc), float(rho), _d(pos), C.byref(L)), "examd_gen_fcc")
    return pos, L.value


def gen_velocities(n, T, seed, types=None, mass=None):
    lib = _L.load()
    v = np.zeros((n, 3))
    t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
    m = None if mass is None else np.ascontiguousarray(mass, dtype=np.float64)
    check(lib.examd_gen_velocities(int(n), _i(t), _d(m), float(T), C.c_uint64(seed), _d(v)), "examd_gen_velocities")
    return v


def gen_random(n, L, dmin, seed, lo=None, hi=None, fixed=None, max_tries=100000):
    """Uniform random positions with minimum separation dmin (periodic).  ``fixed``:
    already placed atoms kept in front; lo/hi: the region to fill."""
    lib = _L.load()
    L = np.asarray(L, dtype=np.float64).reshape(3)
    lo = np.zeros(3) if lo is None else np.asarray(lo, dtype=np.float64).reshape(3)
    hi = L.copy() if hi is None else np.asarray(hi, dtype=np.float64).reshape(3)
    nf = 0 if fixed is None else len(fixed)
    pos = np.zeros((nf + n, 3))
    if nf:
        pos[:nf] = fixed
    check(lib.examd_gen_random(nf + n, nf, _d(np.ascontiguousarray(L)), _d(np.ascontiguousarray(lo)),
                               _d(np.ascontiguousarray(hi)), float(dmin), C.c_uint64(seed), int(max_tries), _d(pos)),
          "examd_gen_random")
    return pos


def gen_jittered_sc(m, rho, jitter, frac_b, seed):
    lib = _L.load()
    pos = np.zeros((m ** 3, 3))
    t = np.zeros(m ** 3, dtype=np.int32)
    L = C.c_double()
    check(lib.examd_gen_jittered_sc(int(m), float(rho), float(jitter), float(frac_b), C.c_uint64(seed), _d(pos),
                                    _i(t), C.byref(L)), "examd_gen_jittered_sc")
    return pos, t, L.value


def own_table():
    """(rows (13,2), lut (125,13)) derived by the library from the 63-entry table."""
    lib = _L.load()
    rows = (C.c_byte * 26)()
    lut = (C.c_ubyte * (125 * 13))()
    check(lib.examd_own_table(rows, lut), "examd_own_table")
    return (np.frombuffer(bytes(rows), dtype=np.int8).reshape(13, 2).copy(),
            np.frombuffer(bytes(lut), dtype=np.uint8).reshape(125, 13).copy())


def tile_split(nb, last_width, tile_len, tile_balance=0):
    """Tile starts along one axis of nb cells, as examd_gpu_create splits it
    (examd_tile_split): nt + 1 ints, the last one nb."""
    lib = _L.load()
    starts = (C.c_int * (nb // 2 + 2))()
    nt = C.c_int()
    check(lib.examd_tile_split(int(nb), float(last_width), int(tile_len), int(tile_balance), starts, C.byref(nt)),
          "examd_tile_split")
    return np.array(starts[:nt.value + 1], dtype=np.int64)


def pinned_empty(shape, dtype=np.float64):
    """numpy array in page-locked host memory (cudaHostAlloc), freed with the array."""
    lib = _L.load()
    n = int(np.prod(shape)) * np.dtype(dtype).itemsize
    ptr = C.c_void_p()
    check(lib.examd_host_alloc(C.byref(ptr), n), "examd_host_alloc")
    buf = (C.c_byte * n).from_address(ptr.value)
    arr = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)
    weakref.finalize(buf, lib.examd_host_free, ptr)
    arr.flags.writeable = True
    return arr
