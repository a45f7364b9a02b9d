"""ctypes front end of the CPU oracle (oracle/examd_oracle*.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` as
the checker and by ``bench.py``'s cpu_baseline leg and reference arm.  The
product package ``examd_gb300`` never imports this module.

Parity status: unpinned against the reference binary (the reference has no
tests or golden vectors and its Fortran cannot be compiled here); the oracle
is pinned by analytic known-answer tests and by an independent O(N^2) sum.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_SO = os.path.join(_HERE, "_build", "libexamd_oracle.so")
_lock = threading.Lock()
_lib = None

ERR_OUTSIDE = 109
ERR_NB_TOO_SMALL = 201


class Counts(C.Structure):
    _fields_ = [("candidates", C.c_int64), ("accepted", C.c_int64), ("zero_d2", C.c_int64)]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, -ffp-contract=off)."""
    srcs = [os.path.join(_HERE, f) for f in ("examd_oracle.c", "examd_oracle_ext.c", "examd_oracle.h")]
    if force or not os.path.exists(_SO) or any(os.path.getmtime(s) > os.path.getmtime(_SO) for s in srcs):
        subprocess.run(["make", "-s", "-C", _HERE, "-B" if force else "all"], check=True)
    return _SO


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            L = C.CDLL(_SO)
            dp = C.POINTER(C.c_double)
            ip = C.POINTER(C.c_int)
            L.exo_forces_midpoint_all.argtypes = [C.c_int64, dp, dp, C.c_double, C.c_double, C.c_double,
                                                  C.c_double, dp, C.POINTER(Counts)]
            L.exo_forces_typed.argtypes = [C.c_int64, dp, ip, dp, C.c_double, C.c_int, dp, dp, dp, dp, dp, dp, dp,
                                           C.POINTER(Counts)]
            L.exo_forces_typed_omp.argtypes = [C.c_int64, dp, ip, dp, C.c_double, C.c_int, dp, dp, dp, dp, dp, dp,
                                               C.c_int, C.POINTER(Counts)]
            L.exo_forces_bruteforce.argtypes = [C.c_int64, dp, ip, dp, C.c_int, dp, dp, dp, dp, dp, dp]
            L.exo_vv_run.argtypes = [C.c_int64, dp, dp, ip, dp, dp, C.c_double, C.c_int, dp, dp, dp, C.c_double,
                                     C.c_int, C.c_int, dp, dp]
            L.exo_identify_block.argtypes = [dp, C.c_double, ip, ip]
            L.exo_domain_create.argtypes = [dp, C.c_double, ip]
            L.exo_midpoint_table.argtypes = [ip]
            L.exo_wrap.argtypes = [C.c_double, C.c_double, C.c_double]
            L.exo_wrap.restype = C.c_double
            _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _i(a):
    return a.ctypes.data_as(C.POINTER(C.c_int))


def _pos(pos):
    return np.ascontiguousarray(pos, dtype=np.float64).reshape(-1, 3)


def midpoint_table() -> np.ndarray:
    out = np.zeros(126, dtype=np.int32)
    lib().exo_midpoint_table(_i(out))
    return out.reshape(63, 2)


def domain_create(box, block_length):
    nb = np.zeros(3, dtype=np.int32)
    lib().exo_domain_create(_d(np.asarray(box, dtype=np.float64)), block_length, _i(nb))
    return nb


def forces_midpoint_all(pos, box, cutoff, eps=1.0, sigma=1.0, block_length=None, forces=None):
    """Restated exaMD_forces_midpoint_all (single species, no energy).

    Returns (forces (n,3), Counts).  ``forces`` when given is accumulated into,
    as the reference does."""
    p = _pos(pos)
    n = p.shape[0]
    f = np.zeros((n, 3)) if forces is None else forces
    assert f.dtype == np.float64 and f.flags.c_contiguous
    bl = 0.5 * cutoff if block_length is None else block_length
    cnt = Counts()
    rc = lib().exo_forces_midpoint_all(n, _d(p), _d(np.asarray(box, dtype=np.float64)), bl, eps, sigma, cutoff,
                                       _d(f), C.byref(cnt))
    if rc != 0:
        raise OracleError(rc)
    return f, cnt


class OracleError(RuntimeError):
    def __init__(self, code):
        super().__init__(f"oracle error {code}")
        self.code = code


def _tables(ntypes, eps, sigma, rc):
    e = np.ascontiguousarray(np.broadcast_to(np.asarray(eps, dtype=np.float64), (ntypes, ntypes)))
    s = np.ascontiguousarray(np.broadcast_to(np.asarray(sigma, dtype=np.float64), (ntypes, ntypes)))
    r = np.ascontiguousarray(np.broadcast_to(np.asarray(rc, dtype=np.float64), (ntypes, ntypes)))
    return e, s, r


def forces_typed(pos, box, rc, eps=1.0, sigma=1.0, types=None, ntypes=1, block_length=None, threads=1,
                 want_virial9=False):
    """Typed LJ with energy and virial over the reference's block loops.

    Returns dict(forces, epot, virial, counts[, virial9])."""
    p = _pos(pos)
    n = p.shape[0]
    e, s, r = _tables(ntypes, eps, sigma, rc)
    bl = 0.5 * float(r.max()) if block_length is None else block_length
    t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
    f = np.zeros((n, 3))
    ep = C.c_double()
    w = C.c_double()
    cnt = Counts()
    box = np.asarray(box, dtype=np.float64)
    tp = _i(t) if t is not None else None
    if threads == 1:
        v9 = np.zeros(9)
        code = lib().exo_forces_typed(n, _d(p), tp, _d(box), bl, ntypes, _d(e), _d(s), _d(r), _d(f),
                                      C.byref(ep), C.byref(w), _d(v9) if want_virial9 else None, C.byref(cnt))
    else:
        v9 = None
        code = lib().exo_forces_typed_omp(n, _d(p), tp, _d(box), bl, ntypes, _d(e), _d(s), _d(r), _d(f),
                                          C.byref(ep), C.byref(w), threads, C.byref(cnt))
    if code != 0:
        raise OracleError(code)
    out = dict(forces=f, epot=ep.value, virial=w.value, counts=cnt)
    if want_virial9 and v9 is not None:
        out["virial9"] = v9.reshape(3, 3)
    return out


def forces_bruteforce(pos, box, rc, eps=1.0, sigma=1.0, types=None, ntypes=1):
    p = _pos(pos)
    n = p.shape[0]
    e, s, r = _tables(ntypes, eps, sigma, rc)
    t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
    f = np.zeros((n, 3))
    ep = C.c_double()
    w = C.c_double()
    code = lib().exo_forces_bruteforce(n, _d(p), _i(t) if t is not None else None,
                                       _d(np.asarray(box, dtype=np.float64)), ntypes, _d(e), _d(s), _d(r), _d(f),
                                       C.byref(ep), C.byref(w))
    if code != 0:
        raise OracleError(code)
    return dict(forces=f, epot=ep.value, virial=w.value)


def vv_run(pos, vel, box, rc, dt, nsteps, eps=1.0, sigma=1.0, types=None, ntypes=1, mass=None,
           block_length=None, threads=1, forces=None):
    """FP64 velocity-Verlet over the oracle's forces.  Returns dict(pos, vel, forces, ekin[], epot[]).
    forces: the forces at pos (e.g. a previous run's), else computed first; either way the run
    makes exactly nsteps force evaluations after that."""
    p = _pos(pos).copy()
    v = _pos(vel).copy()
    n = p.shape[0]
    e, s, r = _tables(ntypes, eps, sigma, rc)
    bl = 0.5 * float(r.max()) if block_length is None else block_length
    t = None if types is None else np.ascontiguousarray(types, dtype=np.int32)
    m = None if mass is None else np.ascontiguousarray(np.broadcast_to(mass, (ntypes,)), dtype=np.float64)
    f0 = (forces_typed(p, box, rc, eps, sigma, types, ntypes, bl, threads)["forces"].copy() if forces is None
          else _pos(forces).copy())
    en = np.zeros(2 * max(nsteps, 1))
    code = lib().exo_vv_run(n, _d(p), _d(v), _i(t) if t is not None else None, _d(m) if m is not None else None,
                            _d(np.asarray(box, dtype=np.float64)), bl, ntypes, _d(e), _d(s), _d(r), dt, nsteps,
                            threads, _d(f0), _d(en))
    if code != 0:
        raise OracleError(code)
    en = en.reshape(-1, 2)[:nsteps]
    return dict(pos=p, vel=v, forces=f0, ekin=en[:, 0].copy(), epot=en[:, 1].copy())
