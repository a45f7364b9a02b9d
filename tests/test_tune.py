"""examd_autotune: the tile shape and CTA width picked by timing, with a text cache."""
import ctypes as C
import os

import numpy as np
import pytest


def test_bad_arguments_are_refused_without_a_device(gpulib):
    from examd_gb300 import _lib
    L = _lib.load()
    p, best = _lib.Params(), _lib.Params()
    L.examd_default_params(C.byref(p))
    box = (_lib.Box * 1)()
    for a in range(3):
        box[0].L[a] = 10.0
    box[0].natoms = 10
    assert L.examd_autotune(C.byref(p), 1, box, -1, None, None, None, C.byref(best), None) == _lib.ERR_ARG
    assert L.examd_autotune(C.byref(p), 0, box, 10, None, None, None, C.byref(best), None) == _lib.ERR_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_tuned_choice_cached_and_equivalent(gpulib, tmp_path, precision, tol):
    L = np.array([18.0, 19.0, 20.0])
    pos = gpulib.gen_random(6000, L, 0.85, 21)
    cache = tmp_path / "tune.txt"
    r = gpulib.autotune(L, [len(pos)], pos, cache=cache, precision=precision, rc=2.5)
    t = sorted(r["tile"])
    assert t[0] in (3, 4, 5, 6) and t[2] - t[0] <= 2
    assert r["warps"] in (4, 8) and r["tile_balance"] in (0, 1) and r["ms"] > 0
    assert r["block_length"] is None or 1.25 * 1.09 <= r["block_length"] <= 1.25 * 1.21
    assert len(cache.read_text().splitlines()) == 1
    r2 = gpulib.autotune(L, [len(pos)], pos, cache=cache, precision=precision, rc=2.5)
    assert r2 == r and len(cache.read_text().splitlines()) == 1  # a hit, no new timing
    with gpulib.MidpointLJ.tuned(L, [len(pos)], pos, cache=cache, precision=precision, rc=2.5) as s:
        assert s.tuning == r
        f, _, _ = s.forces()
    with gpulib.MidpointLJ(L, [len(pos)], precision=precision, rc=2.5) as s:
        s.set_atoms(pos)
        g, _, _ = s.forces()
    fr = np.sqrt((g * g).sum(1).mean())
    assert np.sqrt(((f - g) ** 2).sum(1)).max() / fr <= tol


def test_cache_hit_needs_no_device(gpulib, tmp_path):
    """A cached choice is returned without timing (so without a device): tile,
    warps, tile split and cell edge come from the cache line; entries written
    before the cell edge was tuned (no "|ce" key) or before the pair lists'
    skin entered the key (no "|sk") are not used."""
    from examd_gb300 import _lib
    L = np.array([107.49, 107.49, 107.49])
    n = 1048576
    p = _lib.Params()
    _lib.load().examd_default_params(C.byref(p))
    p.precision = _lib.MIXED
    box = (_lib.Box * 1)()
    for a in range(3):
        box[0].L[a] = L[a]
    box[0].natoms = n
    # the key as examd_autotune forms it; the device name is "unknown" where none can be queried
    ctx = C.c_void_p()
    if _lib.load().examd_gpu_create(C.byref(p), 1, box, C.byref(ctx)) != _lib.ERR_NO_DEVICE:
        _lib.load().examd_gpu_destroy(ctx)
        pytest.skip("the device name in the key is only predictable without a device")
    lg = np.round(np.log2(n) * 4.0) / 4.0
    rho = np.round(n / L.prod() * 20.0) / 20.0
    key = f"unknown|mixed|nt1|rc2.5|boxes1|n{lg:.2f}|rho{rho:.2f}"
    cache = tmp_path / "tune.txt"
    cache.write_text(f"{key}|5 5 5 8 0.5\n"                 # old formats: ignored
                     f"{key}|tb|6 6 6 8 0.41 1\n"
                     f"{key}|ce|6 6 6 4 0.30 1 0\n"
                     f"{key}|ce|sk0|5 4 4 4 0.42 0 0\n"
                     f"{key}|ce|sk0|6 6 5 8 0.40 1 1.375\n"  # the last entry wins
                     f"{key}|ce|sk0.3|6 6 6 8 0.20 1 0\n")  # another skin
    best = _lib.Params()
    ms = C.c_double()
    pos = np.zeros((n, 3))
    rc = _lib.load().examd_autotune(C.byref(p), 1, box, n, pos.ctypes.data_as(C.POINTER(C.c_double)), None,
                                    os.fsencode(str(cache)), C.byref(best), C.byref(ms))
    assert rc == _lib.OK
    assert tuple(best.tile) == (6, 6, 5) and best.warps == 8 and best.tile_balance == 1 and ms.value == 0.40
    assert best.cell_edge == 1.375
