"""examd_autotune: the tile shape and CTA width picked by timing, with a text cache."""
import ctypes as C

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
