"""The CUDA path (through the C ABI) against the oracle's committed golden
fixtures (tests/golden/, made by make_golden.py): a one-type gas, and a
two-type mixture with the Kob-Andersen-type table of the binary-mixture
workload whose closest pairs (|F| up to 2166) take the mixed form's redo
pass.  FP64 form: forces within 1e-12 of F_rms per atom, energy and virial
within 1e-12 relative, candidate and accepted counts equal.  Mixed form:
forces within 1e-5 RMS of F_rms."""
import os

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu]

HERE = os.path.dirname(os.path.abspath(__file__))


def rel_err(f, ref):
    e = np.sqrt(((f - ref) ** 2).sum(1))
    s = np.sqrt((ref * ref).sum(1).mean())
    return e.max() / s, np.sqrt((e * e).mean()) / s


@pytest.mark.parametrize("name", ["oracle_midpoint_gas", "oracle_typed_mixture"])
def test_cuda_path_matches_fixture(gpulib, name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    pos, L = g["pos"], g["box"]
    if "types" in g.files:
        kw, types = dict(eps=g["eps"], sigma=g["sigma"], rc=g["rc"], ntypes=2), g["types"]
    else:
        kw, types = dict(rc=float(g["cutoff"])), None
    with gpulib.MidpointLJ(L, [len(pos)], precision="fp64", **kw) as s:
        s.set_atoms(pos, types)
        f, ep, w = s.forces(energy=True)
        cnt = s.counters()
    mx, _ = rel_err(f, g["forces"])
    assert mx <= 1e-12
    assert ep[0] == pytest.approx(float(g["epot"]), rel=1e-12)
    assert w[0] == pytest.approx(float(g["virial"]), rel=1e-12)
    assert cnt["candidates"] == int(g["candidates"]) and cnt["accepted"] == int(g["accepted"])
    with gpulib.MidpointLJ(L, [len(pos)], precision="mixed", **kw) as s:
        s.set_atoms(pos, types)
        f32, _, _ = s.forces()
    _, rms = rel_err(f32, g["forces"])
    assert rms <= 1e-5
