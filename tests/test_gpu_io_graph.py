"""The force call at new positions with the caller's pinned buffers: from the
second call on with the same buffers it replays a captured CUDA graph (one
per parity of the sort's double buffer).  Its results equal the eager path's
(pageable buffers) bit for bit in the mixed form, with and without
accumulation and energies, across both parities and after a run."""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu]


@pytest.fixture(scope="module")
def case():
    from examd_gb300 import workloads as W
    return W.liquid_fcc(26)  # 70,304 atoms: above the chunked-I/O threshold


def test_graph_replay_equals_eager(gpulib, case):
    rng = np.random.default_rng(3)
    L = case["boxes"][0]
    steps = [(case["pos"] + rng.uniform(-0.02, 0.02, case["pos"].shape)) % L for _ in range(5)]
    kw = dict(precision="mixed", **case["lj"])
    eager, graph = [], []
    with gpulib.MidpointLJ(case["boxes"], case["natoms"], **kw) as s:
        s.set_atoms(case["pos"])
        for p in steps:
            f, e, w = s.forces_at(p, energy=True)
            eager.append((f.copy(), e.copy(), w.copy()))
    hp = gpulib.pinned_empty(case["pos"].shape)
    hf = gpulib.pinned_empty(case["pos"].shape)
    with gpulib.MidpointLJ(case["boxes"], case["natoms"], **kw) as s:
        s.set_atoms(case["pos"])
        for p in steps:
            hp[:] = p
            _, e, w = s.forces_at(hp, out=hf, energy=True)
            graph.append((hf.copy(), e, w))
        # after a run the sorted order and parity moved on: the replay still agrees
        s.run(3, 0.001)
        hp[:] = steps[0]
        s.forces_at(hp, out=hf)
        again = hf.copy()
        # accumulation into the caller's forces
        hf[:] = 1.0
        s.forces_at(hp, out=hf, accumulate=True)
        acc = hf.copy()
    for (fa, ea, wa), (fb, eb, wb) in zip(eager, graph):
        assert np.array_equal(fa, fb)
        assert np.array_equal(ea, eb) and np.array_equal(wa, wb)
    assert np.array_equal(again, eager[0][0])
    assert np.array_equal(acc, eager[0][0] + 1.0)
