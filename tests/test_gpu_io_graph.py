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


def test_graph_replay_with_energy_across_a_run(gpulib, case):
    """The energy variant of the captured force call, with the same pinned
    buffers before and after a run: the run reallocates the per-box energy
    buffers (its first call sizes them for its graph chunk), so the force
    call must capture again instead of replaying a graph that names the old
    ones."""
    kw = dict(precision="mixed", **case["lj"])
    p0 = case["pos"]
    with gpulib.MidpointLJ(case["boxes"], case["natoms"], **kw) as s:
        s.set_atoms(p0)
        f_ref, e_ref, w_ref = s.forces_at(p0, energy=True)
    hp = gpulib.pinned_empty(p0.shape)
    hf = gpulib.pinned_empty(p0.shape)
    with gpulib.MidpointLJ(case["boxes"], case["natoms"], **kw) as s:
        s.set_atoms(p0)
        hp[:] = p0
        for _ in range(3):  # capture at both parities, then a replay
            _, e, w = s.forces_at(hp, out=hf, energy=True)
        assert np.array_equal(hf, f_ref) and np.array_equal(e, e_ref) and np.array_equal(w, w_ref)
        s.run(4, 0.001, graph_chunk=2)
        for _ in range(3):
            _, e, w = s.forces_at(hp, out=hf, energy=True)
            assert np.array_equal(hf, f_ref) and np.array_equal(e, e_ref) and np.array_equal(w, w_ref)
        s.run(6, 0.001, graph_chunk=4)  # grows the energy buffers again
        _, e, w = s.forces_at(hp, out=hf, energy=True)
        assert np.array_equal(hf, f_ref) and np.array_equal(e, e_ref) and np.array_equal(w, w_ref)


def test_graph_replay_with_pair_lists(gpulib, case):
    """Pair lists (mixed form): the captured force call holds the rebuild as
    a conditional graph node.  Replays over positions that move a little
    (no rebuild) and then past half the skin (a rebuild inside the graph)
    equal the eager calls bit for bit, and the rebuilds happen where the
    eager context has them.  The atoms move past half the skin by a common
    shift: random moves that large bring pairs within 0.74 sigma, whose
    large terms the redo pass sums in FP32 in an order that can vary
    between runs."""
    rng = np.random.default_rng(5)
    L = case["boxes"][0]
    shifts = [(0, 0, 0), (0, 0, 0), (0.2, 0.1, -0.05), (0.2, 0.1, -0.05), (0.42, 0.1, -0.05), (0.42, 0.1, -0.05)]
    steps = [(case["pos"] + np.asarray(d) + rng.uniform(-0.02, 0.02, case["pos"].shape)) % L for d in shifts]
    kw = dict(precision="mixed", pair_skin=0.3, **case["lj"])
    eager, graph, b_e, b_g = [], [], [], []
    with gpulib.MidpointLJ(case["boxes"], case["natoms"], **kw) as s:
        s.set_atoms(case["pos"])
        for p in steps:
            f, e, w = s.forces_at(p, energy=True)
            eager.append((f.copy(), e.copy(), w.copy()))
            b_e.append(s.list_info()["builds"])
    hp = gpulib.pinned_empty(case["pos"].shape)
    hf = gpulib.pinned_empty(case["pos"].shape)
    with gpulib.MidpointLJ(case["boxes"], case["natoms"], **kw) as s:
        s.set_atoms(case["pos"])
        for p in steps:
            hp[:] = p
            _, e, w = s.forces_at(hp, out=hf, energy=True)
            graph.append((hf.copy(), e, w))
            b_g.append(s.list_info()["builds"])
    assert b_e == b_g
    assert [b - b_e[0] for b in b_e] == [0, 0, 1, 1, 2, 2]
    for (fa, ea, wa), (fb, eb, wb) in zip(eager, graph):
        assert np.array_equal(fa, fb)
        assert np.array_equal(ea, eb) and np.array_equal(wa, wb)
