"""Pair-list mode (examd_params.pair_skin > 0, mixed form): each tile keeps
the list of its pairs within rc + skin, built by the same midpoint ownership
as the per-evaluation enumeration, and the cells and lists are rebuilt on the
device when some atom has moved more than half the skin since the last
build.

- Where the atoms are where the lists were built, the forces, energies and
  virials equal the enumeration's at the same cell edge bit for bit: the
  list pass forms each pair's separation with the first pass's expressions,
  and the sums are exact fixed point.
- Tiles whose lists do not fit (a list capacity far too small) are computed
  by enumeration from the same offsets: the same bits again, over a whole
  trajectory.
- Along a trajectory the lists are rebuilt every few steps; the forces stay
  within the mixed form's 1e-5 RMS of the FP64 form at the same positions,
  and every pair within rc is computed once (accepted-pair counts of the
  enumeration at those positions equal the FP64 oracle's).
- The force call at new positions rebuilds only when some atom moved more
  than half the skin.
- Energy conservation of the list-mode trajectory matches the per-step
  enumeration's.
"""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu]

SKIN = 0.3
TOL_MIXED_RMS = 1e-5


def frms(f):
    return np.sqrt((f * f).sum(1).mean())


def rel_rms(f, ref):
    return np.sqrt(((f - ref) ** 2).sum(1).mean()) / frms(ref)


@pytest.fixture(scope="module")
def liquid():
    from examd_gb300 import workloads as W
    return W.liquid_fcc(20)  # 32,000 atoms, jittered FCC at rho* 0.8442, rc 2.5


@pytest.fixture(scope="module")
def melted(gpulib, liquid):
    """The liquid after 150 mixed-form steps (no longer a lattice)."""
    c = liquid
    with gpulib.MidpointLJ(c["boxes"], c["natoms"], precision="mixed", **c["lj"]) as s:
        s.set_atoms(c["pos"], c["types"], c["vel"])
        s.run(150, 0.005, graph_chunk=10)
        return s.state()


def test_list_equals_enumeration_at_the_build(gpulib, liquid, melted):
    c = liquid
    pos, _ = melted
    edge = 0.5 * (2.5 + SKIN)
    out = []
    for skin in (0.0, SKIN):
        with gpulib.MidpointLJ(c["boxes"], c["natoms"], precision="mixed", block_length=edge, pair_skin=skin,
                               **c["lj"]) as s:
            s.set_atoms(pos)
            f, e, w = s.forces(energy=True)
            if skin:
                info = s.list_info()
                assert info["builds"] >= 1 and info["fallback_tiles"] == 0 and info["capacity"] > 0
            out.append((f, e, w))
    (f0, e0, w0), (f1, e1, w1) = out
    assert np.array_equal(f0, f1)
    assert np.array_equal(e0, e1) and np.array_equal(w0, w1)


def test_fallback_tiles_equal_listed_tiles(gpulib, liquid, melted):
    """A list capacity of 16 entries: every tile is computed by enumeration
    from the lists' offsets, at every step; the trajectory is the same bit for
    bit as with lists that fit."""
    c = liquid
    pos, vel = melted
    res = []
    for cap in (0, 16):
        with gpulib.MidpointLJ(c["boxes"], c["natoms"], precision="mixed", pair_skin=SKIN,
                               pair_list_capacity=cap, **c["lj"]) as s:
            s.set_atoms(pos, None, vel)
            s.run(40, 0.005, graph_chunk=10)
            f, e, _ = s.forces(energy=True)
            p, v = s.state()
            info = s.list_info()
            res.append((f, e, p, v, info))
    (f0, e0, p0, v0, i0), (f1, e1, p1, v1, i1) = res
    assert i0["fallback_tiles"] == 0 and i1["fallback_tiles"] > 0 and i1["capacity"] == 16
    assert i0["builds"] >= 2 and i1["builds"] >= 2
    assert np.array_equal(p0, p1) and np.array_equal(v0, v1)
    assert np.array_equal(f0, f1) and np.array_equal(e0, e1)


def test_trajectory_forces_against_fp64(gpulib, oracle, liquid, melted):
    c = liquid
    pos, vel = melted
    with gpulib.MidpointLJ(c["boxes"], c["natoms"], precision="mixed", pair_skin=SKIN, **c["lj"]) as s:
        s.set_atoms(pos, None, vel)
        b0 = s.list_info()["builds"]
        for _ in range(4):
            s.run(50, 0.005, graph_chunk=10)
            p, _ = s.state()
            f, e, _ = s.forces(energy=True)
            with gpulib.MidpointLJ(c["boxes"], c["natoms"], precision="fp64", **c["lj"]) as d:
                d.set_atoms(p)
                g, e64, _ = d.forces(energy=True)
                cnt = d.counters()
            assert rel_rms(f, g) <= TOL_MIXED_RMS
            assert abs(e[0] - e64[0]) <= 1e-6 * abs(e64[0])
        builds = s.list_info()["builds"] - b0
    # rebuilt every few steps, not every step
    assert 4 <= builds <= 100
    # the accepted pairs at the last positions: the oracle's
    ref = oracle.forces_typed(p, c["boxes"][0], rc=2.5)
    assert cnt["accepted"] == ref["counts"].accepted


def test_forces_at_rebuilds_only_past_half_the_skin(gpulib, liquid, melted):
    c = liquid
    pos, _ = melted
    L = c["boxes"][0]
    rng = np.random.default_rng(7)
    with gpulib.MidpointLJ(c["boxes"], c["natoms"], precision="mixed", pair_skin=SKIN, **c["lj"]) as s, \
            gpulib.MidpointLJ(c["boxes"], c["natoms"], precision="fp64", **c["lj"]) as d:
        s.set_atoms(pos)
        d.set_atoms(pos)
        b0 = s.list_info()["builds"]
        small = (pos + rng.uniform(-0.05, 0.05, pos.shape)) % L  # |d| < 0.087 < skin/2
        f, _, _ = s.forces_at(small)
        g, _, _ = d.forces_at(small)
        assert rel_rms(f, g) <= TOL_MIXED_RMS
        assert s.list_info()["builds"] == b0
        big = small.copy()
        big[123] = (big[123] + 0.2) % L  # one atom past half the skin
        f, _, _ = s.forces_at(big)
        g, _, _ = d.forces_at(big)
        assert rel_rms(f, g) <= TOL_MIXED_RMS
        assert s.list_info()["builds"] == b0 + 1
        # the atom nearest the high x face crosses the periodic boundary (by
        # less than half the skin): no rebuild, its offset taken at the image
        # nearest its cell
        wrap = big.copy()
        k = int(np.argmax(big[:, 0]))
        assert big[k, 0] + 0.1 >= L[0]
        wrap[k, 0] = (big[k, 0] + 0.1) - L[0]
        f, _, _ = s.forces_at(wrap)
        g, _, _ = d.forces_at(wrap)
        assert rel_rms(f, g) <= TOL_MIXED_RMS
        assert s.list_info()["builds"] == b0 + 1


def test_mixture_batch_against_oracle(gpulib, oracle):
    """Two atom types with per-pair cutoffs, three boxes of different density
    in one batch: each box against the oracle after list-mode steps."""
    from examd_gb300 import workloads as W
    c = W.binary_mixture(m=24)
    lj = c["lj"]
    boxes = np.repeat(c["boxes"], 3, axis=0)
    pos = np.concatenate([c["pos"]] * 3)
    types = np.concatenate([c["types"]] * 3)
    vel = np.concatenate([c["vel"] * f for f in (0.5, 1.0, 1.5)])
    natoms = np.repeat(c["natoms"], 3)
    with gpulib.MidpointLJ(boxes, natoms, precision="mixed", pair_skin=SKIN, **lj) as s:
        s.set_atoms(pos, types, vel)
        s.run(60, 0.003, graph_chunk=10)
        p, _ = s.state()
        f, e, w = s.forces(energy=True)
    kw = dict(rc=lj["rc"], eps=lj["eps"], sigma=lj["sigma"], ntypes=lj["ntypes"])
    n = c["natoms"][0]
    for b in range(3):
        sl = slice(b * n, (b + 1) * n)
        ref = oracle.forces_typed(p[sl], boxes[b], types=types[sl], **kw)
        assert rel_rms(f[sl], ref["forces"]) <= TOL_MIXED_RMS
        assert abs(e[b] - ref["epot"]) <= 1e-6 * abs(ref["epot"])


def test_energy_conservation_like_the_enumeration(gpulib, liquid, melted):
    c = liquid
    pos, vel = melted
    drift = []
    for skin in (0.0, SKIN):
        with gpulib.MidpointLJ(c["boxes"], c["natoms"], precision="mixed", pair_skin=skin, **c["lj"]) as s:
            s.set_atoms(pos, None, vel)
            r = s.run(400, 0.005, graph_chunk=20, energies=True)
        e = (r["ekin"] + r["epot"])[:, 0]
        drift.append(abs(e[-1] - e[0]) / abs(e[0]))
    assert drift[1] <= max(5 * drift[0], 2e-5)


def test_pairs_at_the_cutoff_decided_as_the_fp64_form(gpulib):
    """Isolated pairs at r = rc (1 + delta), |delta| <= 3e-7, where the FP32
    r^2 and the FP64 one can fall on different sides of rc^2: the mixed form
    (per-step enumeration and pair lists) decides each such pair on its FP64
    r^2, so exactly the pairs the FP64 form applies have a force, and each
    within two steps of the fixed-point sums (2^-16) of it."""
    rng = np.random.default_rng(11)
    L = 90.0
    g = np.arange(10) * 9.0 + 1.0  # 9 apart: atoms of different pairs stay 4 apart at least
    centers = np.stack(np.meshgrid(g, g, g[:2], indexing="ij"), -1).reshape(-1, 3)  # 200 pairs
    u = rng.normal(size=centers.shape)
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = 2.5 * (1.0 + rng.uniform(-3e-7, 3e-7, len(centers)))
    pos = np.concatenate([centers, centers + u * r[:, None]])
    box = [L, L, L]
    with gpulib.MidpointLJ(box, [len(pos)], precision="fp64", rc=2.5) as d:
        d.set_atoms(pos)
        g64, _, _ = d.forces()
    on64 = np.linalg.norm(g64, axis=1) > 0
    assert 0 < on64.sum() < len(pos)  # both sides of the cutoff are present
    for skin in (0.0, SKIN):
        with gpulib.MidpointLJ(box, [len(pos)], precision="mixed", rc=2.5, pair_skin=skin) as s:
            s.set_atoms(pos)
            f, _, _ = s.forces()
        on = np.linalg.norm(f, axis=1) > 0
        assert np.array_equal(on, on64)
        assert np.abs(f[on] - g64[on]).max() <= 2.0 ** -16
