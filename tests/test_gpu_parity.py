"""GPU parity: the CUDA path (through the C ABI) against the CPU oracle.

Tolerances: FP64 form within 1e-12 of the oracle per atom, measured as
|dF_i| / F_rms (norm-wise; per-atom |dF_i|/|F_i| is undefined where F_i ~ 0)
and 1e-12 relative on energy and virial; mixed form within 1e-5 RMS
relative to the FP64 path.
"""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu, pytest.mark.timeout(600)] if hasattr(pytest.mark, "timeout") else [pytest.mark.gpu]

TOL64 = 1e-12
TOL_MIXED_RMS = 1e-5


def frms(f):
    return np.sqrt((f * f).sum(1).mean())


def rel_err(f, ref):
    e = np.sqrt(((f - ref) ** 2).sum(1))
    s = frms(ref)
    return e.max() / s, np.sqrt((e * e).mean()) / s


def gas(gl, L, n, dmin, seed):
    return gl.gen_random(n, L, dmin, seed)


def liquid_fcc(gl, nc, rho, jitter, seed):
    pos, L = gl.gen_fcc(nc, rho)
    rng = np.random.default_rng(seed)
    pos = (pos + rng.uniform(-jitter, jitter, pos.shape)) % L
    return pos, L


def test_fp64_matches_oracle_gas(gpulib, oracle):
    L = np.array([16.0, 17.0, 18.0])
    pos = gas(gpulib, L, 2500, 0.8, 1)
    ref = oracle.forces_typed(pos, L, 2.5)
    with gpulib.MidpointLJ(L, [len(pos)], precision="fp64", rc=2.5) as s:
        s.set_atoms(pos)
        f, ep, w = s.forces(energy=True)
        cnt = s.counters()
    mx, _ = rel_err(f, ref["forces"])
    assert mx <= TOL64
    assert ep[0] == pytest.approx(ref["epot"], rel=TOL64)
    assert w[0] == pytest.approx(ref["virial"], rel=TOL64)
    assert cnt["candidates"] == ref["counts"].candidates
    assert cnt["accepted"] == ref["counts"].accepted


def test_fp64_matches_oracle_config1_fcc(gpulib, oracle):
    """32,000 atoms, FCC 20^3 x 4 at rho* = 0.8442, jittered, rc = 2.5."""
    pos, L = liquid_fcc(gpulib, 20, 0.8442, 0.15, 2)
    box = np.full(3, L)
    ref = oracle.forces_typed(pos, box, 2.5, threads=0)
    with gpulib.MidpointLJ(box, [len(pos)], precision="fp64", rc=2.5) as s:
        s.set_atoms(pos)
        f, ep, w = s.forces(energy=True)
    mx, _ = rel_err(f, ref["forces"])
    assert mx <= TOL64
    assert ep[0] == pytest.approx(ref["epot"], rel=TOL64)
    assert w[0] == pytest.approx(ref["virial"], rel=TOL64)
    assert abs(f.sum(0)).max() <= 1e-9 * frms(f) * len(f) ** 0.5


def test_reference_restatement_equals_typed_path(gpulib, oracle):
    """forces_midpoint_all (the restated reference, no energy) against the GPU."""
    L = np.array([13.0, 14.0, 15.0])
    pos = gas(gpulib, L, 1200, 0.85, 3)
    ref, cnt = oracle.forces_midpoint_all(pos, L, 2.5)
    f = gpulib.forces_midpoint_all(pos, L, 2.5)
    mx, _ = rel_err(f, ref)
    assert mx <= TOL64


def test_mixed_vs_fp64(gpulib):
    pos, L = liquid_fcc(gpulib, 12, 0.8442, 0.2, 4)
    box = np.full(3, L)
    with gpulib.MidpointLJ(box, [len(pos)], precision="fp64") as s:
        s.set_atoms(pos)
        f64, e64, w64 = s.forces(energy=True)
    with gpulib.MidpointLJ(box, [len(pos)], precision="mixed") as s:
        s.set_atoms(pos)
        f32, e32, w32 = s.forces(energy=True)
    mx, rms = rel_err(f32, f64)
    assert rms <= TOL_MIXED_RMS
    assert e32[0] == pytest.approx(e64[0], rel=1e-5)
    assert w32[0] == pytest.approx(w64[0], rel=1e-5)


@pytest.mark.parametrize("tile", [(2, 2, 2), (3, 4, 5), (6, 6, 6), (8, 5, 3)])
def test_tile_shape_invariance(gpulib, tile):
    """The reference's serial-vs-parallel check restated: tile shapes must agree."""
    pos, L = liquid_fcc(gpulib, 10, 0.8442, 0.2, 5)
    box = np.full(3, L)
    with gpulib.MidpointLJ(box, [len(pos)], precision="fp64", tile=(4, 4, 4)) as s:
        s.set_atoms(pos)
        f0, e0, _ = s.forces(energy=True)
    with gpulib.MidpointLJ(box, [len(pos)], precision="fp64", tile=tile, warps=4) as s:
        s.set_atoms(pos)
        f1, e1, _ = s.forces(energy=True)
    mx, _ = rel_err(f1, f0)
    assert mx <= 1e-13
    assert e1[0] == pytest.approx(e0[0], rel=1e-13)


def test_repeatable(gpulib):
    """Mixed form: fixed-point force sums, bit-for-bit reproducible.  FP64
    form: FP64 shared-memory atomics, reproducible to rounding."""
    pos, L = liquid_fcc(gpulib, 10, 0.8442, 0.2, 6)
    box = np.full(3, L)
    with gpulib.MidpointLJ(box, [len(pos)], precision="mixed") as s:
        s.set_atoms(pos)
        a, ea, _ = s.forces(energy=True)
        b, eb, _ = s.forces(energy=True)
    assert np.array_equal(a, b) and np.array_equal(ea, eb)
    with gpulib.MidpointLJ(box, [len(pos)], precision="fp64") as s:
        s.set_atoms(pos)
        a, ea, _ = s.forces(energy=True)
        b, eb, _ = s.forces(energy=True)
    mx, _ = rel_err(a, b)
    assert mx <= 1e-14
    assert ea[0] == pytest.approx(eb[0], rel=1e-14)


def test_typed_mixture(gpulib, oracle):
    pos, t, L = gpulib.gen_jittered_sc(16, 1.2, 0.1, 0.2, 7)
    box = np.full(3, L)
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    rc = 2.5 * sig
    ref = oracle.forces_typed(pos, box, rc, eps, sig, t, 2, threads=0)
    with gpulib.MidpointLJ(box, [len(pos)], precision="fp64", eps=eps, sigma=sig, rc=rc, ntypes=2) as s:
        s.set_atoms(pos, types=t)
        f, ep, w = s.forces(energy=True)
    mx, _ = rel_err(f, ref["forces"])
    assert mx <= TOL64
    assert ep[0] == pytest.approx(ref["epot"], rel=TOL64)
    with gpulib.MidpointLJ(box, [len(pos)], precision="mixed", eps=eps, sigma=sig, rc=rc, ntypes=2) as s:
        s.set_atoms(pos, types=t)
        f32, _, _ = s.forces()
    _, rms = rel_err(f32, ref["forces"])
    assert rms <= TOL_MIXED_RMS


def test_batched_boxes_equal_single(gpulib, oracle):
    rng = np.random.default_rng(8)
    boxes, poss = [], []
    for k, n in enumerate((300, 900, 2000)):
        rho = rng.uniform(0.3, 0.9)
        Lk = (n / rho) ** (1 / 3)
        boxes.append([Lk, Lk, Lk])
        poss.append(gpulib.gen_random(n, [Lk] * 3, 0.8, 100 + k))
    allpos = np.concatenate(poss)
    with gpulib.MidpointLJ(np.array(boxes), [len(p) for p in poss], precision="fp64") as s:
        s.set_atoms(allpos)
        f, ep, w = s.forces(energy=True)
    off = 0
    for k, p in enumerate(poss):
        ref = oracle.forces_typed(p, np.array(boxes[k]), 2.5)
        mx, _ = rel_err(f[off:off + len(p)], ref["forces"])
        assert mx <= TOL64
        assert ep[k] == pytest.approx(ref["epot"], rel=TOL64)
        off += len(p)


def test_batched_uneven_density_both_forms(gpulib, oracle):
    """Boxes of density 0.25 to 0.9 in one batch: the lighter boxes get longer
    tiles (up to 2 cells per axis) than the densest one's.  Both forms
    against the oracle per box, and the tile count below that of uniform
    tiles."""
    boxes, poss = [], []
    for k, (n, rho) in enumerate(((4000, 0.9), (3000, 0.25), (2500, 0.5), (1200, 0.35))):
        Lk = (n / rho) ** (1 / 3)
        boxes.append([Lk, Lk, Lk])
        poss.append(gpulib.gen_random(n, [Lk] * 3, 0.8, 200 + k))
    allpos = np.concatenate(poss)
    counts = [len(p) for p in poss]
    out = {}
    for prec in ("fp64", "mixed"):
        with gpulib.MidpointLJ(np.array(boxes), counts, precision=prec, tile=3) as s:
            s.set_atoms(allpos)
            out[prec] = s.forces(energy=True)[:2] + (s.counters()["tiles"],)
    off = 0
    for k, p in enumerate(poss):
        ref = oracle.forces_typed(p, np.array(boxes[k]), 2.5)
        mx, _ = rel_err(out["fp64"][0][off:off + len(p)], ref["forces"])
        assert mx <= TOL64
        assert out["fp64"][1][k] == pytest.approx(ref["epot"], rel=TOL64)
        _, rms = rel_err(out["mixed"][0][off:off + len(p)], ref["forces"])
        assert rms <= TOL_MIXED_RMS
        off += len(p)
    # uniform 3^3 tiles would need sum over boxes of ceil(nb / 3)^3 tiles
    uniform = 0
    for Lk in boxes:
        nb = int(Lk[0] / 1.25)
        uniform += max(1, min(nb // 2, -(-nb // 3))) ** 3
    assert out["mixed"][2] < uniform


def test_accumulate_and_forces_at(gpulib, oracle):
    L = np.array([15.0, 15.0, 16.0])
    pos = gas(gpulib, L, 1500, 0.8, 9)
    pos2 = gas(gpulib, L, 1500, 0.8, 10)
    with gpulib.MidpointLJ(L, [len(pos)], precision="fp64") as s:
        s.set_atoms(pos)
        f1, _, _ = s.forces()
        base = np.random.default_rng(1).normal(size=f1.shape)
        acc = base.copy()
        s.forces(out=acc, accumulate=True)
        np.testing.assert_allclose(acc, base + f1, rtol=1e-14, atol=1e-10)
        f2, _, _ = s.forces_at(pos2)
    ref = oracle.forces_typed(pos2, L, 2.5)
    mx, _ = rel_err(f2, ref["forces"])
    assert mx <= TOL64


def test_vv_trajectory_matches_oracle(gpulib, oracle):
    pos, L = liquid_fcc(gpulib, 6, 0.8442, 0.1, 11)
    box = np.full(3, L)
    vel = gpulib.gen_velocities(len(pos), 0.72, 1)
    ref = oracle.vv_run(pos, vel, box, 2.5, 0.005, 20)
    with gpulib.MidpointLJ(box, [len(pos)], precision="fp64") as s:
        s.set_atoms(pos, vel=vel)
        out = s.run(20, 0.005, energies=True)
        p, v = s.state()
    d = p - ref["pos"]
    d -= np.round(d / L) * L
    assert np.abs(d).max() < 1e-9
    assert np.abs(v - ref["vel"]).max() < 1e-9
    np.testing.assert_allclose(out["epot"][:, 0], ref["epot"], rtol=1e-10)
    np.testing.assert_allclose(out["ekin"][:, 0], ref["ekin"], rtol=1e-10)


def test_graph_run_equals_eager(gpulib):
    """The CUDA-graph step loop runs the same kernels as the eager loop."""
    pos, L = liquid_fcc(gpulib, 8, 0.8442, 0.1, 12)
    box = np.full(3, L)
    vel = gpulib.gen_velocities(len(pos), 1.0, 2)
    res = []
    for chunk in (0, 10):
        with gpulib.MidpointLJ(box, [len(pos)], precision="fp64") as s:
            s.set_atoms(pos, vel=vel)
            out = s.run(30, 0.005, graph_chunk=chunk, energies=True)
            res.append((s.state(), out))
    (p0, v0), o0 = res[0]
    (p1, v1), o1 = res[1]
    d = p0 - p1
    d -= np.round(d / L) * L
    assert np.abs(d).max() < 1e-11 and np.abs(v0 - v1).max() < 1e-11
    np.testing.assert_allclose(o0["epot"], o1["epot"], rtol=1e-12)
    np.testing.assert_allclose(o0["ekin"], o1["ekin"], rtol=1e-12)


def test_errors(gpulib):
    from examd_gb300 import ExamdError, _lib
    with pytest.raises(ExamdError) as e:
        gpulib.MidpointLJ([6.0, 20.0, 20.0], [10])
    assert e.value.code == _lib.ERR_NB_TOO_SMALL
    L = np.array([15.0, 15.0, 15.0])
    pos = gas(gpulib, L, 200, 0.8, 13)
    bad = pos.copy()
    bad[7, 1] = np.nan
    with gpulib.MidpointLJ(L, [len(pos)]) as s:
        with pytest.raises(ExamdError) as e:
            s.set_atoms(bad)
        assert e.value.code == _lib.ERR_NONFINITE
        s.set_atoms(pos)  # the context stays usable
        f, _, _ = s.forces()
        assert np.isfinite(f).all()
    out = pos.copy()
    out[3, 0] = -0.25
    with gpulib.MidpointLJ(L, [len(pos)], strict_box=True) as s:
        with pytest.raises(ExamdError) as e:
            s.set_atoms(out)
        assert e.value.code == _lib.ERR_OUTSIDE
    with gpulib.MidpointLJ(L, [len(pos)]) as s:  # wrapped: same forces as the wrapped input
        s.set_atoms(out)
        f1, _, _ = s.forces()
        w = out.copy()
        w[3, 0] += L[0]
        s.set_atoms(w)
        f2, _, _ = s.forces()
    np.testing.assert_allclose(f1, f2, rtol=1e-12, atol=1e-12)


def test_empty_and_single_atom(gpulib):
    L = np.array([15.0, 15.0, 15.0])
    with gpulib.MidpointLJ(L, [1]) as s:
        s.set_atoms(np.array([[1.0, 2.0, 3.0]]))
        f, ep, _ = s.forces(energy=True)
        assert np.all(f == 0) and ep[0] == 0
    with gpulib.MidpointLJ(L, [0]) as s:
        s.set_atoms(np.zeros((0, 3)))
        f, ep, _ = s.forces(energy=True)
        assert f.shape == (0, 3) and ep[0] == 0


@pytest.mark.parametrize("edge", [1.375, 1.5])
def test_fp64_matches_oracle_at_larger_cell_edges(gpulib, oracle, edge):
    """A cell edge above rc/2 (the autotuner tries 1.1 and 1.2 x rc/2): the
    reference's block rule and 63-entry table at that block length
    (exaMD_domain_create takes it as a parameter, SRC/exaMD_utils.f90:167-190),
    against the oracle at the same length: forces, energy, virial and the
    candidate and accepted pair counts.  Both edges have few significant bits,
    so the library uses them as given."""
    L = np.array([16.0, 17.0, 18.0])
    pos = gas(gpulib, L, 3000, 0.8, 12)
    ref = oracle.forces_typed(pos, L, 2.5, block_length=edge)
    with gpulib.MidpointLJ(L, [len(pos)], precision="fp64", rc=2.5, block_length=edge) as s:
        s.set_atoms(pos)
        f, ep, w = s.forces(energy=True)
        cnt = s.counters()
    mx, _ = rel_err(f, ref["forces"])
    assert mx <= TOL64
    assert ep[0] == pytest.approx(ref["epot"], rel=TOL64)
    assert w[0] == pytest.approx(ref["virial"], rel=TOL64)
    assert cnt["candidates"] == ref["counts"].candidates
    assert cnt["accepted"] == ref["counts"].accepted
    # more candidates than at rc/2, the same accepted pairs
    ref0 = oracle.forces_typed(pos, L, 2.5)
    assert ref["counts"].candidates > ref0["counts"].candidates
    assert ref["counts"].accepted == ref0["counts"].accepted
    with gpulib.MidpointLJ(L, [len(pos)], precision="mixed", rc=2.5, block_length=edge) as s:
        s.set_atoms(pos)
        g, _, _ = s.forces()
    assert rel_err(g, ref["forces"])[1] <= TOL_MIXED_RMS
