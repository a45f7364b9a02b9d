"""Pairs closer than ~0.8 sigma in the mixed form.  Their force terms exceed
the fixed-point range of the shared-memory sums: the first pass leaves them out
and flags the tile, and the redo pass recomputes the flagged tiles and adds
the large terms in FP32.  The FP64 form is the reference for the same atoms."""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu]


def forces(gpulib, pos, L, precision):
    with gpulib.MidpointLJ(L, [len(pos)], precision=precision, rc=2.5) as s:
        s.set_atoms(pos)
        f, e, _ = s.forces(energy=True)
    return f, e[0]


def test_close_pairs_match_fp64(gpulib):
    """40 atoms moved to 0.62-0.75 sigma from another atom of an FCC liquid:
    pair forces of 1.6e3-1.1e4 epsilon/sigma, most of them above the
    fixed-point range (2048)."""
    from examd_gb300 import workloads as W
    c = W.liquid_fcc(8)  # 2048 atoms
    L = np.asarray(c["boxes"][0], dtype=np.float64)
    pos = c["pos"].copy()
    rng = np.random.default_rng(11)
    idx = rng.choice(len(pos), size=80, replace=False).reshape(-1, 2)
    for a, b in idx:
        u = rng.normal(size=3)
        pos[b] = (pos[a] + rng.uniform(0.62, 0.75) * u / np.linalg.norm(u)) % L
    f64, e64 = forces(gpulib, pos, L, "fp64")
    f32, e32 = forces(gpulib, pos, L, "mixed")
    fn = np.sqrt((f64 * f64).sum(1))
    err = np.sqrt(((f32 - f64) ** 2).sum(1))
    big = fn > 1024.0
    assert big.sum() >= 40
    # the large terms arrive in full: what is left is the FP32 separation's
    # rounding (~4e-7 sigma at r ~ 0.7) times 13 r^-1 of the r^-13 term ...
    assert (err[big] / fn[big]).max() <= 1e-4
    # ... and the rest of the atoms keep the mixed form's accuracy
    small = ~big
    frms = np.sqrt((fn[small] ** 2).mean())
    assert np.sqrt((err[small] ** 2).mean()) / frms <= 1e-5
    # the energy is dominated by the closest pairs (r^-12): same rounding argument
    assert e32 == pytest.approx(e64, rel=1e-4)


def test_every_atom_in_close_pairs(gpulib):
    """A jittered simple-cubic lattice at spacing 0.72 sigma: every atom has
    pair terms beyond the fixed-point range, so every tile takes the redo
    pass; forces and energy match the FP64 form, and a second evaluation
    agrees with the first (the redo list empties after each use)."""
    n1, a = 16, 0.72
    g = np.arange(n1) * a
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3) + 0.5 * a
    pos += np.random.default_rng(5).uniform(-0.04, 0.04, pos.shape)
    L = np.full(3, n1 * a)
    f64, e64 = forces(gpulib, pos, L, "fp64")
    with gpulib.MidpointLJ(L, [len(pos)], precision="mixed", rc=2.5) as s:
        s.set_atoms(pos)
        f32, e, _ = s.forces(energy=True)
        f32b, _, _ = s.forces(energy=True)
    frms = np.sqrt((f64 * f64).sum(1).mean())
    err = np.sqrt(((f32 - f64) ** 2).sum(1))
    assert frms > 1e3
    assert err.max() / frms <= 1e-4 and np.sqrt((err * err).mean()) / frms <= 2e-5
    assert e[0] == pytest.approx(e64, rel=1e-5)
    # the large terms' FP32 sums are the only order-dependent part
    assert np.abs(f32b - f32).max() / frms <= 1e-6


def test_first_pass_overflow_goes_to_the_redo_pass(gpulib):
    """The mixed form's first pass holds the largest tile at binning time plus
    6 % + 32 atoms; new positions through forces_at (no capacity update) that
    pack more atoms into a tile send that tile to the redo pass, which
    computes it in full at its own capacity (+25 % + 64).  A sine compression
    along z (pairs down to ~0.65 sigma) does that to the densest tiles: its
    amplitude is the first one whose largest tile falls between the two
    capacities.  Forces and energy match the FP64 form."""
    from examd_gb300 import workloads as W
    c = W.liquid_fcc(16)  # 16,384 atoms
    L = np.asarray(c["boxes"][0], dtype=np.float64)
    pos = c["pos"]

    def squeeze(a):
        p = pos.copy()
        z = pos[:, 2]
        p[:, 2] = (z - a * L[2] / (2 * np.pi) * np.sin(2 * np.pi * z / L[2])) % L[2]
        return p

    def largest_tile(p):
        with gpulib.MidpointLJ(L, [len(p)], precision="mixed", rc=2.5) as s:
            s.set_atoms(p)
            return s.counters()["max_tile_atoms"]

    occ_a = largest_tile(pos)
    cap_first = (occ_a + occ_a // 16 + 32 + 7) // 8 * 8
    cap_redo = (occ_a + occ_a // 4 + 64 + 7) // 8 * 8
    posb = None
    for a in (0.25, 0.3, 0.35, 0.4, 0.45, 0.5):
        if cap_first < largest_tile(squeeze(a)) <= cap_redo:
            posb = squeeze(a)
            break
    assert posb is not None
    with gpulib.MidpointLJ(L, [len(pos)], precision="mixed", rc=2.5) as s:
        s.set_atoms(pos)
        f32, e32, _ = s.forces_at(posb, energy=True)
    f64, e64 = forces(gpulib, posb, L, "fp64")
    frms = np.sqrt((f64 * f64).sum(1).mean())
    err = np.sqrt(((f32 - f64) ** 2).sum(1))
    assert np.sqrt((err * err).mean()) / frms <= 1e-5
    # the largest errors: the closest pairs' r^-13 terms with an FP32 separation
    # (~1e-5 of forces up to ~1e4 at r ~ 0.65); a tile left out or counted
    # twice would be off by the forces themselves
    assert err.max() / np.sqrt((f64 * f64).sum(1)).max() <= 1e-4
    assert e32[0] == pytest.approx(e64, rel=1e-5)
