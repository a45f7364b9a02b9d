"""The pair plug-in (examd_params.potential), the counterpart of the reference's
External :: user_func and its return codes (SRC/exaMD_forces.f90:532-549)."""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu]


def brute_force(pos, L, rcut, eshift, eps=1.0, sigma=1.0):
    """O(N^2) LJ family with minimum image, FP64 (test reference)."""
    d = pos[None, :, :] - pos[:, None, :]          # d[i, j] = x_j - x_i
    d -= np.round(d / L) * L
    r2 = (d * d).sum(-1)
    np.fill_diagonal(r2, np.inf)
    on = r2 <= rcut * rcut
    s6 = np.where(on, (sigma * sigma / np.where(on, r2, 1.0)) ** 3, 0.0)
    dg = np.where(on, -24.0 * eps * (2.0 * s6 * s6 - s6) / np.where(on, r2, 1.0), 0.0)
    f = (dg[:, :, None] * d).sum(1)                # f_i = sum_j dg d_ij
    e = 0.5 * np.where(on, 4.0 * eps * (s6 * s6 - s6) - eshift, 0.0).sum()
    return f, e


def frel(f, ref):
    return np.sqrt(((f - ref) ** 2).sum(1)).max() / np.sqrt((ref * ref).sum(1).mean())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_shifted_equals_lj_minus_shift(gpulib, precision):
    L = np.array([14.0, 15.0, 16.0])
    pos = gpulib.gen_random(2000, L, 0.85, 8)
    rc = 2.5
    out = {}
    for pot in ("lj", "lj_shifted"):
        with gpulib.MidpointLJ(L, [len(pos)], precision=precision, rc=rc, potential=pot) as s:
            s.set_atoms(pos)
            f, e, _ = s.forces(energy=True)
            out[pot] = (f, e[0], s.counters()["accepted"])
    # same forces: bitwise in the mixed form (exact fixed-point sums); the FP64
    # form's FP64 shared atomics add in a varying order
    if precision == "mixed":
        assert np.array_equal(out["lj"][0], out["lj_shifted"][0])
    else:
        assert frel(out["lj_shifted"][0], out["lj"][0]) <= 1e-14
    s6 = (1.0 / rc ** 2) ** 3
    shift = 4.0 * s6 * (s6 - 1.0)
    tol = 1e-12 if precision == "fp64" else 1e-6
    assert out["lj_shifted"][1] == pytest.approx(out["lj"][1] - out["lj"][2] * shift, rel=tol)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_wca_against_brute_force(gpulib, precision, tol):
    """WCA is cut at 2^(1/6) sigma inside rc = 2.5: pairs between the two radii
    reach the pair function and are skipped (retval > 0)."""
    L = np.array([9.0, 9.5, 10.0])
    pos = gpulib.gen_random(700, L, 0.8, 9)
    rw = 2.0 ** (1.0 / 6.0)
    ref_f, ref_e = brute_force(pos, L, rw, -1.0)
    with gpulib.MidpointLJ(L, [len(pos)], precision=precision, rc=2.5, potential="wca") as s:
        s.set_atoms(pos)
        f, e, _ = s.forces(energy=True)
        acc = s.counters()["accepted"]
    d = pos[None] - pos[:, None]
    d -= np.round(d / L) * L
    r2 = (d * d).sum(-1)
    assert acc == int(((r2 <= rw * rw) & (r2 > 0)).sum() // 2)  # only applied pairs count
    assert frel(f, ref_f) <= tol
    assert e[0] == pytest.approx(ref_e, rel=tol)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_coincident_atoms_are_an_error(gpulib, precision):
    from examd_gb300 import _lib
    L = np.array([8.0, 8.0, 8.0])
    pos = gpulib.gen_random(200, L, 1.0, 10)
    pos[17] = pos[3]
    with gpulib.MidpointLJ(L, [len(pos)], precision=precision, rc=2.5) as s:
        s.set_atoms(pos)
        with pytest.raises(_lib.ExamdError) as err:
            s.forces()
    assert err.value.code == _lib.ERR_PAIRFN


def test_wca_needs_rc_over_its_range(gpulib):
    from examd_gb300 import _lib
    with pytest.raises(_lib.ExamdError) as err:
        gpulib.MidpointLJ([10.0, 10.0, 10.0], [10], rc=1.0, block_length=1.25, potential="wca")
    assert err.value.code == _lib.ERR_ARG


@pytest.mark.parametrize("pot", ["lj_shifted", "wca"])
def test_pair_lists_with_other_potentials(gpulib, pot):
    """The pair plug-in in pair-list mode: at the build the list pass gives
    the enumeration's forces and energy bit for bit (same cell edge), and
    after the atoms moved less than half the skin its forces stay within
    1e-5 of an O(N^2) FP64 sum (WCA: pairs between 2^(1/6) sigma and rc are
    in the lists and skipped by the pair function)."""
    L = np.array([14.0, 15.0, 16.0])
    pos = gpulib.gen_random(2000, L, 0.85, 12)
    skin = 0.3
    kw = dict(precision="mixed", rc=2.5, potential=pot, block_length=0.5 * (2.5 + skin))
    out = []
    for sk in (0.0, skin):
        with gpulib.MidpointLJ(L, [len(pos)], pair_skin=sk, **kw) as s:
            s.set_atoms(pos)
            out.append(s.forces(energy=True))
            if sk:
                moved = (pos + np.random.default_rng(3).uniform(-0.05, 0.05, pos.shape)) % L
                f, _, _ = s.forces_at(moved)
                assert s.list_info()["builds"] == 1
    assert np.array_equal(out[0][0], out[1][0]) and np.array_equal(out[0][1], out[1][1])
    rcut, eshift = (2.5, 4.0 * (0.4 ** 6) * (0.4 ** 6 - 1.0)) if pot == "lj_shifted" else (2.0 ** (1.0 / 6.0), -1.0)
    ref_f, _ = brute_force(moved, L, rcut, eshift)
    assert np.sqrt(((f - ref_f) ** 2).sum(1).mean()) / np.sqrt((ref_f * ref_f).sum(1).mean()) <= 1e-5
