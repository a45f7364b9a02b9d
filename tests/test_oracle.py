"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests or golden vectors, so the oracle's restatement of
exaMD_forces_midpoint_all is pinned here by analytic cases and by an
independent O(N^2) minimum-image pair sum; tests/golden/ holds a regression
fixture of the oracle itself (tests/golden/make_golden.py).
"""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def lj_force_on_1(r, eps=1.0, sigma=1.0):
    """x-force on atom 1 at 0 from atom 2 at +r: U'(r)."""
    sr6 = (sigma / r) ** 6
    return 4 * eps * (-12 * sr6 * sr6 / r + 6 * sr6 / r)


def test_two_atoms_analytic(oracle):
    L = np.array([20.0, 20.0, 20.0])
    for r in (0.95, 1.0, 2 ** (1 / 6), 1.5, 2.4):
        pos = np.array([[5.0, 6.0, 7.0], [5.0 + r, 6.0, 7.0]])
        f, c = oracle.forces_midpoint_all(pos, L, 2.5)
        assert c.accepted == 1
        assert f[0, 0] == pytest.approx(lj_force_on_1(r), rel=1e-13, abs=1e-14)
        assert f[1, 0] == -f[0, 0]
        assert np.all(f[:, 1:] == 0.0)


def test_cutoff_inclusive(oracle):
    """d2 > rc^2 skips (user_func.f90:52): a pair at exactly rc is kept."""
    L = np.array([20.0, 20.0, 20.0])
    pos = np.array([[1.0, 1.0, 1.0], [3.5, 1.0, 1.0]])  # dx = 2.5 exactly
    f, c = oracle.forces_midpoint_all(pos, L, 2.5)
    assert c.accepted == 1 and f[0, 0] != 0.0
    pos[1, 0] = 3.5 + 1e-9
    f, c = oracle.forces_midpoint_all(pos, L, 2.5)
    assert c.accepted == 0 and np.all(f == 0.0)


@pytest.mark.parametrize("shift", [(1, 0, 0), (0, 1, 0), (0, 0, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1), (1, 1, 1)])
def test_minimum_image_faces_edges_corners(oracle, shift):
    L = np.array([15.0, 16.0, 17.0])
    a = np.array([0.3, 0.4, 0.2])
    s = np.array(shift)
    d = np.array([-0.75, -0.7, -0.65]) / np.sqrt(s.sum()) * s  # crosses the faces named by shift
    b = (a + d) % L
    f, c = oracle.forces_midpoint_all(np.array([a, b]), L, 2.5)
    r = np.linalg.norm(d)
    ref = lj_force_on_1(r) * d / r  # force on atom 0 from atom 1 at a + d: U'(r) d/r
    assert c.accepted == 1
    np.testing.assert_allclose(f[0], ref, rtol=1e-11, atol=1e-13)
    np.testing.assert_array_equal(f[1], -f[0])


def test_bruteforce_agreement_random(oracle):
    rng = np.random.default_rng(3)
    for L, n, rc in (((16.0, 17.0, 18.0), 900, 2.5), ((12.6, 12.6, 25.1), 700, 2.5), ((20.0, 21.0, 22.0), 1000, 3.0)):
        L = np.array(L)
        pos = rng.uniform(0, 1, (n, 3)) * L
        f, c = oracle.forces_midpoint_all(pos, L, rc)
        b = oracle.forces_bruteforce(pos, L, rc)
        scale = np.sqrt((b["forces"] ** 2).sum(1).mean())
        assert np.abs(f - b["forces"]).max() <= 1e-13 * scale
        t = oracle.forces_typed(pos, L, rc)
        assert np.array_equal(t["forces"], f)
        assert t["epot"] == pytest.approx(b["epot"], rel=1e-12)
        assert t["virial"] == pytest.approx(b["virial"], rel=1e-12)
        assert t["counts"].accepted == c.accepted


def test_candidate_count_formula(oracle):
    """Candidates = self pairs n(n-1)/2 per block + n_a n_b over the 62 classes."""
    rng = np.random.default_rng(5)
    L = np.array([14.0, 15.0, 16.0])
    pos = rng.uniform(0, 1, (600, 3)) * L
    bl = 1.25
    nb = (L / bl).astype(int)
    cell = np.minimum((pos / bl).astype(int), nb - 1)
    cnt = np.zeros(nb, dtype=np.int64)
    np.add.at(cnt, tuple(cell.T), 1)
    tab = oracle.midpoint_table()
    off = lambda s: np.array([(s - 1) % 3 - 1, ((s - 1) // 3) % 3 - 1, (s - 1) // 9 - 1])
    expect = int((cnt * (cnt - 1) // 2).sum())
    idx = np.indices(nb).reshape(3, -1).T
    for a, b in tab[1:]:
        ia = (idx + off(a)) % nb
        ib = (idx + off(b)) % nb
        expect += int((cnt[tuple(ia.T)] * cnt[tuple(ib.T)]).sum())
    _, c = oracle.forces_midpoint_all(pos, L, 2.5)
    assert c.candidates == expect


def test_fcc_lattice(oracle):
    """Perfect FCC: sum F = 0, every |F_i| ~ 0, energy = analytic lattice sum."""
    nc, rho, rc = 6, 0.8442, 2.5
    a = (4 / rho) ** (1 / 3)
    basis = np.array([[0, 0, 0], [.5, .5, 0], [.5, 0, .5], [0, .5, .5]])
    g = np.array([[i, j, k] for k in range(nc) for j in range(nc) for i in range(nc)])
    pos = ((g[:, None, :] + basis[None]) * a).reshape(-1, 3) + 0.01
    L = np.full(3, nc * a)
    t = oracle.forces_typed(pos, L, rc)
    f = t["forces"]
    assert np.abs(f.sum(0)).max() < 1e-10
    assert np.abs(f).max() < 1e-10
    # lattice sum over neighbour shells of one atom
    m = np.arange(-3, 4)
    pts = (np.stack(np.meshgrid(m, m, m, indexing="ij"), -1).reshape(-1, 1, 3) + basis[None]).reshape(-1, 3) * a
    r = np.linalg.norm(pts, axis=1)
    r = r[(r > 0) & (r <= rc)]
    u_atom = 0.5 * np.sum(4 * (r ** -12 - r ** -6))
    assert t["epot"] == pytest.approx(u_atom * len(pos), rel=1e-12)


def test_errors(oracle):
    L = np.array([6.0, 20.0, 20.0])  # 4 blocks of 1.25 on x+... Int(6/1.25) = 4 < 5
    pos = np.array([[1.0, 1.0, 1.0], [2.0, 1.0, 1.0]])
    with pytest.raises(oracle.OracleError) as e:
        oracle.forces_midpoint_all(pos, L, 2.5)
    assert e.value.code == oracle.ERR_NB_TOO_SMALL
    L = np.array([20.0, 20.0, 20.0])
    with pytest.raises(oracle.OracleError) as e:
        oracle.forces_midpoint_all(np.array([[-0.5, 1.0, 1.0], [2.0, 1.0, 1.0]]), L, 2.5)
    assert e.value.code == oracle.ERR_OUTSIDE


def test_accumulates_like_reference(oracle):
    rng = np.random.default_rng(9)
    L = np.array([15.0, 15.0, 15.0])
    pos = rng.uniform(0, 1, (300, 3)) * L
    f1, _ = oracle.forces_midpoint_all(pos, L, 2.5)
    base = rng.normal(size=f1.shape)
    acc = base.copy()
    oracle.forces_midpoint_all(pos, L, 2.5, forces=acc)
    np.testing.assert_allclose(acc, base + f1, rtol=1e-15, atol=1e-12)


def test_omp_matches_serial(oracle):
    rng = np.random.default_rng(11)
    L = np.array([18.0, 18.0, 18.0])
    pos = rng.uniform(0, 1, (1500, 3)) * L
    s = oracle.forces_typed(pos, L, 2.5)
    p = oracle.forces_typed(pos, L, 2.5, threads=4)
    scale = np.sqrt((s["forces"] ** 2).sum(1).mean())
    assert np.abs(p["forces"] - s["forces"]).max() <= 1e-13 * scale
    assert p["epot"] == pytest.approx(s["epot"], rel=1e-12)


def test_typed_mixture_bruteforce(oracle):
    rng = np.random.default_rng(13)
    L = np.array([14.0, 15.0, 16.0])
    pos = rng.uniform(0, 1, (800, 3)) * L
    types = (rng.uniform(size=800) < 0.2).astype(np.int32)
    eps = np.array([[1.0, 1.5], [1.5, 0.5]])
    sig = np.array([[1.0, 0.8], [0.8, 0.88]])
    rc = 2.5 * sig
    t = oracle.forces_typed(pos, L, rc, eps, sig, types, 2)
    b = oracle.forces_bruteforce(pos, L, rc, eps, sig, types, 2)
    scale = np.sqrt((b["forces"] ** 2).sum(1).mean())
    assert np.abs(t["forces"] - b["forces"]).max() <= 1e-13 * scale
    assert t["epot"] == pytest.approx(b["epot"], rel=1e-12)


def test_vv_energy_conservation(oracle):
    """FP64 velocity-Verlet over the oracle forces conserves energy closely."""
    nc, rho = 4, 0.8442
    a = (4 / rho) ** (1 / 3)
    basis = np.array([[0, 0, 0], [.5, .5, 0], [.5, 0, .5], [0, .5, .5]])
    g = np.array([[i, j, k] for k in range(nc) for j in range(nc) for i in range(nc)])
    pos = ((g[:, None, :] + basis[None]) * a).reshape(-1, 3) + 0.05
    L = np.full(3, nc * a)
    rng = np.random.default_rng(2)
    vel = rng.normal(0, np.sqrt(0.72), pos.shape)
    vel -= vel.mean(0)
    out = oracle.vv_run(pos, vel, L, 2.5, 0.002, 50)
    e = out["ekin"] + out["epot"]
    assert np.abs(e - e[0]).max() / abs(e[0]) < 2e-3


def test_vv_continues_from_given_forces(oracle):
    """A run started from a previous run's state and forces continues the same
    trajectory bit for bit (no extra force evaluation at the start)."""
    L = np.array([9.0, 9.5, 10.0])
    rng = np.random.default_rng(5)
    pos = np.stack(np.meshgrid(*[np.arange(0.3, x, 1.12) for x in L], indexing="ij"), -1).reshape(-1, 3)
    pos = (pos + rng.uniform(-0.05, 0.05, pos.shape)) % L
    vel = rng.normal(0, 0.8, pos.shape)
    whole = oracle.vv_run(pos, vel, L, 2.5, 0.004, 12)
    a = oracle.vv_run(pos, vel, L, 2.5, 0.004, 5)
    b = oracle.vv_run(a["pos"], a["vel"], L, 2.5, 0.004, 7, forces=a["forces"])
    assert np.array_equal(b["pos"], whole["pos"]) and np.array_equal(b["vel"], whole["vel"])
    assert np.array_equal(np.concatenate([a["epot"], b["epot"]]), whole["epot"])


def test_golden_fixture_typed_mixture(oracle):
    """The typed oracle reproduces its committed two-type fixture bit for bit,
    and an independent O(N^2) minimum-image sum agrees with it."""
    g = np.load(os.path.join(HERE, "golden", "oracle_typed_mixture.npz"))
    t = oracle.forces_typed(g["pos"], g["box"], g["rc"], g["eps"], g["sigma"], g["types"], 2)
    np.testing.assert_array_equal(t["forces"], g["forces"])
    assert t["epot"] == float(g["epot"]) and t["virial"] == float(g["virial"])
    assert t["counts"].candidates == int(g["candidates"]) and t["counts"].accepted == int(g["accepted"])
    b = oracle.forces_bruteforce(g["pos"], g["box"], g["rc"], g["eps"], g["sigma"], g["types"], 2)
    s = np.sqrt((g["forces"] ** 2).sum(1).mean())
    assert np.sqrt(((b["forces"] - g["forces"]) ** 2).sum(1)).max() / s <= 1e-12
    assert abs(b["epot"] - float(g["epot"])) <= 1e-12 * abs(float(g["epot"]))


def test_golden_fixture(oracle):
    g = np.load(os.path.join(HERE, "golden", "oracle_midpoint_gas.npz"))
    f, c = oracle.forces_midpoint_all(g["pos"], g["box"], float(g["cutoff"]))
    np.testing.assert_array_equal(f, g["forces"])
    assert c.candidates == int(g["candidates"]) and c.accepted == int(g["accepted"])
    t = oracle.forces_typed(g["pos"], g["box"], float(g["cutoff"]))
    assert t["epot"] == float(g["epot"]) and t["virial"] == float(g["virial"])
