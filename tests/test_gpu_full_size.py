"""Size-independent properties at the benchmark sizes (the atom-by-atom
comparison with the oracle at these sizes is in test_gpu_configs_vs_oracle.py):

- Newton's third law: the forces of each box sum to (nearly) zero;
- permutation invariance: forces follow the atoms (bit for bit in the mixed
  form, whose per-pair terms depend only on positions and whose fixed-point
  sums do not depend on the order of the terms);
- translation invariance: a shift of every atom by the same vector (modulo
  the box) leaves the forces unchanged to rounding;
- the mixed form stays within 1e-5 RMS of the FP64 form on the 16.8M-atom
  binary mixture.
"""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu]


def frms(f):
    return np.sqrt((f * f).sum(1).mean())


def rel(f, ref):
    e = np.sqrt(((f - ref) ** 2).sum(1))
    return e.max() / frms(ref), np.sqrt((e * e).mean()) / frms(ref)


@pytest.fixture(scope="module")
def liquid(gpulib):
    from examd_gb300 import workloads as W
    return W.liquid_fcc(64)  # 1,048,576 atoms, rc = 2.5


def forces(gpulib, case, pos, precision, energy=False):
    with gpulib.MidpointLJ(case["boxes"], case["natoms"], precision=precision, **case["lj"]) as s:
        s.set_atoms(pos, case["types"])
        f, e, _ = s.forces(energy=energy)
    return f, e


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-6)])
def test_total_force_vanishes(gpulib, liquid, precision, tol):
    f, _ = forces(gpulib, liquid, liquid["pos"], precision)
    total = np.abs(f.sum(0)).max()
    assert total / (len(f) * frms(f)) <= tol


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_permutation_invariance(gpulib, liquid, precision):
    perm = np.random.default_rng(5).permutation(len(liquid["pos"]))
    f, e = forces(gpulib, liquid, liquid["pos"], precision, energy=True)
    g, e2 = forces(gpulib, liquid, liquid["pos"][perm], precision, energy=True)
    if precision == "mixed":
        assert np.array_equal(g, f[perm])
        assert e2[0] == e[0]
    else:
        assert rel(g, f[perm])[0] <= 1e-13
        assert e2[0] == pytest.approx(e[0], rel=1e-13)


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-11), ("mixed", 1e-5)])
def test_translation_invariance(gpulib, liquid, precision, tol):
    L = liquid["boxes"][0]
    shifted = (liquid["pos"] + np.array([0.37, 1.11, 2.9])) % L
    f, _ = forces(gpulib, liquid, liquid["pos"], precision)
    g, _ = forces(gpulib, liquid, shifted, precision)
    assert rel(g, f)[1] <= tol


def test_mixture_16m_mixed_against_fp64(gpulib):
    """16,777,216-atom 80:20 binary mixture (rho* 1.2, per-pair cutoffs)."""
    from examd_gb300 import workloads as W
    case = W.binary_mixture()
    f32, _ = forces(gpulib, case, case["pos"], "mixed")
    f64, _ = forces(gpulib, case, case["pos"], "fp64")
    mx, rms = rel(f32, f64)
    assert rms <= 1e-5
    assert np.abs(f64.sum(0)).max() / (len(f64) * frms(f64)) <= 1e-11
