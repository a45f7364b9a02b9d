"""Every benchmark configuration at full size, atom by atom against the CPU
oracle (the OpenMP build of the restated exaMD_forces_midpoint_all with its
typed, energy and virial extension, all host threads):

- the 1,048,576-atom liquid at rc 2.5 and 3.0, melted on the GPU first;
- the 524,288-atom liquid slab in vapour (rc 3.0);
- the 512-box ensemble, box by box;
- the 16,777,216-atom 80:20 binary mixture (per-pair cutoffs).

For each: the FP64 form's per-atom forces within TOL64 of the oracle's
(|dF_i| / F_rms), its per-box energy and virial within the sum tolerance, its
candidate and accepted pair counts equal to the oracle's (the reference's
particle-interaction calls and accepted pairs, SRC/exaMD_forces.f90:349-377,
user_func.f90:52), and the mixed form within TOL_MIXED_RMS RMS of the oracle.

The energy and virial are sums of 10^7-10^9 FP64 pair terms taken in
different orders by the two sides; their relative difference grows like
eps * sqrt(terms) (1e-16 * sqrt(3e8) = 2e-12 for the mixture), so the sum
tolerance is 1e-12 up to 10^8 accepted pairs and eps * sqrt(pairs) * 10
above.
"""
import os

import numpy as np
import pytest

pytestmark = [pytest.mark.gpu]

TOL64 = 1e-12
TOL_MIXED_RMS = 1e-5
EPS = 2.0 ** -52


def frms(f):
    return np.sqrt((f * f).sum(1).mean())


def rel_err(f, ref):
    e = np.sqrt(((f - ref) ** 2).sum(1))
    s = frms(ref)
    return e.max() / s, np.sqrt((e * e).mean()) / s


def sum_tol(accepted):
    return max(1e-12, 10.0 * EPS * np.sqrt(float(accepted)))


def oracle_case(O, case, pos):
    """Per-box oracle results over the case's boxes: forces, epot, virial, counts."""
    lj = case["lj"]
    kw = dict(rc=lj["rc"], eps=lj.get("eps", 1.0), sigma=lj.get("sigma", 1.0), ntypes=lj.get("ntypes", 1))
    a0 = np.concatenate([[0], np.cumsum(case["natoms"])])
    t = case["types"]
    f = np.zeros_like(pos)
    ep, w = [], []
    cand = acc = 0
    threads = os.cpu_count() or 1
    for b in range(len(case["natoms"])):
        r = O.forces_typed(pos[a0[b]:a0[b + 1]], case["boxes"][b], types=None if t is None else t[a0[b]:a0[b + 1]],
                           threads=threads, **kw)
        f[a0[b]:a0[b + 1]] = r["forces"]
        ep.append(r["epot"])
        w.append(r["virial"])
        cand += r["counts"].candidates
        acc += r["counts"].accepted
    return f, np.array(ep), np.array(w), cand, acc


def gpu(gpulib, case, pos, precision, count=False):
    with gpulib.MidpointLJ(case["boxes"], case["natoms"], precision=precision, **case["lj"]) as s:
        s.set_atoms(pos, case["types"])
        f, e, w = s.forces(energy=True)
        cnt = s.counters() if count else None
    return f, e, w, cnt


def melted(gpulib, case, steps, dt):
    """The case's atoms after `steps` mixed-form velocity-Verlet steps on the GPU."""
    with gpulib.MidpointLJ(case["boxes"], case["natoms"], precision="mixed", **case["lj"]) as s:
        s.set_atoms(case["pos"], case["types"], case["vel"])
        s.run(steps, dt, graph_chunk=20)
        pos, _ = s.state()
    return pos


def check(gpulib, oracle, case, pos):
    ref_f, ref_e, ref_w, cand, acc = oracle_case(oracle, case, pos)
    f64, e64, w64, cnt = gpu(gpulib, case, pos, "fp64", count=True)
    f32, _, _, _ = gpu(gpulib, case, pos, "mixed")
    a0 = np.concatenate([[0], np.cumsum(case["natoms"])])
    # per-atom forces, norm-wise against each box's own F_rms
    worst = 0.0
    for b in range(len(case["natoms"])):
        sl = slice(a0[b], a0[b + 1])
        if a0[b + 1] > a0[b] and frms(ref_f[sl]) > 0:
            worst = max(worst, rel_err(f64[sl], ref_f[sl])[0])
    tol_sum = sum_tol(acc)
    e_rel = np.abs(e64 - ref_e) / np.maximum(np.abs(ref_e), 1e-300)
    w_rel = np.abs(w64 - ref_w) / np.maximum(np.abs(ref_w), 1e-300)
    _, rms32 = rel_err(f32, ref_f)
    print(f"\n  atoms {len(pos)}: fp64 max |dF|/Frms {worst:.2e}, energy {e_rel.max():.2e}, virial {w_rel.max():.2e} "
          f"(tol {tol_sum:.1e}); candidates {cnt['candidates']} / {cand}, accepted {cnt['accepted']} / {acc}; "
          f"mixed rms {rms32:.2e}")
    assert worst <= TOL64
    assert e_rel.max() <= tol_sum and w_rel.max() <= tol_sum
    assert cnt["candidates"] == cand and cnt["accepted"] == acc
    assert rms32 <= TOL_MIXED_RMS


@pytest.mark.parametrize("rc", [2.5, 3.0])
def test_liquid_1m(gpulib, oracle, rc):
    from examd_gb300 import workloads as W
    case = W.liquid_fcc(64, rc=rc)
    check(gpulib, oracle, case, melted(gpulib, case, 200, 0.005))


def test_slab_524k(gpulib, oracle):
    from examd_gb300 import workloads as W
    case = W.slab()
    check(gpulib, oracle, case, melted(gpulib, case, 100, 0.005))


def test_ensemble_512_boxes(gpulib, oracle):
    from examd_gb300 import workloads as W
    case = W.ensemble()
    check(gpulib, oracle, case, melted(gpulib, case, 100, 0.005))


def test_mixture_16m(gpulib, oracle):
    from examd_gb300 import workloads as W
    case = W.binary_mixture()
    check(gpulib, oracle, case, melted(gpulib, case, 100, 0.003))
