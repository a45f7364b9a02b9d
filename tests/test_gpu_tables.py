"""The mixed form's two layouts of the pair kernel's per-warp tables (wide:
full-width item offsets and x-gaps; compact: 16-bit offsets and FP16 x-gaps
rounded toward zero, chosen where it fits more CTAs on an SM).  The compact
gaps can only prune fewer cells, never more, so the accepted pairs and the
exact fixed-point force sums are the same bit for bit."""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu]


def cases():
    from examd_gb300 import workloads as W
    return {"liquid": lambda: W.liquid_fcc(16),             # 16,384 atoms, one type
            "mixture": lambda: W.binary_mixture(m=32),      # 32,768 atoms, two types
            "ensemble": lambda: W.ensemble(nboxes=24, seed=9)}


@pytest.mark.parametrize("name", ["liquid", "mixture", "ensemble"])
def test_wide_and_compact_tables_agree(gpulib, name):
    c = cases()[name]()
    out = {}
    for tables in ("wide", "compact", "auto"):
        with gpulib.MidpointLJ(c["boxes"], c["natoms"], precision="mixed", pair_tables=tables, **c["lj"]) as s:
            s.set_atoms(c["pos"], c["types"])
            f, e, w = s.forces(energy=True)
            out[tables] = (f, e, w, s.counters())
    fw, ew, ww, cw = out["wide"]
    for tables in ("compact", "auto"):
        f, e, w, cnt = out[tables]
        assert np.array_equal(f, fw), tables
        assert np.array_equal(e, ew) and np.array_equal(w, ww), tables
        assert cnt["accepted"] == cw["accepted"] and cnt["candidates"] == cw["candidates"], tables
        assert cnt["evaluated"] >= cw["evaluated"], tables


def test_bad_table_choice(gpulib):
    with pytest.raises(ValueError):
        gpulib.MidpointLJ([10.0, 10.0, 10.0], [100], precision="mixed", pair_tables="narrow")
