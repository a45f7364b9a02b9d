"""The split of each box axis into tiles (examd_params.tile_balance): 0 by
cell count, 1 by width, where the box's last cell, which absorbs the
remainder of L / edge, counts as two when it is at least 1.5 edges wide.
Either way every cell pair is evaluated once by the cell the reference's
table assigns it to, so the candidate and accepted counts are the
reference's and the forces agree: to 1e-12 in the FP64 form, and within the
mixed form's FP32 rounding of tile-frame coordinates otherwise."""
import numpy as np
import pytest

pytestmark = [pytest.mark.gpu]

L = np.array([19.4, 18.8, 20.7])  # 15.52, 15.04 and 16.56 cell edges of 1.25: wide last cells in x and z


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-5)])
def test_split_by_width_same_pairs_and_forces(gpulib, precision, tol):
    pos = gpulib.gen_random(6000, L, 0.8, 5)
    out = {}
    for tb in (0, 1):
        with gpulib.MidpointLJ(L, [len(pos)], precision=precision, rc=2.5, tile=5, tile_balance=tb) as s:
            s.set_atoms(pos)
            f, e, w = s.forces(energy=True)
            out[tb] = (f, e, w, s.counters())
    (f0, e0, w0, c0), (f1, e1, w1, c1) = out[0], out[1]
    # x: 15 cells in 3 tiles of 5 -> 4 tiles of 4, 4, 4, 3 + the wide cell; y unchanged; z likewise
    assert c1["tiles"] > c0["tiles"] and c1["max_tile_atoms"] < c0["max_tile_atoms"]
    assert c0["candidates"] == c1["candidates"] and c0["accepted"] == c1["accepted"]
    frms = np.sqrt((f0 * f0).sum(1).mean())
    err = np.sqrt(((f1 - f0) ** 2).sum(1))
    if precision == "fp64":
        assert err.max() / frms <= tol
    else:
        assert np.sqrt((err * err).mean()) / frms <= tol
    assert abs(e1[0] - e0[0]) <= tol * abs(e0[0]) and abs(w1[0] - w0[0]) <= tol * abs(w0[0])


def test_bad_split_choice(gpulib):
    with pytest.raises(ValueError):
        gpulib.MidpointLJ(L, [100], precision="mixed", tile_balance=2)
