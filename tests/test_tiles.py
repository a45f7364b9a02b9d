"""The split of a box axis into CTA tiles (examd_tile_split, the rule that
examd_gpu_create applies per axis), checked on the CPU: tiles of at most the
tile length and at least 2 cells, an even split by cell count, and with
tile_balance = 1 one cell fewer in the tile that holds a last cell of 1.5
edges or more (the cell that absorbs the remainder of L / edge)."""
import numpy as np
import pytest

from examd_gb300 import _lib


def test_liquid_axis(gpulib):
    # 1,048,576-atom liquid: L = 107.49, edge 1.25 -> 85 cells, the last 1.995 edges wide
    assert np.array_equal(gpulib.tile_split(85, 1.995, 5, 0), np.arange(0, 86, 5))
    even = gpulib.tile_split(85, 1.995, 6, 0)
    wide = gpulib.tile_split(85, 1.995, 6, 1)
    assert len(even) == len(wide) == 16  # 15 tiles either way
    assert even[-1] - even[-2] == 6 and wide[-1] - wide[-2] == 5  # the wide cell's tile
    assert np.diff(wide).max() == 6 and np.diff(wide).min() == 5


@pytest.mark.parametrize("balance", [0, 1])
def test_split_properties(gpulib, balance):
    for nb in range(5, 260):
        for T in range(2, 9):
            for w in (1.0, 1.3, 1.5, 1.8, 1.999):
                st = gpulib.tile_split(nb, w, T, balance)
                nt = len(st) - 1
                sz = np.diff(st)
                assert st[0] == 0 and st[-1] == nb and sz.min() >= 2, (nb, T, w)
                nv = nb + (1 if balance and w >= 1.5 else 0)
                assert nt == max(1, min(nb // 2, -(-nv // T)))
                if nv == nb:  # the even split by cell count
                    assert np.array_equal(st, np.arange(nt + 1) * nb // nt)
                    if nt < nb // 2:
                        assert sz.max() <= T
                elif not np.array_equal(st, np.arange(nt + 1) * nb // nt):
                    # by width: the wide cell's tile is the shortest, and counting that cell
                    # as two it is no longer than T, as are the others
                    assert sz[-1] == sz.min(), (nb, T, w)
                    if nt < nb // 2:
                        assert sz.max() <= T and sz[-1] + 1 <= T, (nb, T, w)


def test_bad_arguments(gpulib):
    import ctypes as C
    L = _lib.load()
    st = (C.c_int * 600)()
    nt = C.c_int()
    for args in [(0, 1.0, 4, 0), (1024, 1.0, 4, 0), (20, 2.0, 4, 0), (20, 0.5, 4, 0), (20, 1.0, 0, 0),
                 (20, 1.0, 4, 2)]:
        assert L.examd_tile_split(*args, st, C.byref(nt)) == _lib.ERR_ARG, args
    assert L.examd_tile_split(20, 1.0, 4, 0, None, C.byref(nt)) == _lib.ERR_ARG
