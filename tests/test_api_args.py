"""The Python layer refuses malformed arguments before it calls the library
(so on any machine, with or without a GPU), and the library refuses a
missing device cleanly: no CPU fallback."""
import pytest


def test_bad_arguments_raise_value_error(gpulib):
    L = [10.0, 10.0, 10.0]
    for kw in [dict(precision="half"), dict(pair_tables="narrow"), dict(tile_balance=2), dict(potential="morse")]:
        with pytest.raises(ValueError):
            gpulib.MidpointLJ(L, [100], **kw)
    with pytest.raises(ValueError):
        gpulib.MidpointLJ([[10.0, 10.0]], [100])  # boxes are (nboxes, 3)
    with pytest.raises(ValueError):
        gpulib.MidpointLJ([L, L], [100])  # one atom count per box
    with pytest.raises(ValueError):
        gpulib.autotune(L, [10], [[1.0, 1.0, 1.0]] * 10, tile_balance=-1)


def test_valid_arguments_reach_the_library(gpulib):
    from examd_gb300 import _lib
    ctx = None
    try:
        ctx = gpulib.MidpointLJ([10.0, 10.0, 10.0], [100], precision="mixed", tile=5, tile_balance=1)
    except gpulib.ExamdError as e:  # without an sm_103 device: the library says so
        assert e.code == _lib.ERR_NO_DEVICE
    finally:
        if ctx is not None:
            ctx.close()
