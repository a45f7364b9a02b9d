"""The checked build (-DEXAMD_CHECKED): every shared-memory and global index
of the pair kernels (enumeration, list build and list pass), the
binning-scatter and the kick is tested against its array;
a failure sets a status bit (the access goes to element 0 instead) and the
call returns EXAMD_ERR_CHECK, with no trap.  It stands in for a memory
checker, which may not run on this GPU pool.

The small parity tests run here a second time, in a child process that loads
the checked library (EXAMD_CHECKED=1): any index outside its array would make
a call fail with EXAMD_ERR_CHECK, and the results must still match the
oracle and the FP64 path as in the normal build.
"""
import os
import subprocess
import sys

import pytest

pytestmark = [pytest.mark.gpu]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SMALL = ["tests/test_gpu_parity.py", "tests/test_gpu_golden.py", "tests/test_gpu_close_pairs.py",
         "tests/test_gpu_tables.py", "tests/test_gpu_potentials.py", "tests/test_gpu_io_graph.py",
         "tests/test_gpu_tile_balance.py", "tests/test_gpu_pair_list.py"]


@pytest.fixture(scope="module")
def checked_env(gpulib):
    from examd_gb300 import build as B
    B.build(checked=True)
    return dict(os.environ, EXAMD_CHECKED="1")


def test_checked_library_is_the_one_loaded(checked_env):
    r = subprocess.run([sys.executable, "-c", "from examd_gb300 import _lib; print(_lib.load()._name)"],
                       cwd=ROOT, env=checked_env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip().endswith("libexamd_gb300_checked.so")


def test_small_parity_tests_under_the_checked_build(checked_env):
    r = subprocess.run([sys.executable, "-m", "pytest", "-q", "-x", "-m", "gpu", "-p", "no:cacheprovider", *SMALL],
                       cwd=ROOT, env=checked_env, capture_output=True, text=True, timeout=1800)
    assert r.returncode == 0, r.stdout[-4000:] + r.stderr[-2000:]
    assert " passed" in r.stdout and "failed" not in r.stdout
