"""examd_kinetic_static: the per-box kinetic energy of atoms in the caller's own
device arrays, with scratch in a static device array instead of an allocation.

The GPU tests compare it with examd_gpu_kinetic (the context entry point) on
two calls in a row. They pass in a fresh process, where this file's first call
sets up the static array, and after the other tests. Pytest collects the file
last because of its name. The CPU test checks that oversized calls are
rejected before any CUDA call.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
TOL = 1e-12  # relative; the two paths sum the same per-atom terms in different orders


def _call(L, device, atom0, vx, vy, vz, types, mass, ekin, stream=None):
    err = C.create_string_buffer(256)
    a0 = np.ascontiguousarray(atom0, dtype=np.int64)
    m = np.ascontiguousarray(mass, dtype=np.float64)
    rc = L.examd_kinetic_static(int(device), int(a0[-1]), len(a0) - 1,
                                a0.ctypes.data_as(C.POINTER(C.c_int64)), vx, vy, vz, types, len(m),
                                m.ctypes.data_as(C.POINTER(C.c_double)),
                                ekin.ctypes.data_as(C.POINTER(C.c_double)), stream, err, len(err))
    return rc, err.value.decode()


def test_header_limits_match_loader(gpulib):
    from examd_gb300 import _lib
    src = open(os.path.join(ROOT, "include", "examd_gb300.h")).read()
    assert int(re.search(r"#define EXAMD_STATIC_MAX_ATOMS (\d+)", src).group(1)) == _lib.STATIC_MAX_ATOMS
    assert int(re.search(r"#define EXAMD_STATIC_MAX_BOXES (\d+)", src).group(1)) == _lib.STATIC_MAX_BOXES


def test_oversized_calls_rejected_before_device_work(gpulib):
    """Sizes beyond the static scratch are refused on the host with a clear reason."""
    from examd_gb300 import _lib
    L = _lib.load()
    ek = np.zeros(1)
    n = _lib.STATIC_MAX_ATOMS + 1
    rc, msg = _call(L, 0, [0, n], None, None, None, None, [1.0], ek)
    assert rc == _lib.ERR_ARG and "static scratch limit" in msg and str(_lib.STATIC_MAX_ATOMS) in msg
    nb = _lib.STATIC_MAX_BOXES + 1
    ekb = np.zeros(nb)
    rc, msg = _call(L, 0, np.zeros(nb + 1, dtype=np.int64), None, None, None, None, [1.0], ekb)
    assert rc == _lib.ERR_ARG and "static scratch limit" in msg and str(_lib.STATIC_MAX_BOXES) in msg
    rc, msg = _call(L, 0, [0, 2, 0], None, None, None, None, [1.0], np.zeros(2))
    assert rc == _lib.ERR_ARG and "atom0" in msg


def _two_boxes(gl):
    boxes = np.array([[12.0, 12.0, 12.0], [13.0, 12.0, 14.0]])
    counts = [900, 1100]
    rng = np.random.default_rng(11)
    pos = np.concatenate([gl.gen_random(n, b, 0.8, 5 + k) for k, (n, b) in enumerate(zip(counts, boxes))])
    types = (rng.random(sum(counts)) < 0.3).astype(np.int32)
    mass = np.array([1.0, 2.5])
    vel = gl.gen_velocities(sum(counts), 1.3, 17, types=types, mass=mass)
    return boxes, counts, pos, types, mass, vel


@pytest.mark.gpu
def test_matches_context_entry_point_twice(gpulib):
    import torch
    from examd_gb300 import _lib
    L = _lib.load()
    boxes, counts, pos, types, mass, vel = _two_boxes(gpulib)
    with gpulib.MidpointLJ(boxes, counts, ntypes=2, mass=mass, rc=2.5) as s:
        s.set_atoms(pos, types, vel)
        ref = s.kinetic()
    host = np.array([0.5 * (mass[types[a0:a1]] * (vel[a0:a1] ** 2).sum(1)).sum()
                     for a0, a1 in zip([0, counts[0]], [counts[0], sum(counts)])])
    dev = torch.device("cuda:0")
    v = [torch.tensor(np.ascontiguousarray(vel[:, a]), device=dev) for a in range(3)]
    t = torch.tensor(types, device=dev)
    atom0 = [0, counts[0], sum(counts)]
    stream = C.c_void_p(torch.cuda.current_stream(dev).cuda_stream)
    torch.cuda.synchronize(dev)
    out = []
    for _ in range(2):
        ek = np.zeros(2)
        rc, msg = _call(L, 0, atom0, v[0].data_ptr(), v[1].data_ptr(), v[2].data_ptr(), t.data_ptr(), mass, ek,
                        stream)
        assert rc == _lib.OK, msg
        out.append(ek)
    assert np.array_equal(out[0], out[1])
    np.testing.assert_allclose(out[0], ref, rtol=TOL, atol=0)
    np.testing.assert_allclose(out[0], host, rtol=TOL, atol=0)


@pytest.mark.gpu
def test_bad_type_reported_and_status_cleared(gpulib):
    """An out-of-range type sets the status word; the next call starts from zero."""
    import torch
    from examd_gb300 import _lib
    L = _lib.load()
    dev = torch.device("cuda:0")
    n = 1000
    vel = gpulib.gen_velocities(n, 1.0, 3)
    v = [torch.tensor(np.ascontiguousarray(vel[:, a]), device=dev) for a in range(3)]
    bad = torch.zeros(n, dtype=torch.int32, device=dev)
    bad[n // 2] = 3
    torch.cuda.synchronize(dev)
    ek = np.zeros(1)
    rc, msg = _call(L, 0, [0, n], v[0].data_ptr(), v[1].data_ptr(), v[2].data_ptr(), bad.data_ptr(), [1.0, 2.0],
                    ek)
    assert rc == _lib.ERR_ARG and "type" in msg
    rc, msg = _call(L, 0, [0, n], v[0].data_ptr(), v[1].data_ptr(), v[2].data_ptr(), None, [1.0], ek)
    assert rc == _lib.OK, msg
    assert ek[0] == pytest.approx(0.5 * (vel ** 2).sum(), rel=TOL)


@pytest.mark.gpu
def test_host_pointer_rejected(gpulib):
    """Velocity arrays that are not device memory are refused before any launch."""
    from examd_gb300 import _lib
    L = _lib.load()
    vel = np.zeros((3, 64))
    ek = np.zeros(1)
    p = [vel[a].ctypes.data for a in range(3)]
    rc, msg = _call(L, 0, [0, 64], p[0], p[1], p[2], None, [1.0], ek)
    assert rc == _lib.ERR_ARG and "device memory" in msg
