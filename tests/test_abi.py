"""The C ABI library loads without a GPU and exports every symbol include/*.h declares."""
import glob
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names |= set(re.findall(r"\b(examd_\w+)\s*\(", src))
    return names


def test_exports_every_declared_symbol(gpulib):
    from examd_gb300 import _lib
    L = _lib.load()
    names = declared()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_strerror_and_defaults(gpulib):
    import ctypes as C
    from examd_gb300 import _lib
    L = _lib.load()
    assert b"5 cells" in L.examd_gpu_strerror(_lib.ERR_NB_TOO_SMALL)
    p = _lib.Params()
    L.examd_default_params(C.byref(p))
    assert p.ntypes == 1 and p.rc[0] == 2.5 and p.eps[0] == 1.0 and p.precision == _lib.FP64


def test_error_codes_match_header(gpulib):
    """Every EXAMD_ERR_* of the header has the same value in the Python layer
    and a message of its own."""
    from examd_gb300 import _lib
    L = _lib.load()
    src = open(os.path.join(ROOT, "include", "examd_gb300.h")).read()
    codes = dict(re.findall(r"#define EXAMD_(ERR_\w+)\s+(\d+)", src))
    assert len(codes) >= 12
    for name, val in codes.items():
        assert getattr(_lib, name) == int(val), name
        assert L.examd_gpu_strerror(int(val)) != b"unknown status", name


def test_host_generators(gpulib):
    pos, L = gpulib.gen_fcc(3, 0.8442)
    assert pos.shape == (108, 3) and abs(L - 3 * (4 / 0.8442) ** (1 / 3)) < 1e-12
    v = gpulib.gen_velocities(108, 0.72, 1)
    assert np.abs(v.sum(0)).max() < 1e-12
    assert abs((v * v).sum() / (3 * 107) - 0.72) < 1e-12
    p = gpulib.gen_random(200, [10.0, 11.0, 12.0], 0.8, 7)
    d = p[None] - p[:, None]
    d -= np.round(d / np.array([10.0, 11.0, 12.0])) * np.array([10.0, 11.0, 12.0])
    r = np.sqrt((d * d).sum(-1)) + np.eye(200) * 10
    assert r.min() >= 0.8
    q, t, Lq = gpulib.gen_jittered_sc(6, 1.2, 0.1, 0.2, 3)
    assert q.shape == (216, 3) and set(np.unique(t)) <= {0, 1}


def test_no_device_is_reported(gpulib):
    """On a machine without an sm_103 GPU, create fails cleanly (no CPU fallback)."""
    import ctypes as C
    from examd_gb300 import _lib
    L = _lib.load()
    if L is None:
        return
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = False
    if has_gpu:
        return
    p = _lib.Params()
    L.examd_default_params(C.byref(p))
    box = (_lib.Box * 1)()
    for a in range(3):
        box[0].L[a] = 20.0
    box[0].natoms = 10
    ctx = C.c_void_p()
    assert L.examd_gpu_create(C.byref(p), 1, box, C.byref(ctx)) == _lib.ERR_NO_DEVICE


def test_struct_layouts_match_header(tmp_path):
    """The ctypes mirrors of examd_params, examd_box and examd_stats have the
    C structs' sizes and field offsets (compiled from the header with gcc)."""
    import ctypes as C
    import shutil
    import subprocess
    from examd_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    structs = {"examd_params": _lib.Params, "examd_box": _lib.Box, "examd_stats": _lib.Stats}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "examd_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for f in py._fields_:
            lines.append(f'  printf("{cname}.{f[0]} %zu\\n", offsetof({cname}, {f[0]}));')
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = dict(ln.split() for ln in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for f in py._fields_:
            assert int(got[f"{cname}.{f[0]}"]) == getattr(py, f[0]).offset, f"{cname}.{f[0]}"
