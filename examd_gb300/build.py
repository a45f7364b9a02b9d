"""Build recipe of the CUDA library: nvcc, sm_103a only, in-tree output.

    python -m examd_gb300.build            # -> examd_gb300/_lib/libexamd_gb300.so
    python -m examd_gb300.build --checked  # -> examd_gb300/_lib/libexamd_gb300_checked.so

Each translation unit is compiled in parallel; the shared object links the
CUDA runtime statically so that the library carries no dependency on torch.
The checked build (-DEXAMD_CHECKED) tests every shared-memory and global
index of the pair, binning-scatter and kick kernels against its array and
reports a failure as EXAMD_ERR_CHECK; the loader takes it when the
environment has EXAMD_CHECKED=1.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
OBJ_DIR = os.path.join(HERE, "_lib", "obj")
LIB = os.path.join(OUT_DIR, "libexamd_gb300.so")
LIB_CHECKED = os.path.join(OUT_DIR, "libexamd_gb300_checked.so")
OBJ_DIR_CHECKED = os.path.join(HERE, "_lib", "obj_checked")
SOURCES = ["api.cu", "bin.cu", "pair.cu", "step.cu", "static_kinetic.cu", "gen.cpp", "io.cpp", "tune.cpp"]
HEADERS = ["common.cuh", "kernels.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
            "--expt-relaxed-constexpr", *ARCH, *extra]


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    deps = [src] + [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(HERE, "..", "include", "examd_gb300.h")]
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(force: bool = False, verbose: bool = False, extra=(), checked: bool = False) -> str:
    obj_dir = OBJ_DIR_CHECKED if checked else OBJ_DIR
    lib = LIB_CHECKED if checked else LIB
    if checked:
        extra = (*extra, "-DEXAMD_CHECKED")
    os.makedirs(obj_dir, exist_ok=True)
    cc = nvcc()
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(obj_dir, s + ".o")
        if force or _stale(obj, src):
            jobs.append([cc, *_flags(extra), "-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr, flush=True)

    if jobs:
        with ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
            list(ex.map(run, jobs))
    objs = [os.path.join(obj_dir, s + ".o") for s in SOURCES]
    if force or jobs or not os.path.exists(lib):
        tmp = lib + ".tmp"
        run([cc, "-shared", *ARCH, "-o", tmp, *objs, "-cudart", "static"])
        os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv, checked="--checked" in sys.argv))
