"""Measured issue rates of the pipes the pair kernel uses (FP32 FMA, FP64 FMA,
shared-memory atomics), on the GPU the library runs on.

    python -m examd_gb300.peaks        # builds csrc/pipe_rates.cu, prints one JSON line

The FP32 FMA rate is the denominator of the pair kernel's roofline fraction:
the kernel is bound by CUDA-core FP32 issue, not by HBM and not by tensor cores.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

from . import build as B

SRC = os.path.join(B.CSRC, "pipe_rates.cu")
EXE = os.path.join(B.OUT_DIR, "pipe_rates")


def build_probe() -> str:
    os.makedirs(B.OUT_DIR, exist_ok=True)
    if not os.path.exists(EXE) or os.path.getmtime(EXE) < os.path.getmtime(SRC):
        r = subprocess.run([B.nvcc(), "-O3", "-std=c++17", *B.ARCH, SRC, "-o", EXE], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{r.stdout}\n{r.stderr}")
    return EXE


def measure() -> dict:
    r = subprocess.run([build_probe()], capture_output=True, text=True, timeout=120)
    if r.returncode != 0:
        raise RuntimeError(f"pipe_rates failed: {r.stderr.strip()}")
    return json.loads(r.stdout.strip().splitlines()[-1])


if __name__ == "__main__":
    out = measure()
    print(json.dumps(out))
    sys.exit(0)
