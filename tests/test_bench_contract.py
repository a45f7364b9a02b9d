"""bench.py's reference arm on the CPU: the JSON line the benchmark contract
asks of it (metric, unit and config of the GPU arm's default workload,
impl = reference, a cpu_baseline describing the run, and an e2e figure with
no host-device bytes).  The arm times the oracle's velocity-Verlet on the
1,048,576-atom liquid with all host threads."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "atom-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 1 and d["n_gpus"] == 1
    assert d["config"]["workload"] == "lj-liquid-fcc64-1048576-rc2.5" and d["config"]["atoms"] == 1048576
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert "metric" in d and d["metric"].startswith("atom-steps/s")


def test_reference_arm_other_workloads_say_unavailable():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload",
                        "slab"], capture_output=True, text=True, timeout=120, cwd=ROOT)
    assert r.returncode == 0
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith("{")][-1])
    assert d["impl"] == "reference" and "unavailable" in d


def test_gpu_arm_fails_loudly_without_a_device():
    """Without an sm_103 GPU the benchmark's own arm stops with the library's
    no-device status and prints no result line: there is no CPU fallback."""
    import ctypes as C
    from examd_gb300 import _lib
    p = _lib.Params()
    _lib.load().examd_default_params(C.byref(p))
    box = (_lib.Box * 1)()
    for a in range(3):
        box[0].L[a] = 20.0
    box[0].natoms = 10
    ctx = C.c_void_p()
    if _lib.load().examd_gpu_create(C.byref(p), 1, box, C.byref(ctx)) != _lib.ERR_NO_DEVICE:
        _lib.load().examd_gpu_destroy(ctx)
        return  # a device is present: nothing to check here
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--steps", "1", "--warmup", "3"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode != 0
    assert "no usable sm_103 CUDA device" in r.stderr
    assert not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
