"""bench.py's reference arm on the CPU: the JSON line the benchmark contract
asks of it (metric, unit, impl = reference, a cpu_baseline describing the run,
an e2e figure with no host-device bytes, and the same `config` object as the
GPU arm on the same workload), for more than the default workload; and that
its process loads no library of the product."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def _ref_line(*extra, timeout=900):
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", *extra],
                       capture_output=True, text=True, timeout=timeout, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    return json.loads(lines[0])


def test_default_workload_is_the_largest_configuration():
    """The --gpus 1 line runs the 16,777,216-atom binary mixture: the largest
    configuration of the metric that fits one GPU."""
    import bench
    assert bench.DEFAULT_WORKLOAD == "mixture"
    w = bench.WORKLOADS["mixture"]
    assert w["gen"] == "binary_mixture" and w["args"]["m"] ** 3 == 16777216 and w["dt"] == 0.003


def test_reference_arm_line_same_config_as_gpu_arm():
    import bench
    for wl, steps in (("fcc32k", 2), ("liquid", 1)):
        d = _ref_line("--workload", wl, "--steps", str(steps), "--warmup", "3")
        assert d["impl"] == "reference" and d["unit"] == "atom-steps/s" and d["higher_is_better"] is True
        assert d["value"] > 0 and d["steps"] == steps and d["n_gpus"] == 1 and d["warmup"] == 3
        # the GPU arm prints config_of(workload, case) for the same generated case
        assert d["config"] == json.loads(json.dumps(bench.config_of(wl, bench.make_case(wl))))
        cb = d["cpu_baseline"]
        assert cb["value"] == d["value"] and cb["kind"] == "port" and cb["cores"] >= 1 and cb["sample"]
        assert d["e2e"] == {"value": d["value"], "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                            "d2h_bytes_per_step": 0}
        assert d["metric"] == bench.METRIC


SCRIPT = r"""
import json, os, sys
sys.path.insert(0, os.environ["EXAMD_ROOT"])
import bench
class A:
    workload = "fcc32k"; warmup = 3; steps = 1; gpus = 1
bench.run_reference(A, 1, 0)
maps = open("/proc/self/maps").read()
print(json.dumps({"pkg": [m for m in sys.modules if m.startswith("examd_gb300")],
                  "lib": "libexamd_gb300" in maps, "oracle": "libexamd_oracle" in maps}))
"""


def test_reference_arm_loads_no_product_library():
    r = subprocess.run([sys.executable, "-c", SCRIPT], capture_output=True, text=True, timeout=600, cwd=ROOT,
                       env=dict(os.environ, EXAMD_ROOT=ROOT))
    assert r.returncode == 0, r.stderr[-2000:]
    d = json.loads([ln for ln in r.stdout.splitlines() if ln.startswith('{"pkg"')][-1])
    assert d == {"pkg": [], "lib": False, "oracle": True}


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
