"""The N > 1 path of bench.py on CPU: independent replicas joined by a gloo
barrier and a max over ranks of the timed region (no data-path collective).
Two ranks run as separate processes on 127.0.0.1."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, os.environ["EXAMD_ROOT"])
import bench
ws, rk, lr = bench.dist_info()
dist = bench.init_pg(ws)
bench.barrier(dist)
t_local = 10.0 + rk          # this rank's timed region, ms
t = bench.allmax(dist, t_local)
n, steps = 1000, 5
value = n * steps * ws / (t * 1e-3)  # whole-job atom-steps/s, as bench.py reports it

class A:  # the reference arm's arguments; rank 1 must return without work or output
    workload = "liquid"; warmup = 3; steps = 1; gpus = ws
if rk != 0:
    bench.run_reference(A, ws, rk)
bench.barrier(dist)
print(json.dumps({"rank": rk, "ws": ws, "t": t, "value": value}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_replicas_barrier_and_max():
    port = free_port()
    procs = []
    for rk in range(2):
        env = dict(os.environ, RANK=str(rk), LOCAL_RANK=str(rk), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port), EXAMD_ROOT=ROOT)
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=180)
        assert p.returncode == 0, err
        lines = [l for l in out.splitlines() if l.startswith("{")]
        assert len(lines) == 1, out  # rank 1's reference arm printed nothing
        outs.append(json.loads(lines[0]))
    assert {o["rank"] for o in outs} == {0, 1}
    for o in outs:
        assert o["ws"] == 2 and o["t"] == 11.0  # max over ranks
        assert o["value"] == 1000 * 5 * 2 / 11e-3
