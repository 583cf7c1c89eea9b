"""The replicas path of bench.py on CPU: two gloo ranks aggregate their step
times the way the GPU ranks do (max over ranks, whole-job throughput)."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

RANK_SCRIPT = r"""
import json, os, sys
sys.path.insert(0, os.environ["EG_ROOT"])
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank, world = dist.get_rank(), dist.get_world_size()
ms = [10.0, 25.0][rank]
mx = bench.reduce_max_ms(ms, world, "cpu")
print(json.dumps({"rank": rank, "ms": mx, "tflops": bench.job_tflops(1e12, mx, world)}))
dist.destroy_process_group()
"""


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_two_gloo_ranks_take_the_slowest_time():
    port = free_port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, EG_ROOT=ROOT, RANK=str(rank), WORLD_SIZE="2", MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", RANK_SCRIPT], env=env, stdout=subprocess.PIPE,
                                      stderr=subprocess.PIPE, text=True))
    outs = []
    for p in procs:
        out, err = p.communicate(timeout=120)
        assert p.returncode == 0, err
        outs.append(json.loads(out.strip().splitlines()[-1]))
    for o in outs:
        assert o["ms"] == 25.0  # the slower rank's time
        assert abs(o["tflops"] - 2 * 1e12 / 25e-3 / 1e12) < 1e-9  # both ranks' work over that time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max_ms(7.5, 1, "cpu") == 7.5
    assert abs(bench.job_tflops(2e12, 10.0, 1) - 200.0) < 1e-9
