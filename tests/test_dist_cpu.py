"""The multi-GPU bench path is replicas: one process per GPU, a barrier around the
timed region and the slowest rank's time (bench.py's Dist).  Run here as two gloo
ranks on the CPU: the barrier completes, the max and the sum of the ranks' values
are every rank's answer, and value = the units of all ranks / the slowest time."""
import os
import socket
import subprocess
import sys

from conftest import ROOT

SCRIPT = r"""
import os, sys, time
sys.path.insert(0, {root!r})
import bench
d = bench.Dist()
assert d.world == 2 and d.pg is not None and d.device == "cpu"
d.barrier()
ms = 100.0 + 50.0 * d.rank          # rank 1 is the slower one
slowest = d.max(ms)
units = d.sum(1000.0 * (d.rank + 1))
value = units / (slowest / 1e3)
print(f"rank {{d.rank}} slowest {{slowest}} units {{units}} value {{value}}", flush=True)
assert slowest == 150.0 and units == 3000.0
d.close()
"""


def free_port():
    with socket.socket() as sck:
        sck.bind(("127.0.0.1", 0))
        return sck.getsockname()[1]


def test_two_gloo_ranks_reduce_like_the_bench(tmp_path):
    script = tmp_path / "ranks.py"
    script.write_text(SCRIPT.format(root=ROOT))
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), str(script)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("slowest 150.0 units 3000.0") == 2
