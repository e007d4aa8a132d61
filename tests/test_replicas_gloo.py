"""The multi-rank form of the benchmark on the CPU (world size 2, gloo):
replicas share nothing on the data path, and the step time of the job is
the slowest replica's (max over ranks)."""
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CHILD = r"""
import os, sys
sys.path.insert(0, os.environ["ROOT"])
import torch.distributed as dist
import bench
dist.init_process_group("gloo")
rank = dist.get_rank()
ms = [12.5, 17.25][rank]
got = bench.replica_time(ms, dist, "cpu")
assert got == 17.25, got
assert bench.replica_time(3.0, None, "cpu") == 3.0
dist.barrier()
dist.destroy_process_group()
print("rank", rank, "ok")
"""


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_replica_time_is_the_max_over_ranks():
    port = _port()
    procs = []
    for rank in range(2):
        env = dict(os.environ, ROOT=ROOT, RANK=str(rank), WORLD_SIZE="2",
                   LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                   MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD], env=env,
                                      stdout=subprocess.PIPE,
                                      stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate(timeout=120)[0] for p in procs]
    for rank, (p, out) in enumerate(zip(procs, outs)):
        assert p.returncode == 0, out
        assert "rank %d ok" % rank in out
