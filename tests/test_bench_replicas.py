"""The benchmark's multi-rank host logic (replicas only: a barrier and the
max / sum over ranks) on two gloo ranks on the CPU."""
import os
import socket
import subprocess
import sys

from tests.helpers import ROOT

CHILD = r"""
import os, sys
sys.path.insert(0, {root!r})
import bench
dist = bench.dist_init()
rank = int(os.environ["RANK"])
bench.barrier(dist)
mx = bench.allmax(dist, float(rank + 1))
sm = bench.allsum(dist, 10.0 * (rank + 1))
assert mx == 2.0 and sm == 30.0, (mx, sm)
assert os.environ["CUDA_VISIBLE_DEVICES"] == str(rank)
dist.destroy_process_group()
print("ok", rank)
"""


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def test_two_rank_replica_reductions():
    port = _free_port()
    procs = []
    for r in range(2):
        env = dict(os.environ, RANK=str(r), LOCAL_RANK=str(r), WORLD_SIZE="2",
                   MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
        procs.append(subprocess.Popen([sys.executable, "-c", CHILD.format(root=ROOT)], env=env,
                                      stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True))
    outs = [p.communicate(timeout=120)[0] for p in procs]
    for r, (p, o) in enumerate(zip(procs, outs)):
        assert p.returncode == 0, o
        assert "ok %d" % r in o
