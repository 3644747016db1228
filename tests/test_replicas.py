"""Multi-GPU is replicas only: bench.py's aggregation across ranks (barrier,
max over ranks, whole-job throughput), run as world_size-2 gloo ranks on CPU."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_replicas_take_the_slowest_rank():
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()),
           str(HERE / "dist_worker.py")]
    out = subprocess.run(cmd, env=env, capture_output=True, text=True, timeout=180)
    assert out.returncode == 0, out.stderr[-2000:]
    line = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(line) == 1, out.stdout  # rank 0 alone prints
    rec = json.loads(line[0])
    assert rec["ws"] == 2
    assert rec["total"] == 2.0          # max over ranks (rank 1 took 2 s)
    assert rec["value"] == 2 * 10 / 2.0  # all units of all ranks over that time
