"""The multi-rank path of bench.py on CPU (gloo, world size 2): the maximum
of the ranks' times that the timed region reports, and the reference arm
under torchrun, where rank 0 alone times the CPU path and prints one line."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

WORKER = r"""
import os, sys
sys.path.insert(0, sys.argv[1])
import bench
d = bench.Dist(None, backend="gloo")
d.barrier()
x = d.max(1.5 + d.rank)
d.barrier()
with open(os.path.join(sys.argv[2], "rank%d.txt" % d.rank), "w") as f:
    f.write("max %r" % x)
d.close()
"""


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _run_two(args, timeout=300):
    env = dict(os.environ, MASTER_ADDR="127.0.0.1", OMP_NUM_THREADS="2")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(_port())] + args
    return subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True,
                          timeout=timeout)


def test_max_over_ranks_gloo(tmp_path):
    pytest.importorskip("torch")
    w = tmp_path / "worker.py"
    w.write_text(WORKER)
    r = _run_two([str(w), ROOT, str(tmp_path)])
    assert r.returncode == 0, r.stderr[-2000:]
    for rank in (0, 1):
        assert (tmp_path / f"rank{rank}.txt").read_text() == "max 2.5"


def test_reference_arm_prints_once_under_torchrun():
    pytest.importorskip("torch")
    r = _run_two(["bench.py", "--impl", "reference", "--level", "3", "--steps", "2",
                  "--warmup", "3", "--gpus", "2"], timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
