"""The multi-process path of bench.py on CPU (gloo, world size 2): every
rank times its own replica, the job time is the maximum over ranks, and only
rank 0 prints.  Runs without a GPU."""
import json
import os
import socket
import subprocess
import sys

import pytest

from helpers import ROOT

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE="2",
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, ws, _ = bench.dist_init()
    assert (r, ws) == (rank, 2)
    bench.barrier(ws)
    m = bench.allmax(1.5 + rank, ws)
    with open(out, "a") as f:
        f.write(f"{rank} {m}\n")
    torch.distributed.destroy_process_group()


def test_allmax_over_gloo_ranks(tmp_path):
    out = str(tmp_path / "out.txt")
    torch.multiprocessing.spawn(_worker, args=(_free_port(), out), nprocs=2, join=True)
    lines = sorted(open(out).read().split("\n")[:-1])
    assert lines == ["0 2.5", "1 2.5"]


def test_reference_arm_under_torchrun_prints_once(tmp_path):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--workload", "small", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=str(tmp_path))
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
