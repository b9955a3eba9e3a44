"""bench.py's multi-rank plumbing on CPU (gloo, world size 2): the max over
ranks of the per-rank step time, the whole-job replica throughput, and the
reference arm under torchrun (rank 0 prints one line, rank 1 exits 0)."""
import json
import os
import socket
import subprocess
import sys

import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
import bench  # noqa: E402


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        ms = bench.max_over_ranks(1.5 + rank, world, "cpu")
        with open(os.path.join(out_dir, "r%d" % rank), "w") as f:
            f.write(repr(ms))
    finally:
        torch.distributed.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    mp.spawn(_rank_main, args=(2, free_port(), str(tmp_path)), nprocs=2, join=True)
    got = [float(open(tmp_path / ("r%d" % r)).read()) for r in range(2)]
    assert got == [2.5, 2.5]


def test_replica_throughput_is_whole_job():
    assert bench.max_over_ranks(3.25, 1, "cpu") == 3.25
    assert bench.replica_throughput(1000, 4, 2.0) == 4 * 1000 / 2e-3


def test_reference_arm_two_ranks():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port()), "bench.py", "--impl", "reference",
           "--gpus", "2", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["value"] == d["value"]
