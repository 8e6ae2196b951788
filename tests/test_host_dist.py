"""The multi-rank host logic of bench.py on the CPU (no GPU).

The path does not shard: with N ranks each runs its own replica, and the
whole-job figure is N times the rate of the slowest rank.  Two ranks over
the gloo backend (127.0.0.1) check the max-over-ranks reduction the GPU arm
applies to every timed region, and bench.py's reference arm launched by
torch.distributed.run with two ranks checks that rank 0 alone prints its one
JSON line and that every rank exits 0.
"""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE="2")
    dist.init_process_group("gloo", rank=rank, world_size=2)
    sys.path.insert(0, ROOT)
    import bench
    # each rank's timed region: rank 1 is the slower one
    got = bench.max_over_ranks(10.0 + 7.5 * rank, 2, torch.device("cpu"))
    one = bench.max_over_ranks(3.0, 1, torch.device("cpu"))
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"max": got, "single": one}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo(tmp_path):
    port = _free_port()
    torch.multiprocessing.spawn(_rank, args=(port, str(tmp_path)), nprocs=2, join=True)
    for r in range(2):
        d = json.load(open(tmp_path / f"rank{r}.json"))
        assert d["max"] == 17.5 and d["single"] == 3.0


def test_reference_arm_under_torchrun_prints_once():
    """bench.py --impl reference as the driver launches it for N = 2: rank 0
    runs the CPU reference step on a bounded sample and prints one line with
    impl "reference"; rank 1 exits 0 without output."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py",
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
           "--workload", "melt10k"]
    res = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [l for l in res.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, res.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["cores"] >= 1
