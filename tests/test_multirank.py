"""The multi-rank (replicas) path of bench.py on the host: two gloo ranks.

Within one mesh nothing is exchanged, so N GPUs run N replicas and the job's
time is its slowest rank's (max over ranks); rank 0 alone reports.  These
tests run that logic with world_size 2 over gloo on CPU, and the reference
arm under torchrun with two ranks (rank 0 alone measures and prints)."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, out_dir: str):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    r, lr, w = bench.dist_env()
    got = bench.max_over_ranks(10.0 * (rank + 1), w)
    dist.barrier()
    with open(os.path.join(out_dir, "rank%d.json" % rank), "w") as f:
        json.dump({"rank": r, "local_rank": lr, "world": w, "max": got}, f)
    dist.destroy_process_group()


def test_max_over_ranks_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    for rank in (0, 1):
        d = json.loads((tmp_path / ("rank%d.json" % rank)).read_text())
        assert d == {"rank": rank, "local_rank": rank, "world": 2, "max": 20.0}


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5


def test_reference_arm_under_two_ranks_prints_one_line(oracle_lib, tmp_path):
    """torchrun with two ranks: rank 0 times the reference algorithm on the
    host cores and prints the one JSON line; rank 1 exits without work."""
    port = _free_port()
    env = dict(os.environ, HAMSTR_BENCH_DIR=str(tmp_path), OMP_NUM_THREADS="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), "bench.py", "--impl", "reference",
           "--workload", "c1", "--steps", "1", "--warmup", "1"]
    out = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0 and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0
