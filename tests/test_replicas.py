"""Replicas for N > 1 (the path does not shard: one independent block per
rank, no data-path collective): the timing reduction and the whole-job
aggregate of bench.py on a 2-rank gloo group, and the reference arm's
rank-0-only output, all on CPU."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.reduce_max(dist, 100.0 + 25.0 * rank, "cpu")  # the slowest rank sets the job time
    rate = bench.aggregate_rate(world, 1_000_000, 5, ms)
    dist.barrier()
    dist.destroy_process_group()
    Path(out, f"r{rank}.json").write_text(json.dumps({"ms": ms, "rate": rate}))


def test_two_rank_reduction_and_aggregate(tmp_path):
    import torch.multiprocessing as tmp

    port = 29511 + os.getpid() % 1000
    tmp.spawn(_worker, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r = [json.loads((tmp_path / f"r{k}.json").read_text()) for k in range(2)]
    assert r[0]["ms"] == r[1]["ms"] == 125.0
    # 2 ranks x 1e6 cells x 5 steps in 0.125 s
    assert r[0]["rate"] == pytest.approx(2 * 1e6 * 5 / 0.125 / 1e6)


def test_single_process_reduction_is_identity():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.reduce_max(None, 3.5, "cpu") == 3.5


def test_reference_arm_other_ranks_print_nothing(tmp_path):
    """Under torchrun every rank but 0 exits 0 without output (the reference arm
    runs on rank 0 only)."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    out = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2", "--steps",
                          "1", "--warmup", "0"], capture_output=True, text=True, env=env, timeout=120)
    assert out.returncode == 0, out.stderr
    assert out.stdout.strip() == ""
