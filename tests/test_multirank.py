"""The N > 1 benchmark path on CPU: two gloo ranks launched the way a multi-GPU benchmark run
launches bench.py (torchrun, 127.0.0.1). The path shards by replica, so there is no data-path collective; what is
tested is the launch, the max-over-ranks timing reduction and that rank 0 alone prints."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _max_worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      PIS_BENCH_GLOO="1")
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo")
    q.put((rank, bench.max_over_ranks(float(rank + 1) * 1.5, world)))
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29617
    ps = [ctx.Process(target=_max_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    for p in ps:
        p.join(120)
    got = sorted(q.get(timeout=5) for _ in range(2))
    assert got == [(0, 3.0), (1, 3.0)]


def test_reference_arm_two_ranks_prints_once(oracle_lib):
    env = dict(os.environ, PIS_BENCH_GLOO="1")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29618", os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--cells", "6", "--steps", "1", "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300, cwd=ROOT, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0
