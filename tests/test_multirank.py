"""The N-rank bench path on CPU: two gloo ranks on 127.0.0.1 run the same
host logic as `bench.py --gpus 2` under torchrun -- barrier, max-over-ranks
timing, whole-job rate -- and, as replicas, produce identical answers for the
same seeded batch (the oracle stands in for the device here)."""
import json
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, outdir):
    import sys
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    from conftest import load_golden
    from oracle import oracle as O
    bench.rank_barrier(world)
    local_ms = 10.0 + 5.0 * rank  # rank 1 is the slow one
    ms = bench.max_over_ranks(local_ms, world)
    rate = bench.job_rate(1_000_000, world, ms)
    # replicas: every rank answers the same seeded batch
    g = load_golden("sphere_small")
    prim, t, _, _ = O.BVH(g["tris"]).nearest(g["rays"])
    digest = float(np.sum(prim.astype(np.float64) * 1.0001 + np.nan_to_num(t)))
    gathered = [None] * world
    dist.all_gather_object(gathered, digest)
    with open(os.path.join(outdir, f"rank{rank}.json"), "w") as f:
        json.dump({"ms": ms, "rate": rate, "digests": gathered}, f)
    dist.destroy_process_group()


def test_two_gloo_ranks(tmp_path):
    from oracle import oracle as O
    O.build()
    world = 2
    mp.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r in res:
        assert r["ms"] == 15.0  # the slowest rank's time on every rank
        assert r["rate"] == pytest.approx(2 * 1_000_000 / 15e-3 / 1e6)
        assert r["digests"][0] == r["digests"][1]
