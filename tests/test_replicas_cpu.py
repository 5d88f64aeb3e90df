"""bench.py's multi-GPU path (replicas: one process per GPU, each solving its
own graph, no collective on the data path) as two gloo ranks on the CPU: the
process-group setup, the barrier, the slowest-rank time and the whole-job
value."""
import json
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

from conftest import ROOT  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    os.environ.update(RANK=str(rank), LOCAL_RANK=str(rank), WORLD_SIZE=str(world), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port), CUDA_VISIBLE_DEVICES="")
    sys.path.insert(0, ROOT)
    import bench

    dist, r, w, local = bench.dist_setup(world)
    bench.barrier(dist)
    my_ms = 100.0 + 50.0 * r  # rank 1 is the slower replica
    ms = bench.max_over_ranks(dist, my_ms)
    with open(os.path.join(out_dir, f"rank{r}.json"), "w") as f:
        json.dump({"rank": r, "world": w, "local": local, "ms": ms, "value": bench.job_value(w, ms),
                   "backend": dist.get_backend()}, f)
    dist.destroy_process_group()


def test_two_gloo_replicas(tmp_path):
    world = 2
    mp.spawn(_rank, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r, d in enumerate(res):
        assert d["rank"] == r and d["world"] == world and d["backend"] == "gloo"
        assert d["ms"] == 150.0  # every rank sees the slowest replica's time
        assert abs(d["value"] - world * 1000.0 / 150.0) < 1e-12
