"""The N>1 host path on CPU: two gloo ranks shard the shots round-robin and all-reduce the
per-rank gradient sums; the result equals the single-process sum over all shots."""

import os

import numpy as np
import pytest

torch = pytest.importorskip('torch')
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

from stride_gb300 import shards  # noqa: E402


def _per_shot_grad(shot):
    rng = np.random.default_rng(100 + shot)
    return rng.standard_normal((16, 12)).astype(np.float32)


def _worker(rank, world, port, out):
    os.environ['MASTER_ADDR'] = '127.0.0.1'
    os.environ['MASTER_PORT'] = str(port)
    dist.init_process_group('gloo', rank=rank, world_size=world)
    mine = shards.shard_shots(list(range(7)), rank, world)
    g = torch.zeros((16, 12))
    for s in mine:
        g += torch.from_numpy(_per_shot_grad(s))
    shards.allreduce_sum(g)
    out[rank] = g.numpy().copy()
    dist.destroy_process_group()


def test_two_rank_gradient_sum():
    port = 29500 + (os.getpid() % 1000)
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    full = sum(_per_shot_grad(s) for s in range(7))
    for r in range(2):
        np.testing.assert_allclose(out[r], full, rtol=1e-5, atol=1e-5)


def test_shard_assignment_covers_all_shots_once():
    ids = list(range(10))
    parts = [shards.shard_shots(ids, r, 3) for r in range(3)]
    assert sorted(sum(parts, [])) == ids
    assert parts[0] == [0, 3, 6, 9]
