"""One rank of the launcher test: joins the gloo group that bench.launch_ranks set up through
the environment, sums per-shot arrays of its round-robin shots, all-reduces them with the
bench's exchange step and prints the result as JSON (rank 0 only)."""

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import torch  # noqa: E402
import torch.distributed as dist  # noqa: E402

from stride_gb300 import shards  # noqa: E402


def per_shot(shot):
    return np.random.default_rng(100 + shot).standard_normal((8, 6)).astype(np.float32)


def main():
    dist.init_process_group('gloo')
    rank, world = dist.get_rank(), dist.get_world_size()
    g = torch.zeros((8, 6))
    for s in shards.shard_shots(list(range(7)), rank, world):
        g += torch.from_numpy(per_shot(s))
    shards.allreduce_sum(g)
    if rank == 0:
        print(json.dumps({'world': world, 'sum': g.numpy().astype(float).tolist()}))
    dist.destroy_process_group()


if __name__ == '__main__':
    main()
