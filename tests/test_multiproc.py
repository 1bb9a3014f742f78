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


def test_bench_launcher_starts_the_ranks():
    """bench.launch_ranks (what `bench.py --gpus N` does when started without torchrun) runs N
    ranks; their all-reduced per-shot sums equal the single-process sum over all shots."""
    import json
    import bench
    from tests import _rank_sum
    script = os.path.join(os.path.dirname(os.path.abspath(__file__)), '_rank_sum.py')
    rc, out = bench.launch_ranks(2, [script], capture=True)
    assert rc == 0
    lines = [l for l in out.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    got = json.loads(lines[0])
    assert got['world'] == 2
    full = sum(_rank_sum.per_shot(s) for s in range(7))
    np.testing.assert_allclose(np.array(got['sum']), full, rtol=1e-5, atol=1e-5)


def test_bench_reference_arm_under_two_ranks():
    """`bench.py --impl reference --gpus 2` relaunches itself as two ranks; rank 0 alone prints the
    reference arm's line, with n_gpus 2."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, os.path.join(root, 'bench.py'), '--impl', 'reference', '--gpus', '2',
                        '--workload', 'single', '--nt', '40', '--steps', '1', '--warmup', '0'],
                       stdout=subprocess.PIPE, text=True, timeout=600)
    assert r.returncode == 0
    lines = [l for l in r.stdout.splitlines() if l.startswith('{')]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line['impl'] == 'reference' and line['n_gpus'] == 2 and line['steps'] == 1
