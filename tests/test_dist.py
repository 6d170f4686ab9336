"""Multi-process host logic (scisim_gb300/dist.py) with world_size 2 over gloo on the CPU: every rank
computes the same scene assignment, the shards are disjoint and cover the batch, the work is balanced,
each rank's sub-batch is exactly its scenes, and the reductions give the job's time (max) and work
(sum).  No GPU: the data path of a multi-GPU run has no collective, so this is all of its host side.
"""
import os

import numpy as np
import pytest

from scisim_gb300 import dist, scenes


def test_shard_scenes_single_process():
    work = np.array([5, 1, 9, 3, 3, 7, 2, 8], dtype=float)
    parts = dist.shard_scenes(work, 3)
    assert sorted(np.concatenate(parts).tolist()) == list(range(8))
    loads = [work[p].sum() for p in parts]
    assert max(loads) - min(loads) <= work.max()
    assert [p.tolist() for p in dist.shard_scenes(work, 1)] == [list(range(8))]


def test_batch_slice_is_the_scenes():
    b = scenes.ball2d_batch(n_scenes=5, nmax=40, seed=1)
    sub = dist.batch_slice(b, [1, 3])
    for k, s in enumerate([1, 3]):
        one = scenes.batch_scene(b, s)
        two = scenes.batch_scene(sub, k)
        for key in ("q", "v", "r", "m", "plane_x", "plane_n", "mu", "CoR"):
            assert np.array_equal(np.asarray(one[key]), np.asarray(two[key])), key


def _rank(rank, world, port, out_dir):
    import torch.distributed as td
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    td.init_process_group("gloo", rank=rank, world_size=world)
    b = scenes.ball2d_batch(n_scenes=12, nmax=200, seed=7)
    parts = dist.shard_scenes(dist.batch_work(b), world)
    mine = dist.batch_slice(b, parts[rank])
    local_bodies = int(mine["body_off"][-1])
    total = dist.sum_over_ranks(local_bodies)
    slowest = dist.max_over_ranks(10.0 + rank)
    np.save(os.path.join(out_dir, "rank%d.npy" % rank),
            np.array([local_bodies, total, slowest] + parts[rank].tolist(), dtype=np.float64))
    td.barrier()
    td.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_ranks_gloo(tmp_path):
    import socket

    import torch.multiprocessing as mp
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    mp.spawn(_rank, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r0 = np.load(tmp_path / "rank0.npy")
    r1 = np.load(tmp_path / "rank1.npy")
    b = scenes.ball2d_batch(n_scenes=12, nmax=200, seed=7)
    N = int(b["body_off"][-1])
    assert r0[1] == r1[1] == N == r0[0] + r1[0]
    assert r0[2] == r1[2] == 11.0
    s0, s1 = set(r0[3:].astype(int)), set(r1[3:].astype(int))
    assert not (s0 & s1) and (s0 | s1) == set(range(12))
