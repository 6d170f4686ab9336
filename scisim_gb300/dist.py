"""Host side of multi-GPU runs: one process per GPU, no collective on the data path.

A single scene does not shard (every Gauss-Seidel sweep couples all of its contacts), so ranks step
independent work: replicas of a scene, or disjoint slices of a batch of independent scenes.  This
module assigns scenes to ranks by estimated work (longest processing time first), cuts a rank's
sub-batch out of a batch, and reduces timings and counts over ranks (a barrier and a max for time,
a sum for work) through torch.distributed (gloo on the host, NCCL between GPUs).
"""
from __future__ import annotations

import numpy as np


def shard_scenes(work, world_size: int):
    """Scene indices per rank: scenes in decreasing work (ties by index) each go to the rank with the
    least work so far (ties to the lowest rank).  Every scene lands on exactly one rank; each
    rank's list is ascending.  Deterministic, so every rank computes the same assignment."""
    work = np.asarray(work, dtype=np.float64)
    if world_size < 1:
        raise ValueError("world_size must be positive")
    order = sorted(range(work.shape[0]), key=lambda i: (-work[i], i))
    load = [0.0] * world_size
    out = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        out[r].append(i)
        load[r] += float(work[i])
    return [np.array(sorted(x), dtype=np.int64) for x in out]


def batch_work(b) -> np.ndarray:
    """Estimated work per scene of a batch dict: its body count (contacts grow with bodies)."""
    off = np.asarray(b["body_off"])
    return (off[1:] - off[:-1]).astype(np.float64)


def batch_slice(b, scenes):
    """The sub-batch of the given scenes of a Ball2D batch dict (scenes.ball2d_batch layout), with
    its own offsets; other keys are copied."""
    scenes = np.asarray(scenes, dtype=np.int64)
    bo, po = np.asarray(b["body_off"]), np.asarray(b["plane_off"])
    q = np.asarray(b["q"]).reshape(-1, 2)
    v = np.asarray(b["v"]).reshape(-1, 2)
    px, pn = np.asarray(b["plane_x"]).reshape(-1, 2), np.asarray(b["plane_n"]).reshape(-1, 2)
    bodies = np.concatenate([np.arange(bo[s], bo[s + 1]) for s in scenes]) if len(scenes) else np.zeros(0, np.int64)
    planes = np.concatenate([np.arange(po[s], po[s + 1]) for s in scenes]) if len(scenes) else np.zeros(0, np.int64)
    out = dict(b)
    out.update(body_off=np.concatenate([[0], np.cumsum(bo[scenes + 1] - bo[scenes])]).astype(np.int32),
               plane_off=np.concatenate([[0], np.cumsum(po[scenes + 1] - po[scenes])]).astype(np.int32),
               q=q[bodies].reshape(-1), v=v[bodies].reshape(-1), r=np.asarray(b["r"])[bodies],
               m=np.asarray(b["m"])[bodies], plane_x=px[planes], plane_n=pn[planes],
               mu=np.asarray(b["mu"])[scenes], CoR=np.asarray(b["CoR"])[scenes])
    return out


def _reduce(x, op, device):
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()):
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(x, device=None) -> float:
    """The largest value over ranks (the job's time is its slowest rank's)."""
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.MAX, device)


def sum_over_ranks(x, device=None) -> float:
    """The sum over ranks (work done by the whole job)."""
    import torch.distributed as dist
    return _reduce(x, dist.ReduceOp.SUM, device)
