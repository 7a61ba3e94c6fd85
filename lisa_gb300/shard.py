"""Splitting one frame over several GPUs, and merging the pieces.

The estimator's samples are independent, so a frame shards without any
exchange during rendering: rank k renders a contiguous range of sample
indices (``sample_range``; the renderer's per-sample RNG streams are keyed
by the sample index, ``Renderer.set_sample_offset``), and the per-rank pixel
means and variances merge exactly at the end (``merge``), on the host, by a
single gather (``gather_merge``, torch.distributed, any backend).  Scenes of
a batch shard the same way, by scene instead of by sample.
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import numpy as np


def sample_range(rank: int, world: int, spp: int) -> Tuple[int, int]:
    """(first sample, count) of rank `rank` when `spp` samples per pixel are
    split over `world` ranks as evenly as possible."""
    if world <= 0 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    base, extra = divmod(spp, world)
    first = rank * base + min(rank, extra)
    return first, base + (1 if rank < extra else 0)


def scene_partition(num_scenes: int, world: int) -> List[List[int]]:
    """Round-robin assignment of the scenes of a batch to ranks."""
    return [list(range(k, num_scenes, world)) for k in range(world)]


def merge(means: Sequence[np.ndarray], variances: Sequence[np.ndarray], counts: Sequence[int]):
    """Exact merge of per-shard pixel means and unbiased sample variances
    (Chan et al.'s pairwise update, summed over shards).  Returns the mean,
    the variance and the total count."""
    counts = [int(c) for c in counts if c > 0]
    means = [np.asarray(m, np.float64) for m, c in zip(means, counts)]
    variances = [np.asarray(v, np.float64) for v, c in zip(variances, counts)]
    n = float(sum(counts))
    mean = sum(m * c for m, c in zip(means, counts)) / n
    # total sum of squared deviations
    m2 = sum(v * (c - 1) + c * (m - mean) ** 2 for m, v, c in zip(means, variances, counts))
    var = m2 / (n - 1) if n > 1 else np.zeros_like(mean)
    return mean, var, int(n)


def gather_merge(mean: np.ndarray, var: np.ndarray, count: int, group=None, dst: int = 0):
    """Gathers every rank's (mean, variance, count) to rank `dst` and merges
    them there.  Returns the merged (mean, variance, count) on `dst`, None
    elsewhere.  Uses torch.distributed (gloo on CPU, NCCL on GPUs)."""
    import torch
    import torch.distributed as dist

    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    payload = torch.from_numpy(np.concatenate([np.asarray(mean, np.float64).ravel(),
                                               np.asarray(var, np.float64).ravel(),
                                               np.array([float(count)])]))
    if dist.get_backend(group) == "nccl":
        payload = payload.cuda()
    parts = [torch.empty_like(payload) for _ in range(world)] if rank == dst else None
    dist.gather(payload, parts, dst=dst, group=group)
    if rank != dst:
        return None
    k = np.asarray(mean).size
    ms, vs, cs = [], [], []
    for p in parts:
        a = p.cpu().numpy()
        ms.append(a[:k].reshape(np.shape(mean)))
        vs.append(a[k:2 * k].reshape(np.shape(mean)))
        cs.append(int(a[-1]))
    return merge(ms, vs, cs)
