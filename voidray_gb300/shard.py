"""Sharding a progressive render over ranks (one process per GPU).

The path shards by samples: every rank holds a replica of the scene and
renders a disjoint, contiguous range of the frame's sample indices (each
sample index selects its own PCG32 streams, so the union of the ranges is
exactly the single-GPU render's sample set).  There is no collective on the
data path; combining the per-rank sums into one image is one sum
(all_reduce) after rendering.
"""
from __future__ import annotations


def sample_range(total: int, rank: int, world: int) -> tuple[int, int]:
    """(first_sample, count) of `rank`'s share of `total` samples: contiguous,
    disjoint, covering [0, total), sizes differing by at most one."""
    if world <= 0 or not 0 <= rank < world or total < 0:
        raise ValueError("bad shard arguments")
    q, r = divmod(total, world)
    first = rank * q + min(rank, r)
    return first, q + (1 if rank < r else 0)


def render_shard(acc, settings, total_samples: int, rgba_device, width: int, height: int, rank: int, world: int,
                 seed: int = 0, stream: int = 0) -> tuple[int, int]:
    """Renders this rank's sample range into rgba_device (raw per-pixel sums
    scaled by 1/settings.total_samples, as iterative_render accumulates)."""
    from .scene import render_device

    first, count = sample_range(total_samples, rank, world)
    if count:
        render_device(acc, settings, count, rgba_device, width, height, seed=seed, first_sample=first, stream=stream)
    return first, count


def reduce_image(buf, group=None) -> None:
    """Sums the per-rank accumulators in place on every rank (torch tensor;
    nccl for device tensors, gloo for host tensors)."""
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(buf, op=dist.ReduceOp.SUM, group=group)
