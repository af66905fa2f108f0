"""Replicas on several GPUs (one process per GPU): the reference's multi-lane
design (``WavefrontPathTracing``, common/wavefront_path_tracing.hpp:1272, :1345-1408),
where each lane renders the same image with its own random streams and the
lanes' accumulations are merged at readback (``merge_from``, a tree of
pairwise merges).

Sharding: rank k of N renders spp_k = spp / N samples per pixel (the first
spp % N ranks one more) with its RNG seeded at seed_offset + k * path_count,
as ``WavefrontLane::initialize`` seeds lane k (:544-548); the merge is a
sum of the FP64 per-pixel sums and counts (an all-reduce over the process
group), so the merged image has exactly spp samples per pixel.
"""
from __future__ import annotations

import ctypes as C


def shard_config(cfg, rank: int, world: int, path_count: int):
    """This rank's copy of the render config (an ``rgr_render_config``)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank / world size")
    out = type(cfg)()
    C.memmove(C.byref(out), C.byref(cfg), C.sizeof(cfg))
    out.seed_offset = int(cfg.seed_offset) + rank * int(path_count)
    if cfg.spp:
        base, extra = divmod(int(cfg.spp), world)
        out.spp = base + (1 if rank < extra else 0)
    return out


def merge_sums(acc, group=None):
    """Sum the (H, W, 4) FP64 accumulations of all ranks in place (every rank
    gets the merged array); ``acc`` is a numpy array or a torch tensor."""
    import numpy as np
    import torch
    import torch.distributed as dist

    t = acc if isinstance(acc, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(acc))
    dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    if not isinstance(acc, torch.Tensor):
        acc[...] = t.numpy()
    return acc
