"""Multi-GPU helpers for the delta2zreion step (torch.distributed).

Replicas (what bench.py runs): every rank runs whole boxes; the only
collective is the timing reduction (max over ranks) after the timed region.

Radius sharding (for a box whose radii are split across GPUs): rank q runs the
radii shard_radii(n, world, q) of the same delta_lin (broadcast once) and
keeps its partial (zreion, argmax); the partials are merged by one elementwise
max over a packed 64-bit key: the order-preserving bits of the float32 z in
the high word and 255 - r in the low byte, so that the larger z wins and,
for equal z, the smaller radius index wins -- the strict `>` of the serial
loop over ascending radii (delta2zreion_d2z.C:105-146).  Cells never updated
(z = 0, argmax 255) carry the low byte 0 and lose every tie.
"""
from __future__ import annotations

import numpy as np

__all__ = ["max_over_ranks", "shard_radii", "pack_keys", "unpack_keys", "merge_radius_shards"]


def max_over_ranks(value: float, device=None) -> float:
    """max of a scalar over all ranks (identity without an initialised group)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def shard_radii(n_radii: int, world: int, rank: int) -> range:
    """Contiguous block of global radius indices for a rank (sizes differ by at most one)."""
    base, extra = divmod(n_radii, world)
    lo = rank * base + min(rank, extra)
    return range(lo, lo + base + (1 if rank < extra else 0))


def pack_keys(z, argmax):
    """int64 keys of (z float32, global argmax uint8) as described above."""
    import torch
    zb = z.contiguous().to(torch.float32).view(torch.int32).to(torch.int64)
    # negative floats: flip the magnitude bits so that the integer order is the float order
    zb = torch.where(zb < 0, zb ^ 0x7FFFFFFF, zb)
    low = (255 - argmax.to(torch.int64)) & 0xFF
    return (zb << 8) | low


def unpack_keys(key):
    import torch
    zb = key >> 8
    zb = torch.where(zb < 0, zb ^ 0x7FFFFFFF, zb)
    z = zb.to(torch.int32).view(torch.float32)
    am = (255 - (key & 0xFF)).to(torch.uint8)
    return z, am


def merge_radius_shards(z, argmax, group=None):
    """Elementwise (max z, its smallest radius) over all ranks, in place on
    torch tensors (any device the process group supports).  argmax holds
    global radius indices (255 = never updated)."""
    import torch.distributed as dist
    key = pack_keys(z, argmax)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(key, op=dist.ReduceOp.MAX, group=group)
    zm, am = unpack_keys(key)
    z.copy_(zm.view(z.shape))
    argmax.copy_(am.view(argmax.shape))
    return z, argmax


def local_to_global_argmax(argmax_local: np.ndarray, shard: range) -> np.ndarray:
    """Shift shard-local radius indices to global ones (255 stays 255)."""
    a = argmax_local.astype(np.int64)
    return np.where(a == 255, 255, a + shard.start).astype(np.uint8)
