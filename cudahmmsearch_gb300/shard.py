"""Multi-GPU sharding of the MSV search (weak scaling, no device collective).

Every (profile, sequence) pair is independent, so a database is split across
ranks into contiguous index ranges balanced by residue count; each rank
searches its shard on its own GPU; the only exchange is a host gather of the
per-sequence result bytes (xj, flags), concatenated back in sequence order.
"""
from __future__ import annotations

import numpy as np

from . import formats as F


def shard_bounds(lengths: np.ndarray, world: int) -> np.ndarray:
    """world+1 sequence indices splitting the database into contiguous ranges
    of nearly equal residue count (each rank gets at least zero sequences)."""
    lengths = np.asarray(lengths, dtype=np.int64)
    n = len(lengths)
    if world < 1:
        raise ValueError("world must be >= 1")
    cum = np.concatenate([[0], np.cumsum(np.maximum(lengths, 1))])
    targets = cum[-1] * np.arange(world + 1) / world
    b = np.searchsorted(cum, targets, side="left")
    b[0], b[-1] = 0, n
    return np.maximum.accumulate(np.clip(b, 0, n))


def shard(seqs: F.SeqSet, rank: int, world: int) -> tuple[F.SeqSet, int, int]:
    """This rank's shard (a SeqSet) and its [begin, end) range in the database."""
    b = shard_bounds(seqs.lengths, world)
    lo, hi = int(b[rank]), int(b[rank + 1])
    off = seqs.off[lo:hi + 1] - seqs.off[lo]
    codes = seqs.codes[seqs.off[lo]:seqs.off[hi]]
    return F.SeqSet(codes, off.astype(np.int64)), lo, hi


def gather_results(local_xj: np.ndarray, local_flags: np.ndarray, n_total: int, group=None):
    """Concatenate every rank's per-sequence bytes in rank (= sequence) order
    with a host-side gather over torch.distributed (any backend); returns the
    full arrays on every rank."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    local = np.concatenate([local_xj, local_flags]).astype(np.uint8)
    sizes = [None] * world
    dist.all_gather_object(sizes, int(len(local_xj)), group=group)
    parts = [None] * world
    dist.all_gather_object(parts, local.tobytes(), group=group)
    xj = np.concatenate([np.frombuffer(p, np.uint8)[:sz] for p, sz in zip(parts, sizes)])
    fl = np.concatenate([np.frombuffer(p, np.uint8)[sz:] for p, sz in zip(parts, sizes)])
    assert len(xj) == n_total
    return xj, fl
