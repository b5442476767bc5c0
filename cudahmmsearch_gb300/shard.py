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


def shard_view(seqs: F.SeqSet, rank: int, world: int):
    """This rank's shard without a copy, in the argument layout of
    msvgb_search_host / msvgb_db_create: the whole residue buffer, the
    rank's slice of the offsets (n+1 absolute offsets into that buffer) and
    its sequence count. Returns (codes, off, n, begin, end)."""
    b = shard_bounds(seqs.lengths, world)
    lo, hi = int(b[rank]), int(b[rank + 1])
    return seqs.codes, seqs.off[lo:hi + 1], hi - lo, lo, hi


def gather_results(local_xj: np.ndarray, local_flags: np.ndarray, n_total: int | None = None, group=None,
                   device=None):
    """Concatenates every rank's per-sequence bytes (xj, flags) in rank (=
    sequence) order on every rank: one all_gather of the shard sizes, then
    one all_gather of fixed-size uint8 tensors (each rank's bytes padded to
    the largest shard). device: where the tensors live -- a CUDA device for
    NCCL, the CPU (default) for gloo. Returns the full (xj, flags) arrays."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    dev = torch.device("cpu") if device is None else torch.device(device)
    n = int(len(local_xj))
    sizes_t = [torch.zeros(1, dtype=torch.int64, device=dev) for _ in range(world)]
    dist.all_gather(sizes_t, torch.tensor([n], dtype=torch.int64, device=dev), group=group)
    sizes = [int(t.item()) for t in sizes_t]
    cap = max(max(sizes), 1)
    local = torch.zeros(2 * cap, dtype=torch.uint8)
    local[:n] = torch.from_numpy(np.ascontiguousarray(local_xj, dtype=np.uint8))
    local[cap:cap + n] = torch.from_numpy(np.ascontiguousarray(local_flags, dtype=np.uint8))
    local = local.to(dev)
    parts = [torch.empty(2 * cap, dtype=torch.uint8, device=dev) for _ in range(world)]
    dist.all_gather(parts, local, group=group)
    parts = [t.cpu().numpy() for t in parts]
    xj = np.concatenate([pt[:sz] for pt, sz in zip(parts, sizes)])
    fl = np.concatenate([pt[cap:cap + sz] for pt, sz in zip(parts, sizes)])
    if n_total is not None and len(xj) != n_total:
        raise ValueError(f"gathered {len(xj)} sequences, expected {n_total}")
    return xj, fl
