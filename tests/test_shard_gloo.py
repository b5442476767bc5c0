"""Multi-GPU sharding logic on CPU: gloo ranks each score their
residue-balanced shard (with the oracle standing in for a GPU) and gather the
per-sequence bytes with fixed-size tensor all_gathers; the result equals
scoring the whole database at once. One case cuts the shard as a copy, the
other as a view in msvgb_search_host's argument layout (the whole residue
buffer, the rank's slice of absolute offsets, its count)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from cudahmmsearch_gb300 import formats as F
from cudahmmsearch_gb300 import shard as S

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q, view=False):
    import torch.distributed as dist
    from oracle import oracle as O
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    p = F.read_profile(os.path.join(GOLDEN, "m200_s1.prof"))
    s = F.synth_sequences(800, seed=3, lmax=3000)
    if view:
        codes, off, n, lo, hi = S.shard_view(s, rank, world)
        assert off.size == n + 1 and codes is s.codes
        local = F.SeqSet(codes, off)        # absolute offsets into the shared buffer
    else:
        local, lo, hi = S.shard(s, rank, world)
    o = O.msv_batch(p, local, nthreads=1)
    flags = (o["status"] == 16).astype(np.uint8) | (o["pass"] << 1)
    xj, fl = S.gather_results(o["xj"], flags, s.n)
    if rank == 0:
        full = O.msv_batch(p, s, nthreads=2)
        want = (full["status"] == 16).astype(np.uint8) | (full["pass"] << 1)
        q.put((bool(np.array_equal(xj, full["xj"])), bool(np.array_equal(fl, want)), hi - lo))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,view", [(2, False), (2, True), (3, True)])
def test_gloo_ranks_gather_equals_whole(world, view):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q, view)) for r in range(world)]
    for pr in procs:
        pr.start()
    res = q.get(timeout=120)
    for pr in procs:
        pr.join(timeout=120)
        assert pr.exitcode == 0
    assert res[0] and res[1] and res[2] > 0


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shards_cover_and_balance(world):
    s = F.synth_sequences(5000, seed=4, lmax=35000)
    b = S.shard_bounds(s.lengths, world)
    assert b[0] == 0 and b[-1] == s.n and np.all(np.diff(b) >= 0)
    res = [int(s.off[b[r + 1]] - s.off[b[r]]) for r in range(world)]
    assert sum(res) == s.total
    assert max(res) - min(res) <= 2 * int(s.lengths.max()) + 1
    parts = [S.shard(s, r, world)[0] for r in range(world)]
    assert np.array_equal(np.concatenate([p.codes for p in parts]), s.codes)
