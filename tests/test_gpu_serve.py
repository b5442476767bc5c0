"""The serving loop (msvgb_server) through the C ABI: every query's result in
the mix equals the same query run alone on the single-query path (MSV results
are integers: bit-exact); admission blocks while all slots are busy; the
persistent kernel leaves when idle and is restarted by the next submission."""
import concurrent.futures as cf
import time

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    ctx = api.Context(0)
    profs = [api.sample_profile(M, 300 + i, ctx) for i, M in enumerate([60, 150, 400, 777, 1300, 2047, 90, 500])]
    s = F.SeqSet.concat([F.synth_sequences(6000, seed=61, lmax=5000),
                         F.emit_homologs(profs[2], 20, seed=62), F.emit_homologs(profs[4], 20, seed=63),
                         F.emit_homologs(profs[3], 5, seed=64, repeat=20)])
    db = api.DeviceDB(ctx, s)
    alone = [api.search(ctx, api.DeviceProfile(ctx, p), db) for p in profs]
    yield ctx, profs, db, alone
    ctx.close()


def test_results_in_the_mix_equal_results_alone(env):
    ctx, profs, db, alone = env
    srv = api.Server(ctx, db, max_slots=16)
    tickets = [srv.submit(p) for p in profs]          # all in flight together
    for t, (xj, fl) in zip(tickets, alone):
        gx, gf = srv.wait(t)
        assert np.array_equal(gx, xj) and np.array_equal(gf, fl)
    srv.close()


def test_admission_blocks_until_a_slot_frees(env):
    ctx, profs, db, alone = env
    srv = api.Server(ctx, db, max_slots=2)
    assert srv.slots == 2
    order = [i % len(profs) for i in range(12)]
    with cf.ThreadPoolExecutor(max_workers=12) as ex:
        def one(i):
            t = srv.submit(profs[i])
            return i, srv.wait(t)
        for i, (gx, gf) in ex.map(one, order):
            assert np.array_equal(gx, alone[i][0]) and np.array_equal(gf, alone[i][1])
    srv.close()


def test_idle_kernel_leaves_and_restarts(env):
    ctx, profs, db, alone = env
    srv = api.Server(ctx, db, max_slots=4)
    gx, gf = srv.wait(srv.submit(profs[0]))
    assert np.array_equal(gx, alone[0][0])
    time.sleep(1.5)                                   # longer than the kernel's idle bound
    gx, gf = srv.wait(srv.submit(profs[5]))
    assert np.array_equal(gx, alone[5][0]) and np.array_equal(gf, alone[5][1])
    assert srv.launches >= 2
    srv.close()


def test_memory_budget_bounds_slots(env):
    ctx, profs, db, alone = env
    srv = api.Server(ctx, db, max_slots=64, mem_budget=1)
    assert srv.slots == 1
    gx, gf = srv.wait(srv.submit(profs[1]))
    assert np.array_equal(gf, alone[1][1])
    srv.close()


def test_requests_that_fill_the_gpu_run_as_own_searches():
    """A database large enough that the larger models' requests (M x residues
    >= 40e9 cells) run as their own single-query searches while the smaller
    ones go through the serving kernel, all in flight together: every result
    equals the plain path's, whichever way it ran."""
    ctx = api.Context(0)
    Ms = [60, 300, 1100, 1500, 2047, 900]
    profs = [api.sample_profile(M, 700 + i, ctx) for i, M in enumerate(Ms)]
    s = F.SeqSet.concat([F.synth_sequences(80_000, seed=71, lmax=12000)] +
                        [F.emit_homologs(p, 50, seed=72 + i) for i, p in enumerate(profs)])
    n_solo = sum(M * s.total >= 4e10 for M in Ms)
    assert 0 < n_solo < len(Ms)                       # both kinds of request
    db = api.DeviceDB(ctx, s)
    alone = [api.search(ctx, api.DeviceProfile(ctx, p), db) for p in profs]
    srv = api.Server(ctx, db, max_slots=16)          # every request admitted at once
    order = list(range(len(Ms))) + list(range(len(Ms)))[::-1]
    tickets = [srv.submit(profs[i]) for i in order]
    for t, i in zip(tickets, order):
        gx, gf = srv.wait(t)
        assert np.array_equal(gx, alone[i][0]), f"M={Ms[i]} xj"
        assert np.array_equal(gf, alone[i][1]), f"M={Ms[i]} flags"
    assert srv.solo_searches == 2 * n_solo
    assert srv.launches >= 1
    srv.close()
    ctx.close()
