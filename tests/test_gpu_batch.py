"""Many profiles in one persistent launch (msvgb_search_batch / msvgb_batch)
through the C ABI: every (profile, sequence) result equals the single-query
path's and the oracle's; the captured graph replays identically; calibration
on the GPU reproduces the reference's mu."""
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("name", ["m50_s1", "m200_s1", "m400_s1", "m777_s3", "m1500_s2"])
def test_calibration_reproduces_reference_mu(ctx, name):
    ref = F.read_profile(os.path.join(GOLDEN, name + ".prof"))
    got = api.sample_profile(ref.M, int(name.split("_s")[1]), ctx)
    assert np.float32(got.mmu) == np.float32(ref.mmu)
    assert np.float32(got.mlambda) == np.float32(ref.mlambda)


def make_profiles(ctx, Ms, seed0=100):
    return [api.sample_profile(M, seed0 + i, ctx) for i, M in enumerate(Ms)]


def test_batch_equals_single_query_and_oracle(ctx):
    Ms = [1, 17, 50, 64, 120, 200, 333, 400, 650, 777, 1000, 1500, 2000, 2047, 2048, 3000]
    profs = make_profiles(ctx, Ms)
    s = F.SeqSet.concat([F.synth_sequences(2500, seed=41, lmax=8000),
                         F.emit_homologs(profs[5], 30, seed=42), F.emit_homologs(profs[9], 30, seed=43),
                         F.emit_homologs(profs[7], 10, seed=44, repeat=20),
                         F.SeqSet.from_list([np.zeros(0, np.uint8), np.array([3], np.uint8)])])
    db = api.DeviceDB(ctx, s)
    bxj, bfl = api.search_batch(ctx, profs, db)
    sub = np.arange(0, s.n, 7)
    for i, p in enumerate(profs):
        xj, fl = api.search(ctx, api.DeviceProfile(ctx, p), db)
        assert np.array_equal(bxj[i], xj), f"profile {i} (M={p.M}) xj"
        assert np.array_equal(bfl[i], fl), f"profile {i} (M={p.M}) flags"
        o = O.msv_batch(p, s.subset(sub))
        ok = o["status"] == F.eslOK
        assert np.array_equal(bxj[i][sub][ok], o["xj"][ok])
        assert np.array_equal((bfl[i][sub] & api.FLAG_ERANGE) != 0, o["status"] == F.eslERANGE)


def test_batch_graph_replays_identically(ctx):
    import torch
    profs = make_profiles(ctx, [90, 300, 1200], seed0=7)
    s = F.synth_sequences(4000, seed=51, lmax=3000)
    db = api.DeviceDB(ctx, s)
    n = s.n
    out = torch.zeros(2 * len(profs) * n, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()
    b = api.Batch(ctx, profs, db, out.data_ptr(), out.data_ptr() + len(profs) * n)
    assert b.items >= 3
    b.run()
    torch.cuda.synchronize()
    first = out.cpu().numpy().copy()
    out.zero_()
    torch.cuda.synchronize()
    b.run()
    torch.cuda.synchronize()
    assert np.array_equal(out.cpu().numpy(), first)
    want = api.search_batch(ctx, profs, db)
    assert np.array_equal(first[:len(profs) * n].reshape(len(profs), n), want[0])
    b.close()


def test_batch_rejects_oversize_profiles(ctx):
    big = F.profile_from_node_costs(np.zeros((29, 8192), np.uint8), tbm_b=10, tec_b=3, base_b=190,
                                    bias_b=10, scale_b=4.328085, mmu=-9.0, mlambda=0.69)
    db = api.DeviceDB(ctx, F.synth_sequences(10, seed=1))
    with pytest.raises(api.MSVError) as e:
        api.search_batch(ctx, [big], db)
    assert e.value.code == api.eslEINVAL


def test_batch_with_own_searches_equals_single_query_and_oracle(ctx):
    """A database large enough that some profiles (M x residues >= 40e9
    cells) are scored by their own single-query searches on the batch graph's
    branches, beside the persistent kernel for the others: identical to the
    single-query path, and the oracle on a sample."""
    Ms = [120, 300, 700, 1100, 1500, 2500]
    profs = make_profiles(ctx, Ms, seed0=300)
    s = F.SeqSet.concat([F.synth_sequences(118_000, seed=51, lmax=12000)] +
                        [F.emit_homologs(p, 300, seed=52 + i) for i, p in enumerate(profs)])
    assert Ms[-2] * s.total >= 4e10 > Ms[1] * s.total     # both kinds of profile in the batch
    db = api.DeviceDB(ctx, s)
    bxj, bfl = api.search_batch(ctx, profs, db)
    rng = np.random.default_rng(53)
    sub = np.sort(rng.choice(s.n, size=1500, replace=False))
    for i, p in enumerate(profs):
        xj, fl = api.search(ctx, api.DeviceProfile(ctx, p), db)
        assert np.array_equal(bxj[i], xj), f"profile {i} (M={p.M}) xj"
        assert np.array_equal(bfl[i], fl), f"profile {i} (M={p.M}) flags"
        o = O.msv_batch(p, s.subset(sub))
        ok = o["status"] == F.eslOK
        assert np.array_equal(bxj[i][sub][ok], o["xj"][ok])
        assert np.array_equal((bfl[i][sub] & api.FLAG_ERANGE) != 0, o["status"] == F.eslERANGE)
        assert np.array_equal((bfl[i][sub] & api.FLAG_PASS) != 0, o["pass"] == 1)
