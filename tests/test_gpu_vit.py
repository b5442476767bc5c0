"""The ViterbiFilter stage on the GPU (msvgb_vitfilter) against
p7_ViterbiFilter's own golden results and the oracle: statuses and score bit
patterns, for sampled models in hmmsearch's local mode (M = 1 .. 4000: the
register row up to 1536 nodes, the shared-memory row above) and the tutorial
Pfam models, over all sequences and over survivor lists."""
import glob
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O
from tests.vprofiles import crop_vprofile

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
VIT = sorted(os.path.basename(p)[4:-6] for p in glob.glob(os.path.join(GOLDEN, "vit_*.vprof")))
MAX_M = 8192


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0)
    yield c
    c.close()


def expected(st_ref):
    """Golden statuses (eslOK 0, eslERANGE 16, -1 empty) as msvgb_vitfilter reports them."""
    return np.where(st_ref == 16, 1, np.where(st_ref < 0, 2, 0)).astype(np.uint8)


@pytest.mark.parametrize("name", VIT)
def test_vitfilter_matches_reference_golden(ctx, name):
    vp = F.read_vprofile(os.path.join(GOLDEN, "vit_" + name + ".vprof"))
    s = F.read_seqs(os.path.join(GOLDEN, name + ".seqs"))
    st_ref, sc_ref = F.read_vresults(os.path.join(GOLDEN, "vit_" + name + ".vres"))
    assert vp.M <= MAX_M
    dvp = api.DeviceVProfile(ctx, vp)
    db = api.DeviceDB(ctx, s)
    st, sc = api.vitfilter(ctx, dvp, db)
    assert np.array_equal(st, expected(st_ref))
    ok = st_ref == 0
    assert np.array_equal(sc[ok].view(np.uint32), sc_ref[ok].view(np.uint32))
    # a survivor-style list: every other sequence, in reverse order
    ids = np.arange(s.n - 1, -1, -2)
    st2, sc2 = api.vitfilter(ctx, dvp, db, ids)
    assert np.array_equal(st2, st[ids]) and np.array_equal(sc2.view(np.uint32), sc[ids].view(np.uint32))


@pytest.mark.parametrize("name", ["m200_s1", "m400_s1", "tut_pkinase", "m777_s3", "m2400_s1"])
def test_vitfilter_matches_oracle_on_homologs_and_long_targets(ctx, name):
    vp = F.read_vprofile(os.path.join(GOLDEN, "vit_" + name + ".vprof"))
    p = F.read_profile(os.path.join(GOLDEN, name + ".prof"))
    s = F.SeqSet.concat([F.synth_sequences(400, seed=vp.M, lmax=6000), F.emit_homologs(p, 60, seed=vp.M + 1),
                         F.emit_homologs(p, 10, seed=vp.M + 2, repeat=5)])
    o = O.vit_batch(vp, s)
    st, sc = api.vitfilter(ctx, api.DeviceVProfile(ctx, vp), api.DeviceDB(ctx, s))
    assert np.array_equal(st, expected(o["status"]))
    ok = o["status"] == 0
    assert np.array_equal(sc[ok].view(np.uint32), o["sc"][ok].view(np.uint32))
    assert (st == 0).sum() >= 300
    if name == "tut_pkinase":                # Pfam homologs saturate the 16-bit range
        assert (st[400:] == 1).sum() >= 50


# every register-row width of the kernel (nodes per lane), and the shared-memory row above them
ROW_WIDTHS = [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 20, 24, 28, 32, 40, 48, 56]


@pytest.mark.parametrize("cv", ROW_WIDTHS)
def test_vitfilter_every_row_width_matches_oracle(ctx, cv):
    full = F.read_vprofile(os.path.join(GOLDEN, "vit_m2400_s1.vprof"))
    M = 32 * cv - 3 if cv > 1 else 27          # the widest model of this width, less a few nodes
    vp = crop_vprofile(full, M)
    p = F.read_profile(os.path.join(GOLDEN, "m2400_s1.prof"))
    s = F.SeqSet.concat([F.synth_sequences(150, seed=cv, lmax=2500), F.emit_homologs(p, 40, seed=cv + 1)])
    o = O.vit_batch(vp, s)
    st, sc = api.vitfilter(ctx, api.DeviceVProfile(ctx, vp), api.DeviceDB(ctx, s))
    assert np.array_equal(st, expected(o["status"]))
    ok = o["status"] == 0
    assert np.array_equal(sc[ok].view(np.uint32), o["sc"][ok].view(np.uint32))


def test_vitfilter_rejects_bad_indices(ctx):
    vp = F.read_vprofile(os.path.join(GOLDEN, "vit_m50_s1.vprof"))
    db = api.DeviceDB(ctx, F.synth_sequences(10, seed=2))
    with pytest.raises(api.MSVError) as e:
        api.vitfilter(ctx, api.DeviceVProfile(ctx, vp), db, np.array([3, 10]))
    assert e.value.code == api.eslEINVAL


def test_vitfilter_model_size_limit(ctx):
    vp = F.read_vprofile(os.path.join(GOLDEN, "vit_m50_s1.vprof"))
    for M, ok in ((8192, True), (8193, False)):
        Q8 = max(2, (M - 1) // 8 + 1)
        big = F.VProfile(M, np.full((8 * Q8, 8), -300, np.int16), np.zeros((29, Q8, 8), np.int16), vp.xw,
                         vp.scale_w, vp.nj, vp.base_w, vp.ddbound_w)
        if ok:
            api.DeviceVProfile(ctx, big).close()
        else:
            with pytest.raises(api.MSVError) as e:
                api.DeviceVProfile(ctx, big)
            assert e.value.code == api.eslEINVAL


def test_vitfilter_shared_profile_from_threads():
    """One ViterbiFilter profile used at once from threads on their own
    contexts, over databases whose longest sequences differ (the per-length
    move table grows while other calls run): every result equals the
    sequential one."""
    import threading
    vp = F.read_vprofile(os.path.join(GOLDEN, "vit_m200_s1.vprof"))
    sets = [F.synth_sequences(3000, seed=60 + t, lmax=500 * (t + 1) ** 2) for t in range(4)]
    ctxs = [api.Context(0) for _ in sets]
    dvp = api.DeviceVProfile(ctxs[0], vp)
    dbs = [api.DeviceDB(c, s) for c, s in zip(ctxs, sets)]
    got = [None] * len(sets)

    def run(t):
        got[t] = api.vitfilter(ctxs[t], dvp, dbs[t])
    threads = [threading.Thread(target=run, args=(t,)) for t in range(len(sets))]
    for th in threads:
        th.start()
    for th in threads:
        th.join()
    for t, s in enumerate(sets):
        st, sc = api.vitfilter(ctxs[t], dvp, dbs[t])
        assert np.array_equal(got[t][0], st) and np.array_equal(got[t][1].view(np.uint32), sc.view(np.uint32))
    o = O.vit_batch(vp, sets[3].subset(np.arange(0, 3000, 50)))
    st, sc = got[3]
    sub = np.arange(0, 3000, 50)
    assert np.array_equal(sc[sub].view(np.uint32), o["sc"].view(np.uint32))
    for d in dbs:
        d.close()
    dvp.close()
    for c in ctxs:
        c.close()
