"""The hmmsearch-style driver (msvgb_pipeline_run): blocks scored on the GPU,
F1 survivors handed to CPU worker threads with their exact MSV score. The
survivor set, the scores and n_past_msv equal the reference pipeline's MSV
stage (oracle), for several block sizes and worker counts."""
import os
import threading

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


@pytest.mark.parametrize("block,workers", [(1000, 1), (777, 4), (100_000, 3)])
def test_pipeline_survivors_match_reference_msv_stage(ctx, block, workers):
    p = F.read_profile(os.path.join(GOLDEN, "m200_s1.prof"))
    s = F.SeqSet.concat([F.synth_sequences(4000, seed=71, lmax=3000), F.emit_homologs(p, 60, seed=72),
                         F.SeqSet.from_list([np.zeros(0, np.uint8)]), F.emit_homologs(p, 4, seed=73, repeat=20)])
    o = O.msv_batch(p, s)
    got = {}
    lock = threading.Lock()

    def on_survivor(i, usc, xj, fl):
        with lock:
            got[i] = usc
        return False

    n_past = api.pipeline_run(ctx, p, s, on_survivor, block_size=block, n_workers=workers)
    want = np.nonzero(o["pass"] == 1)[0]
    assert n_past == len(want) == len(got)
    assert sorted(got) == list(want)
    for i in want:
        assert np.float32(got[i]).view(np.uint32) == np.float32(o["sc"][i]).view(np.uint32)


def test_pipeline_continuation_can_stop_the_run(ctx):
    p = F.read_profile(os.path.join(GOLDEN, "m200_s1.prof"))
    s = F.SeqSet.concat([F.emit_homologs(p, 50, seed=74), F.synth_sequences(2000, seed=75)])
    with pytest.raises(api.MSVError) as e:
        api.pipeline_run(ctx, p, s, lambda i, usc, xj, fl: True, block_size=100, n_workers=2)
    assert e.value.code == 1


@pytest.mark.parametrize("name", ["tut_globins4", "tut_fn3", "tut_pkinase"])
def test_pipeline_on_tutorial_models_equals_reference_msv_stage(ctx, name):
    """The driver on a real Pfam model (the reference's tutorial library) and
    its golden targets: n_past_msv and every survivor's score equal the
    reference's own MSV stage (the golden fixtures came from its
    p7_MSVFilter and F1 gate)."""
    p = F.read_profile(os.path.join(GOLDEN, name + ".prof"))
    s = F.read_seqs(os.path.join(GOLDEN, name + ".seqs"))
    r = F.read_results(os.path.join(GOLDEN, name + ".res"))
    got = {}
    lock = threading.Lock()

    def on_survivor(i, usc, xj, fl):
        with lock:
            got[i] = usc
        return False

    n_past = api.pipeline_run(ctx, p, s, on_survivor, block_size=50, n_workers=3)
    want = np.nonzero(r.passed == 1)[0]
    assert n_past == len(want) == len(got) and sorted(got) == list(want)
    for i in want:
        assert np.float32(got[i]).view(np.uint32) == r.sc[i].view(np.uint32)


def test_dropin_from_many_threads(ctx):
    """p7_MSVFilter is called from hmmsearch's worker threads: concurrent
    drop-in calls on one context (serialised inside) and on per-thread
    contexts give the reference's results."""
    p = F.read_profile(os.path.join(GOLDEN, "tut_pkinase.prof"))
    s = F.read_seqs(os.path.join(GOLDEN, "tut_pkinase.seqs"))
    r = F.read_results(os.path.join(GOLDEN, "tut_pkinase.res"))
    errors = []

    def work(c, idx):
        try:
            for i in idx:
                L = int(s.lengths[i])
                dsq = np.concatenate([[255], s.seq(i), [255]]).astype(np.uint8)
                st, sc = c.MSVFilter(dsq, L, p, api.tjb_b(p.scale_b, L))
                if st != r.status[i] or np.float32(sc).view(np.uint32) != r.sc[i].view(np.uint32):
                    errors.append(i)
        except Exception as e:                      # surfaced below
            errors.append(repr(e))

    own = [api.Context(0) for _ in range(2)]
    try:
        threads = [threading.Thread(target=work, args=(ctx if t < 3 else own[t - 3], range(t, s.n, 5)))
                   for t in range(5)]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
    finally:
        for c in own:
            c.close()
    assert not errors
