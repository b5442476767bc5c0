"""The filter stages after MSV on the GPU, through the C ABI: the bias filter
(msvgb_biasfilter) bit for bit against p7_bg_FilterScore's golden scores, and
the pipeline driver with GPU bias and Viterbi stages (msvgb_pipeline_filters)
against the stage every sequence reached in the reference's own p7_Pipeline
(tests/golden/pipe_*.pres), its counters, and the oracle."""
import glob
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
PIPE = sorted(os.path.basename(p)[5:-5] for p in glob.glob(os.path.join(GOLDEN, "pipe_*.pres")))


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0)
    yield c
    c.close()


def load(name):
    r = F.read_pipe(os.path.join(GOLDEN, "pipe_" + name + ".pres"))
    s = F.read_seqs(os.path.join(GOLDEN, "pipe_" + name + ".seqs"))
    prof = os.path.join(GOLDEN, "pipe_" + name + ".prof")
    p = F.read_profile(prof if os.path.exists(prof) else os.path.join(GOLDEN, name + ".prof"))
    vp = F.read_vprofile(os.path.join(GOLDEN, "vit_" + name + ".vprof"))
    return r, s, p, vp


def bits(a):
    return np.asarray(a, np.float32).view(np.uint32)


@pytest.mark.parametrize("name", PIPE)
def test_biasfilter_matches_reference(ctx, name):
    r, s, p, vp = load(name)
    db = api.DeviceDB(ctx, s)
    got = api.biasfilter(ctx, r.compo, r.M, db)
    ne = s.lengths > 0
    assert np.array_equal(bits(got[ne]), bits(r.fsc[ne]))
    ids = np.nonzero(ne)[0][::-3]                         # a reversed survivor-style list
    assert np.array_equal(bits(api.biasfilter(ctx, r.compo, r.M, db, ids)), bits(r.fsc[ids]))


@pytest.mark.parametrize("name", PIPE)
@pytest.mark.parametrize("block_size", [64, 100_000])
def test_pipeline_filters_match_reference(ctx, name, block_size):
    r, s, p, vp = load(name)
    hits, st = api.pipeline_filters(ctx, p, s, vprof=vp, compo=r.compo, vmu=r.vmu, vlambda=r.vlambda,
                                    block_size=block_size, F1=r.F1, F2=r.F2, n_workers=3)
    want = np.nonzero(r.stage == 3)[0]
    assert np.array_equal(hits["seq_index"], want)
    assert np.array_equal(bits(hits["usc"]), bits(r.usc[want]))
    assert np.array_equal(bits(hits["nullsc"]), bits(r.nullsc[want]))
    assert np.array_equal(bits(hits["filtersc"]), bits(r.fsc[want]))
    assert np.array_equal(bits(hits["vfsc"]), bits(r.vfsc[want]))          # NaN where Viterbi was skipped
    ne = r.stage != 255
    assert (st.nseqs, st.nres) == (s.n, s.total)
    assert st.n_past_msv == int((r.stage[ne] >= 1).sum())
    assert st.n_past_bias == int((r.stage[ne] >= 2).sum())
    assert st.n_past_vit == int((r.stage[ne] == 3).sum())


def test_pipeline_filters_variants_match_oracle(ctx):
    """--nobias, and stopping after the bias stage, against the oracle on a
    larger synthetic set with homologs and biased sequences."""
    r, s0, p, vp = load("tut_pkinase")
    s = F.SeqSet.concat([s0, F.synth_sequences(3000, seed=77, lmax=4000), F.emit_homologs(p, 40, seed=78)])
    usc = O.msv_batch(p, s)["sc"]
    for do_bias in (True, False):
        o = O.pipe_batch(vp, s, usc, r.compo, mmu=r.mmu, mlambda=r.mlambda, vmu=r.vmu, vlambda=r.vlambda,
                         do_bias=do_bias)
        hits, st = api.pipeline_filters(ctx, p, s, vprof=vp, compo=r.compo if do_bias else None, vmu=r.vmu,
                                        vlambda=r.vlambda, block_size=1000)
        want = np.nonzero(o["stage"] == 3)[0]
        assert np.array_equal(hits["seq_index"], want)
        assert np.array_equal(bits(hits["filtersc"]), bits(o["filtersc"][want]))
        assert np.array_equal(bits(hits["vfsc"]), bits(o["vfsc"][want]))
        assert st.n_past_bias == int((o["stage"][o["stage"] != 255] >= 2).sum())
    hits, st = api.pipeline_filters(ctx, p, s, compo=r.compo, block_size=1000)   # no Viterbi stage
    o = O.pipe_batch(vp, s, usc, r.compo, mmu=r.mmu, mlambda=r.mlambda, vmu=r.vmu, vlambda=r.vlambda)
    want = np.nonzero((o["stage"] >= 2) & (o["stage"] != 255))[0]
    assert np.array_equal(hits["seq_index"], want) and np.isnan(hits["vfsc"]).all()
    assert st.n_past_vit == 0 and st.n_past_bias == want.size


def test_pipeline_filters_stop_and_errors(ctx):
    r, s, p, vp = load("tut_globins4")
    seen = []

    def stop(i, *a):
        seen.append(i)
        return True
    with pytest.raises(api.MSVError) as e:
        api.pipeline_filters(ctx, p, s, vprof=vp, compo=r.compo, vmu=r.vmu, vlambda=r.vlambda, on_hit=stop,
                             n_workers=1)
    assert e.value.code == api.eslFAIL
    assert len(seen) == 1
    other = F.read_vprofile(os.path.join(GOLDEN, "vit_tut_fn3.vprof"))
    with pytest.raises(api.MSVError) as e:
        api.pipeline_filters(ctx, p, s, vprof=other, compo=r.compo)
    assert e.value.code == api.eslEINVAL
    with pytest.raises(api.MSVError) as e:
        api.biasfilter(ctx, r.compo, r.M, api.DeviceDB(ctx, s), np.array([s.n]))
    assert e.value.code == api.eslEINVAL


def test_fn3_pipeline_statistics_match_tutorial_output(ctx):
    """tutorial/fn3.out:106-112: one 86-node query, one target of 2554
    residues (7LESS_DROME), passed the MSV, bias and Vit filters."""
    r, s, p, vp = load("tut_fn3")
    i = 46                                                  # globins45.fa (45), HBB_HUMAN, then 7LESS_DROME
    one = s.subset(np.array([i]))
    hits, st = api.pipeline_filters(ctx, p, one, vprof=vp, compo=r.compo, vmu=r.vmu, vlambda=r.vlambda)
    assert p.M == 86
    assert (st.nseqs, st.nres) == (1, 2554)
    assert (st.n_past_msv, st.n_past_bias, st.n_past_vit) == (1, 1, 1)
    assert hits["seq_index"].tolist() == [0] and r.stage[i] == 3


def test_biasfilter_matches_oracle_at_scale(ctx):
    """Millions of rows: background sequences, sequences drawn from the
    model's composition and from its commonest residues, all 29 codes."""
    r, s0, p, vp = load("tut_pkinase")
    rng = np.random.default_rng(9)
    top = np.argsort(-r.compo)[:4]
    extra = [rng.choice(20, size=int(rng.integers(50, 3000)), p=r.compo / r.compo.sum()).astype(np.uint8)
             for _ in range(300)]
    extra += [rng.choice(top, size=int(rng.integers(50, 3000))).astype(np.uint8) for _ in range(300)]
    extra += [rng.integers(0, 29, size=int(rng.integers(1, 2000)), dtype=np.uint8) for _ in range(300)]
    s = F.SeqSet.concat([F.synth_sequences(6000, seed=31, lmax=6000), F.SeqSet.from_list(extra)])
    got = api.biasfilter(ctx, r.compo, r.M, api.DeviceDB(ctx, s))
    want = O.bias_batch(r.compo, r.M, s)
    assert s.total > 2_500_000
    assert np.array_equal(got.view(np.uint32), want.view(np.uint32))


def test_pipeline_filters_large_block_equals_small_blocks(ctx):
    """A block above 64M residues goes through the MSV stage in several
    chunks (sorted chunk by chunk, searched as they arrive) and stays resident
    for the bias and Viterbi stages, which then list their sequences by
    length: the same hits, scores and counters as small blocks (one chunk
    each)."""
    p = F.read_profile(os.path.join(GOLDEN, "pipe_m400_s1.prof"))
    vp = F.read_vprofile(os.path.join(GOLDEN, "vit_m400_s1.vprof"))
    r = F.read_pipe(os.path.join(GOLDEN, "pipe_m400_s1.pres"))
    s = F.SeqSet.concat([F.synth_sequences(200_000, seed=1200, lmax=35000),
                         F.emit_homologs(p, 4000, seed=1201, lmax=35000)])
    assert s.total >= 64 << 20
    kw = dict(vprof=vp, compo=r.compo, vmu=r.vmu, vlambda=r.vlambda, n_workers=3)
    big, sb = api.pipeline_filters(ctx, p, s, block_size=s.n, **kw)
    small, ss = api.pipeline_filters(ctx, p, s, block_size=s.n // 4 + 1, **kw)
    assert sb.n_past_msv == ss.n_past_msv > 0 and sb.n_past_bias == ss.n_past_bias
    assert sb.n_past_vit == ss.n_past_vit > 0
    assert np.array_equal(big["seq_index"], small["seq_index"])
    for f in ("usc", "nullsc", "filtersc", "vfsc"):
        assert np.array_equal(bits(big[f]), bits(small[f])), f
