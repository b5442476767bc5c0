"""The bias-filter oracle and the oracle of p7_Pipeline's filter gates,
pinned to the reference's own results (tests/golden/pipe_*.pres, written by
p7_bg_FilterScore and the p7_Pipeline stage sequence of HMMER 3.1b1): the
bias-filter score of every sequence bit for bit, the stage every sequence
reaches, and the ViterbiFilter score where the pipeline runs it."""
import glob
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
PIPE = sorted(os.path.basename(p)[5:-5] for p in glob.glob(os.path.join(GOLDEN, "pipe_*.pres")))


def load(name):
    r = F.read_pipe(os.path.join(GOLDEN, "pipe_" + name + ".pres"))
    s = F.read_seqs(os.path.join(GOLDEN, "pipe_" + name + ".seqs"))
    prof = os.path.join(GOLDEN, "pipe_" + name + ".prof")
    p = F.read_profile(prof if os.path.exists(prof) else os.path.join(GOLDEN, name + ".prof"))
    vp = F.read_vprofile(os.path.join(GOLDEN, "vit_" + name + ".vprof"))
    return r, s, p, vp


def test_pipe_goldens_cover_every_stage():
    assert len(PIPE) == 7
    total = np.zeros(4, np.int64)
    for name in PIPE:
        r = F.read_pipe(os.path.join(GOLDEN, "pipe_" + name + ".pres"))
        total += np.bincount(r.stage[r.stage < 4], minlength=4)
    assert (total >= 50).all(), total


@pytest.mark.parametrize("name", PIPE)
def test_bias_filter_matches_reference(name):
    r, s, p, vp = load(name)
    assert r.M == p.M == vp.M
    b = O.bias_batch(r.compo, r.M, s)
    ne = s.lengths > 0
    assert np.array_equal(b[ne].view(np.uint32), r.fsc[ne].view(np.uint32))


@pytest.mark.parametrize("name", PIPE)
def test_pipeline_stages_match_reference(name):
    r, s, p, vp = load(name)
    o = O.msv_batch(p, s)
    ne = s.lengths > 0
    assert np.array_equal(o["sc"][ne].view(np.uint32), r.usc[ne].view(np.uint32))
    q = O.pipe_batch(vp, s, r.usc, r.compo, mmu=r.mmu, mlambda=r.mlambda, vmu=r.vmu, vlambda=r.vlambda,
                     F1=r.F1, F2=r.F2)
    assert np.array_equal(q["stage"], r.stage)
    assert np.array_equal(q["nullsc"][ne].view(np.uint32), r.nullsc[ne].view(np.uint32))
    assert np.array_equal(q["vfsc"].view(np.uint32), r.vfsc.view(np.uint32))   # NaN where not run, same bits


def test_nobias_skips_the_filter():
    r, s, p, vp = load("tut_fn3")
    q = O.pipe_batch(vp, s, r.usc, r.compo, mmu=r.mmu, mlambda=r.mlambda, vmu=r.vmu, vlambda=r.vlambda,
                     do_bias=False)
    assert not (q["stage"] == 1).any()
    past = q["stage"] >= 1
    assert np.array_equal(q["filtersc"][past], q["nullsc"][past])
    assert (q["stage"] >= 2).sum() >= (r.stage >= 2).sum()
