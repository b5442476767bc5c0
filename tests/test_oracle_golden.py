"""The CPU oracle against the golden vectors produced by the reference's own
compiled p7_MSVFilter and p7_Pipeline MSV stage (tests/golden/make_golden.py).
Bit-exact: status, float score bit pattern, F1 pass flag."""
import glob
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.res")))


def load_case(name):
    p = F.read_profile(os.path.join(GOLDEN, name + ".prof"))
    s = F.read_seqs(os.path.join(GOLDEN, name + ".seqs"))
    r = F.read_results(os.path.join(GOLDEN, name + ".res"))
    return p, s, r


def test_golden_cases_present():
    assert len(CASES) >= 10


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    p, s, r = load_case(name)
    o = O.msv_batch(p, s)
    assert np.array_equal(o["status"], r.status)
    assert np.array_equal(o["sc"].view(np.uint32), r.sc.view(np.uint32))
    assert np.array_equal(o["pass"], r.passed)


@pytest.mark.parametrize("name", CASES)
def test_oracle_xj_reproduces_score(name):
    """The float score is a function of (xJ, tjb_b(L)) only (msvfilter.c:205-210)."""
    p, s, r = load_case(name)
    o = O.msv_batch(p, s)
    for i in np.nonzero(o["status"] == F.eslOK)[0][:50]:
        L = int(s.lengths[i])
        sc = O.score_from_xj(int(o["xj"][i]), O.tjb_b(p.scale_b, L), p.base_b, p.scale_b)
        assert np.float32(sc).view(np.uint32) == r.sc[i].view(np.uint32)


def test_golden_covers_overflow_and_full_msv():
    n_erange = n_full = 0
    for name in CASES:
        p, s, r = load_case(name)
        o = O.msv_batch(p, s)
        n_erange += int((r.status == F.eslERANGE).sum())
        n_full += int(o["path"].sum())
    assert n_erange >= 5
    assert n_full >= 20


@pytest.mark.parametrize("name", ["m1_s1", "m2_s1", "m17_s2"])
def test_plain_msv_differs_from_ssv_floor_only_where_expected(name):
    """Without the SSV decision the plain recurrence can score lower (SSV floors
    the running max at the begin score); the reference result is the SSV one.
    On these tiny models the floor matters for some short targets: the plain
    recurrence must differ there, and only ever by scoring lower."""
    p, s, r = load_case(name)
    diffs = 0
    for i in range(s.n):
        if r.status[i] != F.eslOK:
            continue
        st, xj, sc, _ = O.msv_filter(p, s.seq(i), full_only=True)
        if np.float32(sc).view(np.uint32) != r.sc[i].view(np.uint32):
            diffs += 1
            assert sc < r.sc[i]
        # the full restatement (SSV decision first) is the reference's score
        st2, xj2, sc2, _ = O.msv_filter(p, s.seq(i))
        assert np.float32(sc2).view(np.uint32) == r.sc[i].view(np.uint32)
    assert diffs > 0
