"""The drop-in p7_MSVFilter (msvgb_MSVFilter) keeps a per-context cache of
uploaded profiles. A cache hit must never score a profile with another
profile's tables: entries are found by the caller's rbv pointer or by a
content hash, and confirmed byte for byte. These tests make both keys lie --
every content hash collides (MSVGB_TEST_HASH_BITS=0), and one rbv buffer is
rewritten in place with another profile -- and check every call against the
oracle (p7_MSVFilter restated in C, pinned to the reference's goldens)."""
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def _call(ctx, p, codes):
    L = len(codes)
    dsq = np.concatenate([[255], codes, [255]]).astype(np.uint8)
    return ctx.MSVFilter(dsq, L, p, api.tjb_b(p.scale_b, L))


def _oracle(p, codes):
    st, xj, sc, _ = O.msv_filter(p, codes)
    return st, sc


def _same(got, want):
    return got[0] == want[0] and np.float32(got[1]).view(np.uint32) == np.float32(want[1]).view(np.uint32)


@pytest.fixture
def colliding_ctx(monkeypatch):
    monkeypatch.setenv("MSVGB_TEST_HASH_BITS", "0")       # read when the context is created
    ctx = api.Context(0)
    yield ctx
    ctx.close()


def test_colliding_hashes_never_share_tables(colliding_ctx):
    profs = [F.read_profile(os.path.join(GOLDEN, "m200_s1.prof")),
             api.sample_profile(200, 2),                       # same M, other content
             api.sample_profile(200, 3),
             F.read_profile(os.path.join(GOLDEN, "m400_s1.prof"))]
    s = F.SeqSet.concat([F.synth_sequences(12, seed=41, lmax=900)] +
                        [F.emit_homologs(p, 2, seed=42 + i) for i, p in enumerate(profs)])
    for i in range(s.n):
        for p in profs:                                        # interleaved: every call switches profile
            assert _same(_call(colliding_ctx, p, s.seq(i)), _oracle(p, s.seq(i)))


def test_rbv_buffer_rewritten_in_place(colliding_ctx):
    """The same rbv address holds another profile's bytes on the next call."""
    a, b = api.sample_profile(300, 5), api.sample_profile(300, 6)
    assert not np.array_equal(a.rbv, b.rbv)
    buf = np.ascontiguousarray(a.rbv.copy())
    p = F.Profile(M=a.M, rbv=buf, tbm_b=a.tbm_b, tec_b=a.tec_b, base_b=a.base_b, bias_b=a.bias_b,
                  scale_b=a.scale_b, mmu=a.mmu, mlambda=a.mlambda)
    s = F.SeqSet.concat([F.emit_homologs(a, 3, seed=51), F.emit_homologs(b, 3, seed=52),
                         F.synth_sequences(4, seed=53, lmax=600)])
    for i in range(s.n):
        for src in (a, b, a):
            buf[...] = src.rbv                                 # same pointer, new content
            p.tbm_b, p.tec_b, p.base_b, p.bias_b = src.tbm_b, src.tec_b, src.base_b, src.bias_b
            assert _same(_call(colliding_ctx, p, s.seq(i)), _oracle(src, s.seq(i)))
