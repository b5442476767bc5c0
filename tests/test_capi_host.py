"""CPU-only checks of the C ABI library: it loads, exports every function
include/msvgb.h declares, its host-side score helpers equal the oracle's
restatement of the reference expressions, and it fails cleanly without a GPU."""
import ctypes
import os
import re

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions(header="msvgb.h"):
    src = open(os.path.join(ROOT, "include", header)).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(msvgb_\w+)\s*\(", src)))


def test_library_exports_every_declared_function():
    lib = api.lib()
    declared = header_functions()
    assert len(declared) >= 18
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(api.EXPORTS) == declared


def test_probe_library_exports_its_header():
    """The benchmark's peak probes live in a library of their own."""
    lib = ctypes.CDLL(os.path.join(ROOT, "cudahmmsearch_gb300", "libmsvgb_probe.so"))
    declared = header_functions("msvgb_probe.h")
    assert declared == ["msvgb_measure_int_peak", "msvgb_measure_smem_peak", "msvgb_probe_last_error"]
    for name in declared:
        assert hasattr(lib, name), name
    assert not hasattr(api.lib(), "msvgb_measure_int_peak")


@pytest.mark.parametrize("L", [0, 1, 2, 3, 10, 100, 300, 1000, 5000, 35000, 100000])
def test_tjb_matches_oracle(L):
    scale = np.float32(3.0 / 0.69314718055994529)
    assert api.tjb_b(float(scale), L) == O.tjb_b(float(scale), L)


def test_score_and_f1_match_oracle():
    p = F.read_profile(os.path.join(ROOT, "tests", "golden", "m200_s1.prof"))
    lib = api.lib()
    rng = np.random.default_rng(0)
    for _ in range(300):
        L = int(rng.integers(1, 5000))
        xj = int(rng.integers(0, 255))
        tjb = O.tjb_b(p.scale_b, L)
        sc = lib.msvgb_score(xj, 0, L, p.base_b, p.scale_b)
        assert np.float32(sc).view(np.uint32) == np.float32(O.score_from_xj(xj, tjb, p.base_b, p.scale_b)).view(np.uint32)
        P = ctypes.c_double()
        got = lib.msvgb_f1_pass(sc, L, p.mmu, p.mlambda, 0.02, ctypes.byref(P))
        want, _, Pw = O.f1_pass(sc, L, p.mmu, p.mlambda, 0.02)
        assert bool(got) == want and P.value == Pw
    assert lib.msvgb_score(0, api.FLAG_ERANGE, 100, p.base_b, p.scale_b) == float("inf")


def test_context_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(api.MSVError):
        api.Context(0)


def test_filter_stage_helpers_match_reference():
    """The host expressions of the stages after MSV, against the reference's
    own pipeline results (tests/golden/pipe_*.pres) and the oracle:
    p7_bg_NullOne, the stage gate, the ViterbiFilter score from xC."""
    import glob
    lib = api.lib()
    gold = os.path.join(ROOT, "tests", "golden")
    for pres in sorted(glob.glob(os.path.join(gold, "pipe_*.pres"))):
        name = os.path.basename(pres)[5:-5]
        r = F.read_pipe(pres)
        s = F.read_seqs(os.path.join(gold, "pipe_" + name + ".seqs"))
        vp = F.read_vprofile(os.path.join(gold, "vit_" + name + ".vprof"))
        vo, keep = api._vom_struct(vp)
        for i in range(s.n):
            L = int(s.lengths[i])
            if L == 0:
                continue
            ns = lib.msvgb_null_score(L)
            assert np.float32(ns).view(np.uint32) == r.nullsc[i:i + 1].view(np.uint32)[0]
            ok, P = api.stage_pass(float(r.usc[i]), float(r.nullsc[i]), r.mmu, r.mlambda, r.F1)
            assert ok == (r.stage[i] >= 1)
            assert P == O.gumbel_P(float(r.usc[i]), float(r.nullsc[i]), r.mmu, r.mlambda)
            if r.stage[i] >= 1:
                ok2, _ = api.stage_pass(float(r.usc[i]), float(r.fsc[i]), r.mmu, r.mlambda, r.F1)
                assert ok2 == (r.stage[i] >= 2)
            if np.isfinite(r.vfsc[i]):
                st, sc, xc = O.vit_filter(vp, s.seq(i))
                got = lib.msvgb_vit_score(xc, 1 if st == 16 else 0, L, ctypes.byref(vo))
                assert np.float32(got).view(np.uint32) == r.vfsc[i:i + 1].view(np.uint32)[0]


def test_bias_length_term_matches_reference():
    """msvgb_bias_length_term(fwd, L) adds exactly what p7_bg_FilterScore adds
    to the Forward score: the reference's score minus the Forward part of the
    oracle's restatement, for every sequence of a golden set."""
    lib = api.lib()
    gold = os.path.join(ROOT, "tests", "golden")
    r = F.read_pipe(os.path.join(gold, "pipe_tut_fn3.pres"))
    s = F.read_seqs(os.path.join(gold, "pipe_tut_fn3.seqs"))
    for i in range(0, s.n, 7):
        L = int(s.lengths[i])
        if L == 0:
            continue
        p1 = np.float32(L) / np.float32(L + 1)
        fwd = np.float32(r.fsc[i]) - (np.float32(L) * np.float32(np.log(p1))) - np.float32(np.log(np.float32(1.0 - np.float64(p1))))
        # the library's term applied to a Forward score gives back a float sum of the same three terms
        got = lib.msvgb_bias_length_term(float(fwd), L)
        want = np.float32(np.float32(fwd) + np.float32(L) * np.float32(np.log(p1))) + np.float32(np.log(np.float32(1.0 - np.float64(p1))))
        assert abs(float(got) - float(want)) <= 1e-5 * max(1.0, abs(float(want)))


@pytest.mark.parametrize("bad", ["dtype", "size", "stride"])
def test_search_host_rejects_bad_result_buffers(bad):
    """search_host's out=(xj, flags) must be two contiguous uint8 arrays of n
    entries; anything else is refused on the host, before any GPU call."""
    s = F.synth_sequences(10, seed=3, lmax=50)
    ok = np.zeros(s.n, np.uint8)
    wrong = {"dtype": np.zeros(s.n, np.int16), "size": np.zeros(s.n + 1, np.uint8),
             "stride": np.zeros(2 * s.n, np.uint8)[::2]}[bad]
    with pytest.raises(ValueError):
        api.search_host(None, None, s, out=(ok, wrong))
