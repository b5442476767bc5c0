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


def header_functions():
    src = open(os.path.join(ROOT, "include", "msvgb.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(msvgb_\w+)\s*\(", src)))


def test_library_exports_every_declared_function():
    lib = api.lib()
    declared = header_functions()
    assert len(declared) >= 18
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(api.EXPORTS) == declared


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
