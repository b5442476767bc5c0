"""The SSV pass with 16 or 8 lanes per sequence (several sequences per warp in
lockstep) followed by the full MSV on the undecided ones: bit-exact with the
reference's golden vectors and the oracle, including models whose length
disables SSV for some targets (all of them then go to the full MSV)."""
import glob
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
CASES = sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.res")))


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0)
    yield c
    c.close()


def lanes_ok(M, G):
    return G == 32 or (2 * G <= M < 64 * G)


@pytest.mark.parametrize("f16_only", [False, True])
@pytest.mark.parametrize("G", [16, 8])
@pytest.mark.parametrize("name", CASES)
def test_lanes_match_reference_golden(ctx, name, G, f16_only):
    p = F.read_profile(os.path.join(GOLDEN, name + ".prof"))
    if not lanes_ok(p.M, G):
        pytest.skip("model length outside this lane count's range")
    s = F.read_seqs(os.path.join(GOLDEN, name + ".seqs"))
    r = F.read_results(os.path.join(GOLDEN, name + ".res"))
    dp = api.DeviceProfile(ctx, p)
    dp.set_lanes(G)
    assert dp.lanes == G
    if f16_only:
        dp.set_int8_words(0)
    xj, fl = api.search(ctx, dp, api.DeviceDB(ctx, s))
    assert np.array_equal((fl & api.FLAG_ERANGE) != 0, r.status == F.eslERANGE)
    assert np.array_equal((fl & api.FLAG_PASS) != 0, r.passed == 1)
    sc = api.scores(p, s.lengths, xj, fl)
    assert np.array_equal(sc.view(np.uint32), r.sc.view(np.uint32))


@pytest.mark.parametrize("M,G", [(16, 8), (17, 8), (31, 8), (32, 16), (100, 8), (127, 8), (128, 16),
                                 (255, 8), (300, 16), (511, 8), (777, 16), (1023, 16)])
def test_lanes_random_profiles_and_extremes(ctx, M, G):
    rng = np.random.default_rng(M * 10 + G)
    for bias, tbm in ((int(rng.integers(5, 40)), int(rng.integers(5, 60))), (90, 130), (14, 120)):
        costs = rng.integers(0, 60, size=(F.KP_AMINO, M)).astype(np.uint8)
        p = F.profile_from_node_costs(costs, tbm_b=tbm, tec_b=3, base_b=190, bias_b=bias,
                                      scale_b=4.328085, mmu=-9.0, mlambda=0.69)
        seqs = [rng.integers(0, 20, size=L).astype(np.uint8) for L in (1, 2, 3, 5, 17, 250, 1999)]
        s = F.SeqSet.concat([F.SeqSet.from_list(seqs + [np.zeros(0, np.uint8)]),
                             F.synth_sequences(400, seed=M + G, lmax=4000)])
        o = O.msv_batch(p, s)
        dp = api.DeviceProfile(ctx, p)
        dp.set_lanes(G)
        xj, fl = api.search(ctx, dp, api.DeviceDB(ctx, s))
        ok = o["status"] == F.eslOK
        nonempty = s.lengths > 0
        assert np.array_equal((fl & api.FLAG_ERANGE) != 0, o["status"] == F.eslERANGE)
        assert np.array_equal(xj[ok], o["xj"][ok])
        assert np.array_equal(((fl & api.FLAG_PASS) != 0)[nonempty], o["pass"][nonempty] == 1)
        assert np.array_equal(((fl & api.FLAG_FULL) != 0)[nonempty], o["path"][nonempty] == 1)
        assert np.all((fl[~nonempty] & api.FLAG_EMPTY) != 0)


def test_lanes_rejected_out_of_range(ctx):
    p = F.read_profile(os.path.join(GOLDEN, "m2400_s1.prof"))
    dp = api.DeviceProfile(ctx, p)
    with pytest.raises(api.MSVError):
        dp.set_lanes(16)
    with pytest.raises(api.MSVError):
        dp.set_lanes(12)


# (DP words per lane, lanes, 8-bit words) of the compiled mixed-width kernels
HYB = [(10, 8, 4), (13, 8, 4), (17, 8, 4), (18, 8, 8), (26, 8, 8), (26, 8, 12), (32, 8, 8), (32, 8, 16),
       (13, 16, 4), (23, 16, 4), (24, 16, 8), (32, 16, 8)]


def _random_profile(rng, M, bias, tbm):
    costs = rng.integers(0, 60, size=(F.KP_AMINO, M)).astype(np.uint8)
    return F.profile_from_node_costs(costs, tbm_b=tbm, tec_b=3, base_b=190, bias_b=bias,
                                     scale_b=4.328085, mmu=-9.0, mlambda=0.69)


@pytest.mark.parametrize("C,G,CI", HYB)
def test_mixed_width_table_matches_oracle(ctx, C, G, CI):
    """The mixed-width SSV table (the last CI words of a lane as 8-bit costs)
    at both ends of the model-length range of its DP width, with ordinary
    and extreme scalar costs (SSV guard off, tjb+tbm wrap, large bias)."""
    rng = np.random.default_rng(C * 100 + G + CI)
    for M in (2 * G * (C - 1), 2 * G * C - 1):
        for bias, tbm in ((int(rng.integers(5, 40)), int(rng.integers(5, 60))), (90, 130), (14, 120)):
            p = _random_profile(rng, M, bias, tbm)
            seqs = [rng.integers(0, 20, size=L).astype(np.uint8) for L in (1, 2, 3, 5, 17, 250, 1999)]
            s = F.SeqSet.concat([F.SeqSet.from_list(seqs + [np.zeros(0, np.uint8)]),
                                 F.synth_sequences(300, seed=M + CI, lmax=3000)])
            o = O.msv_batch(p, s)
            dp = api.DeviceProfile(ctx, p)
            dp.set_lanes(G)
            dp.set_int8_words(CI)
            assert dp.int8_words == CI
            xj, fl = api.search(ctx, dp, api.DeviceDB(ctx, s))
            ok = o["status"] == F.eslOK
            nonempty = s.lengths > 0
            assert np.array_equal((fl & api.FLAG_ERANGE) != 0, o["status"] == F.eslERANGE)
            assert np.array_equal(xj[ok], o["xj"][ok])
            assert np.array_equal(((fl & api.FLAG_PASS) != 0)[nonempty], o["pass"][nonempty] == 1)
            assert np.array_equal(((fl & api.FLAG_FULL) != 0)[nonempty], o["path"][nonempty] == 1)


@pytest.mark.parametrize("name,G,CI", [("m400_s1", 8, 8), ("m400_s1", 8, 12), ("m400_s1", 16, 4),
                                       ("m200_s1", 8, 4)])
def test_mixed_width_table_matches_reference_golden(ctx, name, G, CI):
    p = F.read_profile(os.path.join(GOLDEN, name + ".prof"))
    s = F.read_seqs(os.path.join(GOLDEN, name + ".seqs"))
    r = F.read_results(os.path.join(GOLDEN, name + ".res"))
    dp = api.DeviceProfile(ctx, p)
    dp.set_lanes(G)
    dp.set_int8_words(CI)
    xj, fl = api.search(ctx, dp, api.DeviceDB(ctx, s))
    assert np.array_equal((fl & api.FLAG_ERANGE) != 0, r.status == F.eslERANGE)
    assert np.array_equal((fl & api.FLAG_PASS) != 0, r.passed == 1)
    sc = api.scores(p, s.lengths, xj, fl)
    assert np.array_equal(sc.view(np.uint32), r.sc.view(np.uint32))


def test_mixed_width_rejects_uncompiled_and_32_lanes(ctx):
    p = F.read_profile(os.path.join(GOLDEN, "m400_s1.prof"))
    dp = api.DeviceProfile(ctx, p)
    dp.set_lanes(32)
    with pytest.raises(api.MSVError):
        dp.set_int8_words(8)
    dp.set_lanes(8)
    with pytest.raises(api.MSVError):
        dp.set_int8_words(24)          # not compiled for 26 words at 8 lanes
    dp.set_int8_words(12)
    dp.set_lanes(8)
    assert dp.int8_words == 8          # set_lanes restores the default share (26 words per lane: 8)
    dp.set_int8_words(0)
    assert dp.int8_words == 0


@pytest.mark.parametrize("M", [1024, 1100, 1500, 1984, 2047])
def test_split_32_lane_passes_match_oracle(ctx, M):
    """Models of 1024 to 2047 nodes at 32 lanes: the SSV pass on 32-lane
    groups with the mixed-width table, then the full MSV of the undecided on
    the same groups, with ordinary and extreme scalar costs."""
    rng = np.random.default_rng(M + 7)
    for bias, tbm in ((int(rng.integers(5, 40)), int(rng.integers(5, 60))), (90, 130), (14, 120)):
        p = _random_profile(rng, M, bias, tbm)
        seqs = [rng.integers(0, 20, size=L).astype(np.uint8) for L in (1, 2, 3, 5, 17, 250, 2999)]
        s = F.SeqSet.concat([F.SeqSet.from_list(seqs + [np.zeros(0, np.uint8)]),
                             F.synth_sequences(200, seed=M, lmax=4000)])
        o = O.msv_batch(p, s)
        dp = api.DeviceProfile(ctx, p)
        dp.set_lanes(32)
        assert dp.lanes == 32 and dp.int8_words == 8
        xj, fl = api.search(ctx, dp, api.DeviceDB(ctx, s))
        ok = o["status"] == F.eslOK
        nonempty = s.lengths > 0
        assert np.array_equal((fl & api.FLAG_ERANGE) != 0, o["status"] == F.eslERANGE)
        assert np.array_equal(xj[ok], o["xj"][ok])
        assert np.array_equal(((fl & api.FLAG_PASS) != 0)[nonempty], o["pass"][nonempty] == 1)
        assert np.array_equal(((fl & api.FLAG_FULL) != 0)[nonempty], o["path"][nonempty] == 1)


@pytest.mark.parametrize("name", ["m1500_s2", "m2400_s1"])
def test_32_lanes_match_reference_golden(ctx, name):
    """32 lanes: the split passes at M = 1500, the fused kernel at M = 2400."""
    p = F.read_profile(os.path.join(GOLDEN, name + ".prof"))
    s = F.read_seqs(os.path.join(GOLDEN, name + ".seqs"))
    r = F.read_results(os.path.join(GOLDEN, name + ".res"))
    dp = api.DeviceProfile(ctx, p)
    dp.set_lanes(32)
    assert dp.int8_words == (8 if p.M < 2048 else 0)
    xj, fl = api.search(ctx, dp, api.DeviceDB(ctx, s))
    assert np.array_equal((fl & api.FLAG_ERANGE) != 0, r.status == F.eslERANGE)
    assert np.array_equal((fl & api.FLAG_PASS) != 0, r.passed == 1)
    sc = api.scores(p, s.lengths, xj, fl)
    assert np.array_equal(sc.view(np.uint32), r.sc.view(np.uint32))
