"""GPU parity through the C ABI (libmsvgb.so) against the reference's golden
vectors and the oracle. Bit-exact: xJ, float score bit pattern (+inf on
overflow) and the F1 pass flag, for both SSV arithmetic variants."""
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


def load_case(name):
    return (F.read_profile(os.path.join(GOLDEN, name + ".prof")),
            F.read_seqs(os.path.join(GOLDEN, name + ".seqs")),
            F.read_results(os.path.join(GOLDEN, name + ".res")))


def check_against_oracle(p, s, xj, fl, o):
    nonempty = s.lengths > 0
    assert np.array_equal((fl & api.FLAG_ERANGE) != 0, o["status"] == F.eslERANGE)
    ok = o["status"] == F.eslOK
    assert np.array_equal(xj[ok], o["xj"][ok])
    assert np.array_equal(((fl & api.FLAG_PASS) != 0)[nonempty], o["pass"][nonempty] == 1)
    assert np.array_equal(((fl & api.FLAG_FULL) != 0)[nonempty], o["path"][nonempty] == 1)
    assert np.all((fl[~nonempty] & api.FLAG_EMPTY) != 0)


@pytest.mark.parametrize("variant", [0, 1])
@pytest.mark.parametrize("name", CASES)
def test_search_matches_reference_golden(ctx, name, variant):
    p, s, r = load_case(name)
    dp = api.DeviceProfile(ctx, p, variant)
    db = api.DeviceDB(ctx, s)
    xj, fl = api.search(ctx, dp, db)
    assert np.array_equal((fl & api.FLAG_ERANGE) != 0, r.status == F.eslERANGE)
    assert np.array_equal((fl & api.FLAG_PASS) != 0, r.passed == 1)
    sc = api.scores(p, s.lengths, xj, fl)
    assert np.array_equal(sc.view(np.uint32), r.sc.view(np.uint32))


@pytest.mark.parametrize("name", ["m1_s1", "m17_s2", "m200_s1", "m2400_s1"])
def test_dropin_msvfilter_matches_reference_golden(ctx, name):
    p, s, r = load_case(name)
    for i in range(0, s.n, max(1, s.n // 25)):
        L = int(s.lengths[i])
        dsq = np.concatenate([[255], s.seq(i), [255]]).astype(np.uint8)
        st, sc = ctx.MSVFilter(dsq, L, p, api.tjb_b(p.scale_b, L))
        assert st == r.status[i]
        assert np.float32(sc).view(np.uint32) == r.sc[i].view(np.uint32)


def test_dropin_rejects_small_omx(ctx):
    p, s, r = load_case("m200_s1")
    dsq = np.concatenate([[255], s.seq(0), [255]]).astype(np.uint8)
    with pytest.raises(api.MSVError) as e:
        ctx.MSVFilter(dsq, int(s.lengths[0]), p, 10, allocQ16=p.Q - 1)
    assert e.value.code == api.eslEINVAL


def test_dropin_empty_sequence_matches_oracle(ctx):
    p, _, _ = load_case("m50_s1")
    st, sc = ctx.MSVFilter(np.array([255, 255], np.uint8), 0, p, api.tjb_b(p.scale_b, 0))
    ost, oxj, osc, _ = O.msv_filter(p, np.zeros(0, np.uint8))
    assert st == ost and np.float32(sc).view(np.uint32) == np.float32(osc).view(np.uint32)


@pytest.mark.parametrize("variant", [0, 1])
def test_m200_20000_sequences_match_oracle(ctx, variant):
    """The M=200 (seed 1) profile against 20,000 synthetic sequences: lognormal
    lengths (median 300, sigma 0.7) clipped to [10, 5000], 0.5% X, 1% homologs."""
    p, _, _ = load_case("m200_s1")
    bgs = F.synth_sequences(19800, seed=11, lmax=5000)
    hom = F.emit_homologs(p, 200, seed=12)
    s = F.SeqSet.concat([bgs, hom])
    o = O.msv_batch(p, s)
    dp = api.DeviceProfile(ctx, p, variant)
    db = api.DeviceDB(ctx, s)
    xj, fl = api.search(ctx, dp, db)
    check_against_oracle(p, s, xj, fl, o)
    assert o["pass"].sum() >= 200


def test_m400_50000_subset_matches_oracle(ctx):
    """50,000-sequence subset of the M=400 workload (lengths clipped to [10, 35000], 2% homologs)."""
    p, _, _ = load_case("m400_s1")
    s = F.SeqSet.concat([F.synth_sequences(49000, seed=21, lmax=35000), F.emit_homologs(p, 1000, seed=22)])
    o = O.msv_batch(p, s)
    xj, fl = api.search(ctx, api.DeviceProfile(ctx, p), api.DeviceDB(ctx, s))
    check_against_oracle(p, s, xj, fl, o)


def test_m2400_length_extremes_and_saturation(ctx):
    """M=2400: lognormal plus long uniform [5000, 35000] lengths, and saturation
    sequences (an emitted core repeated 20 times) that must overflow to +inf."""
    p, _, _ = load_case("m2400_s1")
    s = F.SeqSet.concat([F.synth_sequences(1800, seed=31, lmax=35000, uniform_frac=0.1),
                         F.emit_homologs(p, 100, seed=32, repeat=20)])
    o = O.msv_batch(p, s)
    xj, fl = api.search(ctx, api.DeviceProfile(ctx, p), api.DeviceDB(ctx, s))
    check_against_oracle(p, s, xj, fl, o)
    assert (o["status"] == F.eslERANGE).sum() >= 50


@pytest.mark.parametrize("M", [1, 2, 3, 15, 16, 17, 63, 64, 65, 127, 128, 129, 1000, 2559, 2560, 3072, 3199, 3200,
                               3583, 4095, 4096, 6000, 8191])
def test_model_size_corners(ctx, M):
    """Node counts around the striping and lane boundaries, random profiles
    built directly from cost tables, tiny and all-X sequences."""
    rng = np.random.default_rng(M)
    costs = rng.integers(0, 40, size=(F.KP_AMINO, M)).astype(np.uint8)
    costs[20] = 255; costs[27:] = 255                       # gap, '*', '~': -inf scores
    p = F.profile_from_node_costs(costs, tbm_b=int(rng.integers(5, 60)), tec_b=3, base_b=190,
                                  bias_b=int(rng.integers(5, 40)), scale_b=3.0 / 0.6931471805599453,
                                  mmu=-9.0, mlambda=0.69)
    seqs = [rng.integers(0, 20, size=L).astype(np.uint8) for L in (1, 2, 3, 4, 5, 7, 16, 17, 100, 333)]
    seqs += [np.full(50, F.CODE_X, np.uint8), np.zeros(0, np.uint8), rng.integers(0, 29, size=77).astype(np.uint8)]
    s = F.SeqSet.from_list(seqs)
    o = O.msv_batch(p, s)
    for variant, lanes in ((0, None), (1, None), (None, None), (None, 8), (None, 16)):
        dp = api.DeviceProfile(ctx, p, variant)
        if lanes and 2 * lanes <= p.M < 64 * lanes:
            dp.set_lanes(lanes)                       # lane groups, long targets at 32 lanes beside them
        xj, fl = api.search(ctx, dp, api.DeviceDB(ctx, s))
        check_against_oracle(p, s, xj, fl, o)


@pytest.mark.parametrize("bias,tbm,base", [(0, 0, 190), (126, 5, 190), (200, 10, 190), (40, 100, 190),
                                           (14, 120, 100), (60, 40, 255), (90, 130, 190)])
def test_extreme_scalar_costs(ctx, bias, tbm, base):
    """Bias/transition corners: SSV guard off, tjb+tbm wrapping mod 256,
    base below tjb+tbm, bias >= 65 where the xB clamp matters."""
    rng = np.random.default_rng(bias * 1000 + tbm)
    M = 150
    costs = rng.integers(0, 255, size=(F.KP_AMINO, M)).astype(np.uint8)
    p = F.profile_from_node_costs(costs, tbm_b=tbm, tec_b=3, base_b=base, bias_b=bias,
                                  scale_b=3.0 / 0.6931471805599453, mmu=-9.0, mlambda=0.69)
    s = F.SeqSet.concat([F.synth_sequences(300, seed=bias + 7, lmax=3000),
                         F.SeqSet.from_list([rng.integers(0, 20, size=L).astype(np.uint8) for L in (1, 2, 9, 40000)])])
    o = O.msv_batch(p, s)
    for variant, lanes in ((0, None), (1, None), (None, None), (None, 8), (None, 16)):
        dp = api.DeviceProfile(ctx, p, variant)
        if lanes and 2 * lanes <= p.M < 64 * lanes:
            dp.set_lanes(lanes)                       # lane groups, long targets at 32 lanes beside them
        xj, fl = api.search(ctx, dp, api.DeviceDB(ctx, s))
        check_against_oracle(p, s, xj, fl, o)


def test_invalid_inputs_rejected(ctx):
    p, s, _ = load_case("m50_s1")
    bad = F.SeqSet.from_list([np.array([1, 2, 29], np.uint8)])
    with pytest.raises(api.MSVError) as e:
        api.DeviceDB(ctx, bad)
    assert e.value.code == api.eslEINVAL
    big = F.profile_from_node_costs(np.zeros((29, 8192), np.uint8), tbm_b=10, tec_b=3, base_b=190,
                                    bias_b=10, scale_b=4.328085, mmu=-9.0, mlambda=0.69)
    with pytest.raises(api.MSVError) as e:
        api.DeviceProfile(ctx, big)
    assert e.value.code == api.eslEINVAL


def test_kernel_launch_counter_advances(ctx):
    p, s, _ = load_case("m50_s1")
    prof, db = api.DeviceProfile(ctx, p), api.DeviceDB(ctx, s)
    before = api.kernel_launches()
    api.search(ctx, prof, db)
    assert api.kernel_launches() == before + 1      # a small search runs fused at 32 lanes, whatever the lane choice
    # lanes set explicitly apply at any size: the lane-group SSV pass and the
    # full-MSV pass, plus a 32-lane launch for targets of 2400 residues or more
    prof.set_lanes(8)
    before = api.kernel_launches()
    api.search(ctx, prof, db)
    assert api.kernel_launches() == before + 2 + int((s.lengths >= 2400).any())
    prof.set_lanes(32)
    before = api.kernel_launches()
    api.search(ctx, prof, db)
    assert api.kernel_launches() == before + 1


def test_profile_reused_across_databases_at_the_same_address(ctx):
    """A profile caches per-database length tables; a database created after
    another was destroyed (often at the same device address) must not reuse
    the old tables."""
    p, _, _ = load_case("m200_s1")
    prof = api.DeviceProfile(ctx, p)
    for k in range(4):
        s = F.SeqSet.concat([F.synth_sequences(300, seed=90 + k, lmax=300 + 1500 * k), F.emit_homologs(p, 5, seed=k)])
        db = api.DeviceDB(ctx, s)
        xj, fl = api.search(ctx, prof, db)
        o = O.msv_batch(p, s)
        check_against_oracle(p, s, xj, fl, o)
        db.close()


@pytest.mark.parametrize("chunk", [0, 1000, 60000])
def test_search_host_equals_resident_search(ctx, chunk):
    """msvgb_search_host (chunked upload and packing under the search) gives
    the resident path's results for any chunking, lane count and length mix."""
    p, _, _ = load_case("m400_s1")
    s = F.SeqSet.concat([F.synth_sequences(3000, seed=5, lmax=9000), F.emit_homologs(p, 50, seed=6),
                         F.SeqSet.from_list([np.zeros(0, np.uint8), np.array([7], np.uint8)])])
    o = O.msv_batch(p, s)
    for variant, lanes in ((None, None), (1, None), (None, 8)):
        dp = api.DeviceProfile(ctx, p, variant)
        if lanes:
            dp.set_lanes(lanes)
        a = api.search(ctx, dp, api.DeviceDB(ctx, s))
        b = api.search_host(ctx, dp, s, chunk_residues=chunk)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
        check_against_oracle(p, s, b[0], b[1], o)
    e = api.search_host(ctx, api.DeviceProfile(ctx, p), F.SeqSet.from_list([]))
    assert e[0].size == 0 and e[1].size == 0


@pytest.mark.parametrize("M", [2700, 3500, 4095, 5500, 8000])
def test_models_with_tables_in_global_memory(ctx, M):
    """Sampled models too large for shared-memory tables (M >= 2560): both
    tables stream from global memory; homologs, overflow repeats and long
    targets bit-exact with the oracle."""
    p = api.sample_profile(M, 7, ctx)
    s = F.SeqSet.concat([F.synth_sequences(300, seed=M, lmax=12000, uniform_frac=0.1),
                         F.emit_homologs(p, 20, seed=M + 1), F.emit_homologs(p, 5, seed=M + 2, repeat=6)])
    o = O.msv_batch(p, s)
    dp = api.DeviceProfile(ctx, p)
    assert dp.variant == 1 and dp.lanes == 32
    xj, fl = api.search(ctx, dp, api.DeviceDB(ctx, s))
    check_against_oracle(p, s, xj, fl, o)
    assert o["pass"].sum() >= 20


def test_search_host_default_chunks_equal_resident_search(ctx):
    """A database large enough for the default chunking (several chunks,
    sorted chunk by chunk, searched as each chunk's residues arrive, one
    full-MSV list at the end) and for lane groups: identical to the resident
    search, and to the oracle on a sample."""
    p, _, _ = load_case("m400_s1")
    s = F.SeqSet.concat([F.synth_sequences(200_000, seed=81, lmax=20000), F.emit_homologs(p, 2000, seed=82),
                         F.emit_homologs(p, 50, seed=83, repeat=20),
                         F.SeqSet.from_list([np.zeros(0, np.uint8), np.array([7], np.uint8)])])
    assert s.total >= 64 << 20
    dp = api.DeviceProfile(ctx, p)
    assert dp.lanes < 32
    a = api.search(ctx, dp, api.DeviceDB(ctx, s))
    for chunk in (0, s.total // 5):
        b = api.search_host(ctx, dp, s, chunk_residues=chunk)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    sub = np.random.default_rng(84).choice(s.n, size=3000, replace=False)
    sub = np.sort(np.concatenate([sub, np.arange(s.n - 1052, s.n)]))
    check_against_oracle(p, s.subset(sub), b[0][sub], b[1][sub], O.msv_batch(p, s.subset(sub)))


@pytest.mark.parametrize("code", [29, 30, 200, 255])
def test_search_host_rejects_invalid_codes_in_a_later_chunk(ctx, code):
    """An invalid residue code in a chunk searched after the first: the call
    fails with eslEINVAL (the chunk's search runs before the flag is read, on
    the padding code stored in its place), and the context stays usable."""
    p, _, _ = load_case("m200_s1")
    s = F.synth_sequences(4000, seed=91, lmax=3000)
    codes = s.codes.copy()
    codes[s.off[3500] + 1] = code
    bad = F.SeqSet(codes, s.off)
    dp = api.DeviceProfile(ctx, p)
    with pytest.raises(api.MSVError) as e:
        api.search_host(ctx, dp, bad, chunk_residues=s.total // 8)
    assert e.value.code == api.eslEINVAL
    good = api.search_host(ctx, dp, s, chunk_residues=s.total // 8)
    ref = api.search(ctx, dp, api.DeviceDB(ctx, s))
    assert np.array_equal(good[0], ref[0]) and np.array_equal(good[1], ref[1])


def test_host_sort_for_sequences_over_4M_residues(ctx):
    """A target longer than 4M residues sends the length sort to the host
    (resident creation, and the chunked host search with its per-chunk key):
    results equal the oracle's for every sequence, the long one included."""
    p, _, _ = load_case("m200_s1")
    rng = np.random.default_rng(97)
    long_seq = rng.integers(0, 20, size=4_300_000).astype(np.uint8)
    s = F.SeqSet.concat([F.synth_sequences(3000, seed=98, lmax=4000), F.emit_homologs(p, 20, seed=99),
                         F.SeqSet.from_list([long_seq]), F.synth_sequences(500, seed=100, lmax=900)])
    dp = api.DeviceProfile(ctx, p)
    a = api.search(ctx, dp, api.DeviceDB(ctx, s))
    b = api.search_host(ctx, dp, s, chunk_residues=s.total // 3)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    check_against_oracle(p, s, a[0], a[1], O.msv_batch(p, s))
