"""The lane-count autotuner (msvgb_autotune / msvgb_tune_*) and the paths that
consult it: the fixed rule before tuning, a measured table that saves and
loads, rejection of foreign or malformed tables, and bit-exact results from
the plain, batched and serving paths when a table puts different length bins
of one profile on different lane counts."""
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def valid(M, lanes):
    return lanes == 32 or 2 <= M // (2 * lanes) + 1 <= 32


def test_rule_before_tuning():
    ctx = api.Context(0)
    try:
        for M, want in ((1, 32), (15, 32), (16, 8), (100, 8), (479, 8), (511, 8), (512, 16), (1023, 16), (1024, 32), (3000, 32)):
            assert ctx.tune_lanes(M)[0] == want, M
        for M, L, want in ((100, 50, 8), (100, 5000, 8), (600, 50, 16), (600, 599, 16), (600, 600, 32),
                           (1023, 149, 16), (1024, 50, 32)):
            assert ctx.tune_lanes(M, L)[0] == want, (M, L)
    finally:
        ctx.close()


@pytest.fixture(scope="module")
def tuned(tmp_path_factory):
    ctx = api.Context(0)
    path = str(tmp_path_factory.mktemp("tune") / "table.txt")
    assert ctx.autotune(budget_s=20.0, cache=path) == "measured"
    yield ctx, path
    ctx.close()


def test_autotune_table_is_valid_and_round_trips(tuned):
    ctx, path = tuned
    lines = open(path).read().splitlines()
    assert lines[0] == "msvgb-tune 2" and lines[1].startswith("device ")
    rows = [l for l in lines if l.startswith("m ")]
    assert len(rows) >= 5
    other = api.Context(0)
    try:
        assert other.autotune(cache=path) == "loaded"
        for M in (20, 50, 100, 250, 400, 700, 1000, 1500):
            for L in (-1, 50, 300, 1000, 5000):
                g = ctx.tune_lanes(M, L)
                assert g == other.tune_lanes(M, L)
                assert g[0] in (32, 16, 8) and valid(M, g[0])
                assert g[1] in (0, 1)
    finally:
        other.close()


def test_tune_load_rejects_foreign_and_malformed(tuned, tmp_path):
    ctx, path = tuned
    lines = open(path).read().splitlines()
    foreign = tmp_path / "foreign.txt"
    foreign.write_text("\n".join(["msvgb-tune 2", "device Some_Other_GPU 7"] + lines[2:]) + "\n")
    with pytest.raises(api.MSVError) as e:
        ctx.tune_load(str(foreign))
    assert e.value.code == api.eslEINCOMPAT
    bad = tmp_path / "bad.txt"
    bad.write_text("msvgb-tune 2\n" + lines[1] + "\nlbins 1 2 3\n")
    with pytest.raises(api.MSVError) as e:
        ctx.tune_load(str(bad))
    assert e.value.code == api.eslEFORMAT
    with pytest.raises(api.MSVError) as e:
        ctx.tune_load(str(tmp_path / "missing.txt"))
    assert e.value.code == api.eslENOTFOUND


def forced_table(path, out, per_bin, mix):
    """The measured table with every row's choices replaced: per_bin[b] and mix
    are candidate indices (0: 32 lanes f16, 1: 32 lanes int8, 2: 16 lanes, 3: 8 lanes)."""
    lines = open(path).read().splitlines()
    res = []
    for l in lines:
        if l.startswith("m "):
            t = l.split()
            gi = t.index("gcups")
            t = t[:3] + [str(x) for x in per_bin] + [str(mix)] + t[gi:]
        res.append(" ".join(t) if l.startswith("m ") else l)
    open(out, "w").write("\n".join(res) + "\n")


@pytest.fixture(scope="module")
def mixed_ctx(tuned, tmp_path_factory):
    _, path = tuned
    out = str(tmp_path_factory.mktemp("forced") / "forced.txt")
    forced_table(path, out, per_bin=[3, 2, 0, 1], mix=3)
    ctx = api.Context(0)
    ctx.tune_load(out)
    yield ctx
    ctx.close()


def mixed_db():
    rng = np.random.default_rng(5)
    # every length bin populated: [0,150) [150,600) [600,2400) [2400,inf)
    parts = [F.SeqSet.from_list([rng.integers(0, 20, size=L).astype(np.uint8)
                                 for L in rng.integers(lo, hi, size=n)])
             for lo, hi, n in ((1, 150, 900), (150, 600, 600), (600, 2400, 200), (2400, 7000, 40))]
    return F.SeqSet.concat(parts + [F.SeqSet.from_list([np.zeros(0, np.uint8)])])


def test_forced_choices_are_what_the_context_reports(mixed_ctx):
    assert mixed_ctx.tune_lanes(100, 50)[0] == 8
    assert mixed_ctx.tune_lanes(100, 300)[0] == 16
    assert mixed_ctx.tune_lanes(100, 1000) == (32, 1)
    assert mixed_ctx.tune_lanes(100, 5000) == (32, 0)
    assert mixed_ctx.tune_lanes(100)[0] == 8
    assert mixed_ctx.tune_lanes(700, 50)[0] == 16     # 8 lanes cannot hold M = 700: the rule's choice
    assert mixed_ctx.tune_lanes(700, 300)[0] == 16     # the forced table's [150, 600) choice
    assert mixed_ctx.tune_lanes(700, 1000) == (32, 1)


def test_batch_with_per_bin_lanes_matches_oracle(mixed_ctx):
    Ms = [17, 40, 100, 333, 511, 700, 1000, 1800]
    profs = [api.sample_profile(M, 300 + i, mixed_ctx) for i, M in enumerate(Ms)]
    s = F.SeqSet.concat([mixed_db(), F.emit_homologs(profs[2], 40, seed=8), F.emit_homologs(profs[3], 20, seed=9, repeat=8)])
    db = api.DeviceDB(mixed_ctx, s)
    bxj, bfl = api.search_batch(mixed_ctx, profs, db)
    nonempty = s.lengths > 0
    for i, p in enumerate(profs):
        o = O.msv_batch(p, s)
        ok = o["status"] == F.eslOK
        assert np.array_equal(bxj[i][ok], o["xj"][ok]), f"M={p.M}"
        assert np.array_equal((bfl[i] & api.FLAG_ERANGE) != 0, o["status"] == F.eslERANGE)
        assert np.array_equal(((bfl[i] & api.FLAG_PASS) != 0)[nonempty], o["pass"][nonempty] == 1)
        assert np.array_equal(((bfl[i] & api.FLAG_FULL) != 0)[nonempty], o["path"][nonempty] == 1)
        assert np.all((bfl[i][~nonempty] & api.FLAG_EMPTY) != 0)


def test_plain_and_served_with_tuned_lanes_match_oracle(mixed_ctx):
    s = mixed_db()
    db = api.DeviceDB(mixed_ctx, s)
    profs = [api.sample_profile(M, 400 + M, mixed_ctx) for M in (60, 300, 900)]
    srv = api.Server(mixed_ctx, db, max_slots=4, mem_budget=256 << 20)
    try:
        tickets = [srv.submit(p) for p in profs]
        served = [srv.wait(t) for t in tickets]
    finally:
        srv.close()
    for p, (sxj, sfl) in zip(profs, served):
        dp = api.DeviceProfile(mixed_ctx, p)
        assert dp.lanes == mixed_ctx.tune_lanes(p.M)[0]
        xj, fl = api.search(mixed_ctx, dp, db)
        o = O.msv_batch(p, s)
        ok = o["status"] == F.eslOK
        for gx, gf in ((xj, fl), (sxj, sfl)):
            assert np.array_equal(gx[ok], o["xj"][ok]), f"M={p.M}"
            assert np.array_equal((gf & api.FLAG_ERANGE) != 0, o["status"] == F.eslERANGE)
            assert np.array_equal(((gf & api.FLAG_PASS) != 0)[s.lengths > 0], o["pass"][s.lengths > 0] == 1)
