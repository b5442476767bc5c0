"""The on-disk formats feeding the device: pressed profiles and FASTA files
searched on the GPU give the reference's golden results, a packed database
saved and loaded back searches identically, and corrupted database files are
rejected before anything reaches the device. Includes the reference
tutorial's fn3 / 7LESS_DROME search (tutorial/fn3.out:109-110: one target,
passed the MSV filter)."""
import os

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F

pytestmark = pytest.mark.gpu
GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
SYMBOLS = "ACDEFGHIKLMNPQRSTVWY-BJZOUX*~"


@pytest.fixture(scope="module")
def ctx():
    c = api.Context(0)
    yield c
    c.close()


def load_case(name):
    return (F.read_profile(os.path.join(GOLDEN, name + ".prof")),
            F.read_seqs(os.path.join(GOLDEN, name + ".seqs")),
            F.read_results(os.path.join(GOLDEN, name + ".res")))


def check_golden(p, s, r, xj, fl):
    assert np.array_equal((fl & api.FLAG_ERANGE) != 0, r.status == F.eslERANGE)
    assert np.array_equal((fl & api.FLAG_PASS) != 0, r.passed == 1)
    sc = api.scores(p, s.lengths, xj, fl)
    assert np.array_equal(sc.view(np.uint32), r.sc.view(np.uint32))


def test_fn3_finds_7less_drome(ctx):
    p, s, r = load_case("tut_fn3")
    i = 46                                   # globins45.fa (45), HBB_HUMAN, then 7LESS_DROME
    assert s.lengths[i] == 2554              # "2554 residues searched"
    xj, fl = api.search(ctx, api.DeviceProfile(ctx, p), api.DeviceDB(ctx, s.subset(np.array([i]))))
    assert fl[0] & api.FLAG_PASS             # "Passed MSV filter: 1"
    assert (fl[0] & api.FLAG_ERANGE) != 0 and r.status[i] == F.eslERANGE


@pytest.mark.parametrize("name", ["tut_globins4", "tut_fn3", "tut_pkinase", "m400_s1"])
def test_pressed_profile_and_fasta_search_equal_golden(ctx, name, tmp_path):
    p, s, r = load_case(name)
    h3f = str(tmp_path / "lib.h3f")
    api.write_h3f(h3f, [("other", F.read_profile(os.path.join(GOLDEN, "m50_s1.prof"))), (name, p)])
    (_, _), (got_name, q) = api.read_h3f(h3f)
    assert got_name == name
    fa = tmp_path / "t.fa"
    with open(fa, "w") as f:
        for i in range(s.n):
            seq = "".join(SYMBOLS[c] for c in s.seq(i))
            f.write(f">s{i} desc\n" + "\n".join(seq[k:k + 60] for k in range(0, len(seq), 60)) + "\n")
    t, names = api.read_fasta(str(fa))
    assert names == [f"s{i}" for i in range(s.n)] and np.array_equal(t.codes, s.codes)
    xj, fl = api.search(ctx, api.DeviceProfile(ctx, q), api.DeviceDB(ctx, t))
    check_golden(p, s, r, xj, fl)


def test_packed_database_round_trip(ctx, tmp_path):
    p, s0, _ = load_case("tut_pkinase")
    s = F.SeqSet.concat([s0, F.synth_sequences(3000, seed=9, lmax=6000),
                         F.SeqSet.from_list([np.zeros(0, np.uint8), np.array([5], np.uint8)])])
    db = api.DeviceDB(ctx, s)
    path = str(tmp_path / "db.msvdb")
    db.save(path)
    back = api.DeviceDB.load(ctx, path)
    assert back.n == s.n and back.residues == s.total
    assert np.array_equal(back.lengths, s.lengths)
    for variant in (None, 1):
        dp = api.DeviceProfile(ctx, p, variant)
        a = api.search(ctx, dp, db)
        b = api.search(ctx, dp, back)
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_packed_database_rejects_corruption(ctx, tmp_path):
    s = F.SeqSet.concat([F.synth_sequences(200, seed=3, lmax=900), F.SeqSet.from_list([np.array([1, 2, 3], np.uint8)])])
    db = api.DeviceDB(ctx, s)
    path = tmp_path / "db.msvdb"
    db.save(str(path))
    good = bytearray(path.read_bytes())
    n = s.n
    hdr = 8 + 3 * 8
    len_off, start_off = hdr, hdr + 4 * n
    orig_off, codes_off = start_off + 8 * n, start_off + 16 * n
    lens = np.frombuffer(bytes(good[len_off:len_off + 4 * n]), np.int32)
    starts = np.frombuffer(bytes(good[start_off:start_off + 8 * n]), np.int64)
    last = n - 1                                      # the shortest sequence (3 residues)
    assert lens[last] == 3

    def corrupt(what, fn):
        b = bytearray(good)
        fn(b)
        p = tmp_path / (what + ".msvdb")
        p.write_bytes(bytes(b))
        with pytest.raises(api.MSVError) as e:
            api.DeviceDB.load(ctx, str(p))
        assert e.value.code == api.eslEFORMAT, what

    corrupt("magic", lambda b: b.__setitem__(slice(0, 8), b"NOTADB!!"))
    corrupt("truncated", lambda b: b.__delitem__(slice(len(b) - 100, len(b))))
    corrupt("code", lambda b: b.__setitem__(codes_off + int(starts[0]), 40))
    corrupt("padding", lambda b: b.__setitem__(codes_off + int(starts[last]) + 3, 5))
    corrupt("orig", lambda b: b.__setitem__(slice(orig_off, orig_off + 8), np.int64(n).tobytes()))
    corrupt("unsorted", lambda b: b.__setitem__(slice(len_off, len_off + 4), np.int32(1).tobytes()))
    corrupt("misaligned", lambda b: b.__setitem__(slice(start_off, start_off + 8), np.int64(int(starts[0]) + 4).tobytes()))
    with pytest.raises(api.MSVError) as e:
        api.DeviceDB.load(ctx, str(tmp_path / "missing.msvdb"))
    assert e.value.code == api.eslENOTFOUND


def test_database_memory_is_returned(ctx):
    """Databases come from a stream-ordered pool that keeps at most 4 GiB
    mapped: creating and destroying a database many times does not grow the
    device memory in use beyond that."""
    import torch
    s = F.synth_sequences(400_000, seed=3, lmax=4000)        # ~150 MB packed
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(25):
        db = api.DeviceDB(ctx, s)
        db.close()
    free1, _ = torch.cuda.mem_get_info()
    assert free0 - free1 < (4 << 30) + (256 << 20)
    for _ in range(25):
        db = api.DeviceDB(ctx, s)
        db.close()
    free2, _ = torch.cuda.mem_get_info()
    assert abs(free1 - free2) < (64 << 20)                    # steady state: nothing leaks
