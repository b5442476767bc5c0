"""On-disk formats through the C ABI, host side only: the pressed MSV profile
reader/writer (.h3f, HMMER 3/f) and the FASTA reader. Pinned against the
reference's own tutorial files when they are present (the pressed minifam
library and FASTA files, whose reference readings are the tut_* golden
fixtures), and against Easel's documented digitization rules otherwise."""
import os
import struct

import numpy as np
import pytest

from cudahmmsearch_gb300 import api
from cudahmmsearch_gb300 import formats as F

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
TUTORIAL = os.environ.get("MSVGB_REFERENCE_TUTORIAL", "/root/reference/code/tutorial")
has_tutorial = pytest.mark.skipif(not os.path.isdir(TUTORIAL), reason="reference tutorial files not present")
TUT_MODELS = ["tut_globins4", "tut_fn3", "tut_pkinase"]


def golden_profile(name):
    return F.read_profile(os.path.join(GOLDEN, name + ".prof"))


def same_msv_fields(a, b):
    assert a.M == b.M
    assert np.array_equal(a.rbv, b.rbv)
    assert (a.tbm_b, a.tec_b, a.base_b, a.bias_b) == (b.tbm_b, b.tec_b, b.base_b, b.bias_b)
    assert np.float32(a.scale_b) == np.float32(b.scale_b)
    assert np.float32(a.mmu) == np.float32(b.mmu) and np.float32(a.mlambda) == np.float32(b.mlambda)


@has_tutorial
def test_reference_pressed_library_reads_as_the_reference_configures_it():
    got = api.read_h3f(os.path.join(TUTORIAL, "minifam.h3f"))
    assert [n for n, _ in got] == ["globins4", "fn3", "Pkinase"]
    for (_, p), name in zip(got, TUT_MODELS):
        same_msv_fields(p, golden_profile(name))


def h3f_records(b):
    """(sbv, rbv, evparam) byte ranges of each record of a pressed file."""
    pos, out = 0, []
    while pos < len(b):
        M, alpha, n = struct.unpack_from("<3i", b, pos + 4)
        q = max(2, (M - 1) // 16 + 1)
        sbv = pos + 4 + 12 + (n + 1) + 4 + 3 + 4 + 2
        rbv = sbv + 29 * (q + 17) * 16
        ev = rbv + 29 * q * 16
        out.append(((sbv, rbv), (rbv, ev), (ev, ev + 8)))
        pos = ev + 6 * 4 + 3 * 8 + 20 * 4 + 4
    return out


@has_tutorial
def test_writer_tables_equal_the_reference_pressed_ones(tmp_path):
    ref = open(os.path.join(TUTORIAL, "minifam.h3f"), "rb").read()
    profs = api.read_h3f(os.path.join(TUTORIAL, "minifam.h3f"))
    out = str(tmp_path / "mine.h3f")
    api.write_h3f(out, profs)
    mine = open(out, "rb").read()
    rr, mr = h3f_records(ref), h3f_records(mine)
    assert len(rr) == len(mr) == 3
    for a, b in zip(rr, mr):
        for (a0, a1), (b0, b1) in zip(a, b):     # sbv (sf_conversion of rbv), rbv, evparam[MMU, MLAMBDA]
            assert ref[a0:a1] == mine[b0:b1]


def test_h3f_round_trip(tmp_path):
    names = ["m50_s1", "m400_s1", "m2400_s1", "tut_fn3"]
    profs = [(n, golden_profile(n)) for n in names]
    path = str(tmp_path / "lib.h3f")
    api.write_h3f(path, profs)
    back = api.read_h3f(path)
    assert [n for n, _ in back] == names
    for (_, a), (_, b) in zip(profs, back):
        same_msv_fields(a, b)


def test_h3f_errors(tmp_path):
    path = str(tmp_path / "one.h3f")
    api.write_h3f(path, [("x", golden_profile("m50_s1"))])
    good = open(path, "rb").read()
    cases = {
        "truncated": good[:-10],
        "bad_magic": b"\0\0\0\0" + good[4:],
        "older_format": struct.pack("<I", 0xb3e5e6f3) + good[4:],
        "bad_sentinel": good[:-4] + b"\0\0\0\0",
    }
    for what, data in cases.items():
        p = tmp_path / (what + ".h3f")
        p.write_bytes(data)
        with pytest.raises(api.MSVError) as e:
            api.read_h3f(str(p))
        assert e.value.code == api.eslEFORMAT, what
    dna = bytearray(good)
    struct.pack_into("<i", dna, 8, 2)                # alphabet type: not amino
    (tmp_path / "dna.h3f").write_bytes(bytes(dna))
    with pytest.raises(api.MSVError) as e:
        api.read_h3f(str(tmp_path / "dna.h3f"))
    assert e.value.code == api.eslEINCOMPAT
    with pytest.raises(api.MSVError) as e:
        api.read_h3f(str(tmp_path / "missing.h3f"))
    assert e.value.code == api.eslENOTFOUND
    (tmp_path / "empty.h3f").write_bytes(b"")
    assert api.read_h3f(str(tmp_path / "empty.h3f")) == []


@has_tutorial
def test_reference_fasta_files_read_as_easel_reads_them():
    g = F.read_seqs(os.path.join(GOLDEN, "tut_fn3.seqs"))    # globins45.fa, HBB_HUMAN, ... as Easel digitized them
    s45, names45 = api.read_fasta(os.path.join(TUTORIAL, "globins45.fa"))
    hbb, names1 = api.read_fasta(os.path.join(TUTORIAL, "HBB_HUMAN"))
    assert s45.n == 45 and hbb.n == 1 and names1 == ["HBB_HUMAN"]
    assert names45[0] == "MYG_ESCGI"
    for i in range(45):
        assert np.array_equal(s45.seq(i), g.seq(i)), names45[i]
    assert np.array_equal(hbb.seq(0), g.seq(45))


SYMBOLS = "ACDEFGHIKLMNPQRSTVWY-BJZOUX*~"


def expected_codes(text):
    out = []
    for ch in text:
        if ch in " \t\r\n":
            continue
        if ch in "._":
            out.append(20)
        else:
            out.append(SYMBOLS.index(ch.upper()))
    return np.array(out, np.uint8)


def test_fasta_digitization_rules(tmp_path):
    rng = np.random.default_rng(3)
    records, text = [], []
    for i in range(40):
        L = int(rng.integers(0, 300))
        chars = rng.choice(list(SYMBOLS + SYMBOLS.lower().replace("-", "") + "._"), size=L)
        seq = "".join(chars)
        width = int(rng.integers(5, 80))
        lines = [seq[k:k + width] for k in range(0, len(seq), width)]
        eol = "\r\n" if i % 7 == 0 else "\n"
        head = f">seq{i}" + (f" some description {i}" if i % 3 else "")
        body = eol.join(" " + l if i % 5 == 0 else l for l in lines)
        text.append(head + eol + body + (eol if i % 4 else eol + eol))
        records.append((f"seq{i}", seq))
    path = tmp_path / "t.fa"
    path.write_text("\n\n" + "".join(text))
    s, names = api.read_fasta(str(path))
    assert names == [n for n, _ in records]
    for i, (_, seq) in enumerate(records):
        assert np.array_equal(s.seq(i), expected_codes(seq)), i


def test_fasta_errors_and_empty(tmp_path):
    for what, data in {"digit": ">a\nACD1E\n", "no_header": "ACDE\n>a\nAC\n", "no_name": ">  \nACD\n",
                       "illegal": ">a\nAC#D\n"}.items():
        p = tmp_path / (what + ".fa")
        p.write_text(data)
        with pytest.raises(api.MSVError) as e:
            api.read_fasta(str(p))
        assert e.value.code == api.eslEFORMAT, what
    p = tmp_path / "nonascii.fa"
    p.write_bytes(b">a\nAC\xc3\xa9D\n")
    with pytest.raises(api.MSVError) as e:
        api.read_fasta(str(p))
    assert e.value.code == api.eslEFORMAT
    (tmp_path / "empty.fa").write_text("")
    s, names = api.read_fasta(str(tmp_path / "empty.fa"))
    assert s.n == 0 and names == []
    (tmp_path / "blank.fa").write_text(">x\n\n>y\nAC\n")
    s, names = api.read_fasta(str(tmp_path / "blank.fa"))
    assert names == ["x", "y"] and s.lengths.tolist() == [0, 2]
    (tmp_path / "spaced.fa").write_bytes(b">\t name desc\rACD\r>z\rW\r")    # blanks before the name; '\r' line ends
    s, names = api.read_fasta(str(tmp_path / "spaced.fa"))
    assert names == ["name", "z"] and s.lengths.tolist() == [3, 1]
    with pytest.raises(api.MSVError) as e:
        api.read_fasta(str(tmp_path / "missing.fa"))
    assert e.value.code == api.eslENOTFOUND


@has_tutorial
def test_reference_pressed_rest_reads_as_the_reference_configures_it():
    """tutorial/minifam.h3p (hmmpress's second file): the ViterbiFilter part of
    each model equals the reference's own hmmsearch-configured profile
    (tests/golden/vit_tut_*.vprof) except the N/J/C move costs (pressed at
    length 400, configured at 100; recomputed per target length), and the
    .h3f record's composition and Viterbi Gumbel parameters equal those the
    reference's pipeline used (tests/golden/pipe_tut_*.pres)."""
    rest = api.read_h3p(os.path.join(TUTORIAL, "minifam.h3p"))
    msv = api.read_h3f(os.path.join(TUTORIAL, "minifam.h3f"), filter_params=True)
    assert [n for n, _ in rest] == ["globins4", "fn3", "Pkinase"] == [r[0] for r in msv]
    for (name, vp), (_, p, compo, vmu, vlambda), g in zip(rest, msv, ["tut_globins4", "tut_fn3", "tut_pkinase"]):
        want = F.read_vprofile(os.path.join(GOLDEN, "vit_" + g + ".vprof"))
        pipe = F.read_pipe(os.path.join(GOLDEN, "pipe_" + g + ".pres"))
        assert vp.M == want.M == p.M
        assert np.array_equal(vp.twv, want.twv) and np.array_equal(vp.rwv, want.rwv)
        assert (vp.scale_w, vp.nj, vp.base_w, vp.ddbound_w) == (want.scale_w, want.nj, want.base_w, want.ddbound_w)
        assert np.array_equal(vp.xw[0], want.xw[0]) and np.array_equal(vp.xw[1:, 1], want.xw[1:, 1])
        assert np.array_equal(compo.view(np.uint32), pipe.compo.view(np.uint32))
        assert (np.float32(vmu), np.float32(vlambda)) == (np.float32(pipe.vmu), np.float32(pipe.vlambda))


def test_h3p_errors(tmp_path):
    with pytest.raises(api.MSVError) as e:
        api.read_h3p(str(tmp_path / "missing.h3p"))
    assert e.value.code == api.eslENOTFOUND
    bad = tmp_path / "bad.h3p"
    bad.write_bytes(b"\x00" * 64)
    with pytest.raises(api.MSVError) as e:
        api.read_h3p(str(bad))
    assert e.value.code == api.eslEFORMAT


@has_tutorial
def test_h3p_rejects_corrupted_records(tmp_path):
    """The reference's minifam.h3p cut or altered at record boundaries and
    inside fields: every damaged copy is eslEFORMAT, never a wrong profile."""
    good = open(os.path.join(TUTORIAL, "minifam.h3p"), "rb").read()
    rest = api.read_h3p(os.path.join(TUTORIAL, "minifam.h3p"))
    M0 = rest[0][1].M

    def check(name, data):
        p = tmp_path / (name + ".h3p")
        p.write_bytes(data)
        with pytest.raises(api.MSVError) as e:
            api.read_h3p(str(p))
        assert e.value.code == api.eslEFORMAT, name

    for cut in (3, 11, 40, len(good) // 3, len(good) // 2, len(good) - 4, len(good) - 1):
        check(f"cut{cut}", good[:cut])
    bad = bytearray(good)
    bad[0] ^= 0xFF                                            # magic
    check("magic", bytes(bad))
    bad = bytearray(good)
    bad[4:8] = np.int32(M0 + 1).tobytes()                     # M: every later field shifts
    check("M", bytes(bad))
    bad = bytearray(good)
    bad[12:16] = np.int32(-5).tobytes()                       # name length
    check("namelen", bytes(bad))
