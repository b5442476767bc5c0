"""Regenerates the golden MSV vectors in tests/golden/ from the reference itself.

Needs oracle/_ref/refgen, built from the reference's own sources by
``make -C oracle/ref REF=<reference>/code`` (x86-64 only: the reference MSV is
SSE2 code). For every case it

  1. samples the profile with HMMER's p7_hmm_Sample / p7_Calibrate /
     p7_ProfileConfig / p7_oprofile_Convert (``refgen profile``),
  2. builds a sequence set: fixed tiny lengths, lognormal-length background
     sequences with 0.5% X, sequences over all 29 codes (gap, degenerate,
     '*' and '~' included), p7_ProfileEmit homologs, and "saturation"
     sequences (an emitted sequence repeated R times) that drive the uint8
     score to overflow,
  3. scores every sequence with the reference's p7_MSVFilter and the
     p7_Pipeline MSV stage (``refgen score``).

Files per case NAME: NAME.prof (MSVPROF1), NAME.seqs (MSVSEQS1), NAME.res (MSVRES01).

The tut_* cases use the reference's tutorial models and sequences instead
(the Pfam models globins4, fn3 and Pkinase of tutorial/minifam, configured and
converted as hmmsearch does, ``refgen hmmfile``; tutorial/globins45.fa,
HBB_HUMAN and 7LESS_DROME read by Easel's sequence reader, ``refgen seqfile``;
p7_ProfileEmit homologs and saturation repeats of each model; background
sequences), so the fixtures pin the path on real profiles, including the
fn3 / 7LESS_DROME search of tutorial/fn3.out.
The vit_* files pin the ViterbiFilter stage (vit_NAME.vprof: the model's
int16 ViterbiFilter profile; vit_NAME.vres: p7_ViterbiFilter status and score
for every sequence of NAME.seqs).
The pipe_* files pin the bias filter and the gates of p7_Pipeline around it
and around the ViterbiFilter (pipe_NAME.seqs: NAME.seqs plus sequences that
reach the later stages -- local-mode homologs, their shuffles (the model's
composition without its order), background sequences carrying a short homolog
fragment, and i.i.d. draws from a homolog's composition; pipe_NAME.pres: the
reference's p7_bg_FilterScore for every sequence and the stage each one
reached, ``refgen pipe`` / ``refgen pipefile``; for the sampled models also
pipe_NAME.prof, the MSV part of the model in hmmsearch's local configuration,
and the composition hmmbuild would give the model). Sequences drawn from the
model's commonest residues, or a homolog fragment in model-composition
flanks, are what the bias filter rejects.
Run:  python tests/golden/make_golden.py [reference code dir]
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
from cudahmmsearch_gb300 import formats as F  # noqa: E402

REFGEN = os.path.join(ROOT, "oracle", "_ref", "refgen")
LCFG = 400
MODE_UNILOCAL = 3

# (name, M, seed, n_lognormal, lognormal lmax, n_homologs, n_saturation, repeat)
CASES = [
    ("m1_s1", 1, 1, 40, 400, 6, 2, 20),
    ("m2_s1", 2, 1, 40, 400, 6, 2, 20),
    ("m3_s5", 3, 5, 40, 400, 6, 2, 20),
    ("m16_s1", 16, 1, 40, 600, 6, 2, 20),
    ("m17_s2", 17, 2, 40, 600, 6, 2, 20),
    ("m33_s3", 33, 3, 40, 800, 6, 2, 20),
    ("m50_s1", 50, 1, 60, 1000, 8, 3, 20),
    ("m200_s1", 200, 1, 120, 5000, 10, 3, 20),      # the M=200, seed 1 profile of the 20,000-sequence workload
    ("m400_s1", 400, 1, 80, 3000, 8, 3, 20),        # the M=400, seed 1 profile of the 2,000,000-sequence workload
    ("m777_s3", 777, 3, 40, 2000, 6, 2, 8),
    ("m1500_s2", 1500, 2, 30, 2000, 6, 2, 5),
    ("m2400_s1", 2400, 1, 30, 2000, 6, 3, 5),       # the M=2400, seed 1 profile of the length-extremes workload
]


def run(*args):
    subprocess.check_call([REFGEN] + [str(a) for a in args])


def make_case(name, M, seed, n_ln, lmax, n_hom, n_sat, rep):
    prof = os.path.join(HERE, name + ".prof")
    seqs = os.path.join(HERE, name + ".seqs")
    res = os.path.join(HERE, name + ".res")
    tmp = os.path.join(HERE, "_tmp.seqs")
    run("profile", M, seed, LCFG, MODE_UNILOCAL, prof)
    parts = []
    for j, L in enumerate([1, 2, 3, 4, 10]):
        parts.append(F.synth_sequences(6, seed=1000 * seed + M + j, median=L, sigma=0.0, lmin=L, lmax=L))
    parts.append(F.synth_sequences(n_ln, seed=2000 * seed + M, lmax=lmax))
    rng = np.random.default_rng(3000 * seed + M)
    allcodes = [rng.integers(0, F.KP_AMINO, size=int(L), dtype=np.uint8) for L in (1, 5, 37, 250)]
    allx = [np.full(L, F.CODE_X, np.uint8) for L in (1, 40)]
    parts.append(F.SeqSet.from_list(allcodes + allx))
    run("emit", M, seed, 100, MODE_UNILOCAL, n_hom, 17 * seed + 1, 1, tmp)
    parts.append(F.read_seqs(tmp))
    run("emit", M, seed, 20, MODE_UNILOCAL, n_sat, 19 * seed + 2, rep, tmp)
    parts.append(F.read_seqs(tmp))
    os.remove(tmp)
    s = F.SeqSet.concat(parts)
    F.write_seqs(s, seqs)
    run("score", M, seed, LCFG, MODE_UNILOCAL, seqs, res)
    r = F.read_results(res)
    print(f"{name}: M={M} n={s.n} residues={s.total} erange={(r.status == 16).sum()} "
          f"pass={int(r.passed.sum())}")


# tutorial models: (name, index in tutorial/minifam)
TUT_MODELS = [("tut_globins4", 0), ("tut_fn3", 1), ("tut_pkinase", 2)]
TUT_SEQFILES = ["globins45.fa", "HBB_HUMAN", "7LESS_DROME"]


def make_tutorial(tut):
    minifam = os.path.join(tut, "minifam")
    tmp = os.path.join(HERE, "_tmp.seqs")
    common = []
    for f in TUT_SEQFILES:
        run("seqfile", os.path.join(tut, f), tmp)
        common.append(F.read_seqs(tmp))
    run("randseq", 60, 300, 7, tmp)
    common.append(F.read_seqs(tmp))
    for k, (name, idx) in enumerate(TUT_MODELS):
        prof = os.path.join(HERE, name + ".prof")
        seqs = os.path.join(HERE, name + ".seqs")
        res = os.path.join(HERE, name + ".res")
        run("hmmfile", minifam, idx, 0, prof)
        run("emitfile", minifam, idx, 30, 100 + k, tmp)
        hom = F.read_seqs(tmp)
        sat = F.SeqSet.from_list([np.tile(hom.seq(i), 20) for i in range(3)])   # saturation repeats
        s = F.SeqSet.concat(common + [hom, sat])
        F.write_seqs(s, seqs)
        run("scorefile", minifam, idx, seqs, res)
        r = F.read_results(res)
        print(f"{name}: M={F.read_profile(prof).M} n={s.n} residues={s.total} "
              f"erange={(r.status == 16).sum()} pass={int(r.passed.sum())}")
    os.remove(tmp)


# ViterbiFilter goldens (vit_NAME.vprof / .vres over NAME.seqs): the sampled
# cases in hmmsearch's local mode, and the tutorial models as hmmsearch
# configures them
VIT_SAMPLED = ["m1_s1", "m2_s1", "m16_s1", "m17_s2", "m33_s3", "m50_s1", "m200_s1", "m400_s1", "m777_s3",
               "m1500_s2", "m2400_s1"]


def make_vit(tut):
    for name in VIT_SAMPLED:
        M, seed = name[1:].split("_s")
        run("vit", M, seed, os.path.join(HERE, "vit_" + name + ".vprof"), os.path.join(HERE, "vit_" + name + ".vres"),
            os.path.join(HERE, name + ".seqs"))
    for name, idx in TUT_MODELS:
        run("vitfile", os.path.join(tut, "minifam"), idx, os.path.join(HERE, "vit_" + name + ".vprof"),
            os.path.join(HERE, "vit_" + name + ".vres"), os.path.join(HERE, name + ".seqs"))
    make_vit_widths()
    print("vit goldens:", len(VIT_SAMPLED) + len(TUT_MODELS) + len(VIT_WIDTHS))


# models for the GPU kernel's row forms: M=1100 (40 nodes per lane, two per
# register), M=4000 (the shared-memory row), and the widest model of several
# register-row widths (5, 9, 13, 20, 28 nodes per lane); each over background
# sequences, homologs and saturation repeats
VIT_WIDTHS = [("vitmid_m1100_s4", 1100, 4), ("vitwide_m4000_s7", 4000, 7), ("vitw5_m157_s5", 157, 5),
              ("vitw9_m285_s9", 285, 9), ("vitw13_m413_s13", 413, 13), ("vitw20_m637_s20", 637, 20),
              ("vitw28_m893_s28", 893, 28)]


def make_vit_widths(only=None):
    tmp = os.path.join(HERE, "_tmp.seqs")
    for name, M, seed in VIT_WIDTHS:
        if only is not None and name not in only:
            continue
        parts = [F.synth_sequences(24, seed=M + 1, lmax=3000)]
        run("emit", M, seed, 100, MODE_LOCAL, 6, M + 2, 1, tmp)
        parts.append(F.read_seqs(tmp))
        run("emit", M, seed, 20, MODE_LOCAL, 2, M + 3, 4, tmp)
        parts.append(F.read_seqs(tmp))
        F.write_seqs(F.SeqSet.concat(parts), os.path.join(HERE, name + ".seqs"))
        run("vit", M, seed, os.path.join(HERE, "vit_" + name + ".vprof"), os.path.join(HERE, "vit_" + name + ".vres"),
            os.path.join(HERE, name + ".seqs"))
    if os.path.exists(tmp):
        os.remove(tmp)


# pipeline goldens: sampled models in hmmsearch's local mode, and the tutorial models
PIPE_SAMPLED = ["m50_s1", "m200_s1", "m400_s1", "m777_s3"]
MODE_LOCAL = 1


def pipe_extras(hom, seed, compo):
    """Sequences for the later filter stages, built from homologs hom and the
    model composition compo."""
    rng = np.random.default_rng(seed)
    out = [hom.seq(i) for i in range(hom.n)]
    for i in range(hom.n):                                       # shuffles: composition only
        h = hom.seq(i)
        out.append(rng.permutation(np.tile(h, 1 + (i % 3))))
    bg = F.synth_sequences(hom.n, seed=seed + 1, lmax=3000)
    for i in range(hom.n):                                       # a short homolog fragment in background
        h, b = hom.seq(i), bg.seq(i)
        w = int(rng.integers(8, 48))
        a = int(rng.integers(0, max(1, len(h) - w)))
        c = int(rng.integers(0, len(b) + 1))
        out.append(np.concatenate([b[:c], h[a:a + w], b[c:]]))
    for i in range(hom.n // 2):                                  # i.i.d. draws from a homolog's composition
        h = hom.seq(i)
        out.append(rng.choice(h, size=int(rng.integers(50, 1500))).astype(np.uint8))
    top = np.argsort(-compo)
    for k in (2, 3, 5):                                          # the model's k commonest residues: bias-filter rejects
        pr = compo[top[:k]] / compo[top[:k]].sum()
        for _ in range(8):
            out.append(rng.choice(top[:k], size=int(rng.integers(100, 2000)), p=pr).astype(np.uint8))
    pr = compo / compo.sum()
    for i in range(hom.n // 2):                                  # a homolog fragment in model-composition flanks
        h = hom.seq(i)
        f = rng.choice(20, size=int(rng.integers(200, 1500)), p=pr).astype(np.uint8)
        c = int(rng.integers(0, len(f)))
        w = int(rng.integers(10, 30))
        a = int(rng.integers(0, max(1, len(h) - w)))
        out.append(np.concatenate([f[:c], h[a:a + w], f[c:]]))
    return F.SeqSet.from_list(out)


def make_pipe(tut):
    tmp = os.path.join(HERE, "_tmp.seqs")
    jobs = []
    for k, name in enumerate(PIPE_SAMPLED):
        M, seed = name[1:].split("_s")
        run("emit", M, seed, 100, MODE_LOCAL, 24, 500 + k, 1, tmp)
        jobs.append((name, ("pipe", M, seed), F.read_seqs(tmp)))
    for k, (name, idx) in enumerate(TUT_MODELS):
        run("emitfile", os.path.join(tut, "minifam"), idx, 24, 600 + k, tmp)
        jobs.append((name, ("pipefile", os.path.join(tut, "minifam"), idx), F.read_seqs(tmp)))
    os.remove(tmp)
    for k, (name, cmd, hom) in enumerate(jobs):
        base = os.path.join(HERE, name + ".seqs")
        seqs = os.path.join(HERE, "pipe_" + name + ".seqs")
        pres = os.path.join(HERE, "pipe_" + name + ".pres")
        prof = [os.path.join(HERE, "pipe_" + name + ".prof")] if cmd[0] == "pipe" else []
        run(*cmd, pres, base, *prof)                             # first pass: the model's composition
        s = F.SeqSet.concat([F.read_seqs(base), pipe_extras(hom, 700 + 10 * k, F.read_pipe(pres).compo)])
        F.write_seqs(s, seqs)
        run(*cmd, pres, seqs, *prof)
        r = F.read_pipe(pres)
        print(f"pipe_{name}: n={s.n} stages={np.bincount(r.stage[r.stage < 4], minlength=4).tolist()} "
              f"vit_run={int(np.isfinite(r.vfsc).sum())}")


def main():
    if not os.path.exists(REFGEN):
        sys.exit("oracle/_ref/refgen missing: make -C oracle/ref REF=<reference>/code")
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("MSVGB_REFERENCE_CODE")
    if not ref or not os.path.isdir(ref):
        sys.exit("usage: make_golden.py <reference>/code  (or set MSVGB_REFERENCE_CODE)")
    for c in CASES:
        make_case(*c)
    make_tutorial(os.path.join(ref, "tutorial"))
    make_vit(os.path.join(ref, "tutorial"))
    make_pipe(os.path.join(ref, "tutorial"))


if __name__ == "__main__":
    main()
