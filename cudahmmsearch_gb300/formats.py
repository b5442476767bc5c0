"""On-disk and in-memory formats for MSV profiles, sequence sets and results.

The profile record is the MSV part of HMMER's ``P7_OPROFILE``
(src/impl_sse/impl_sse.h:77-87): the striped uint8 match-cost table ``rbv``
laid out ``[Kp][Q][16]`` where byte ``z`` of vector ``q`` holds node
``k = q + 1 + z*Q`` and padding nodes hold 255 (src/impl_sse/p7_oprofile.c:619-635),
plus the scalar costs ``tbm_b, tec_b, base_b, bias_b``, ``scale_b`` and the
E-value parameters ``evparam[p7_MMU], evparam[p7_MLAMBDA]``.

Sequences are Easel digital codes (easel/esl_alphabet.c:275, amino alphabet
"ACDEFGHIKLMNPQRSTVWY-BJZOUX*~", K=20, Kp=29, X=26), concatenated without the
255 sentinels, with an int64 offset array of n+1 entries.

File formats (little-endian; written by oracle/ref/refgen.c and by this module):
  profile "MSVPROF1": int32 M, Q, Kp, Lcfg; uint8 tbm, tec, tjb, base, bias, pad[3];
                      float32 scale; float64 mmu, mlambda; uint8 rbv[Kp*Q*16]
  seqs    "MSVSEQS1": int64 n, total; int64 off[n+1]; uint8 codes[total]
  result  "MSVRES01": int64 n; int32 status[n]; float32 sc[n]; float64 nullsc[n];
                      float64 P[n]; uint8 pass[n]
"""
from __future__ import annotations

import dataclasses
import struct

import numpy as np

KP_AMINO = 29
K_AMINO = 20
CODE_X = 26

# Easel status codes (easel/easel.h:95-114)
eslOK = 0
eslEINVAL = 11
eslERANGE = 16
eslENORESULT = 19

# Amino background composition used by HMMER's null model, Swiss-Prot 50.8
# (src/hmmer.c:163-186, p7_AminoFrequencies), A..Y in Easel code order.
AMINO_BG = np.array([
    0.0787945, 0.0151600, 0.0535222, 0.0668298, 0.0397062, 0.0695071, 0.0229198,
    0.0590092, 0.0594422, 0.0963728, 0.0237718, 0.0414386, 0.0482904, 0.0395639,
    0.0540978, 0.0683364, 0.0540687, 0.0673417, 0.0114135, 0.0304133], dtype=np.float32)


def nqb(M: int) -> int:
    """p7O_NQB(M) = max(2, ceil(M/16)) (src/impl_sse/impl_sse.h:26)."""
    return max(2, (M - 1) // 16 + 1)


@dataclasses.dataclass
class Profile:
    M: int
    rbv: np.ndarray          # uint8 [Kp, Q, 16]
    tbm_b: int
    tec_b: int
    base_b: int
    bias_b: int
    scale_b: float           # float32 value
    mmu: float
    mlambda: float
    tjb_cfg: int = 0         # tjb_b at the configuration length (per-sequence value is recomputed)
    Lcfg: int = 0

    @property
    def Q(self) -> int:
        return nqb(self.M)

    @property
    def Kp(self) -> int:
        return int(self.rbv.shape[0])

    def node_costs(self) -> np.ndarray:
        """rbv re-indexed by node: uint8 [Kp, M] with column k-1 = node k."""
        Q = self.Q
        k = np.arange(self.M)
        return self.rbv[:, k % Q, k // Q]


def profile_from_node_costs(costs: np.ndarray, *, tbm_b: int, tec_b: int, base_b: int,
                            bias_b: int, scale_b: float, mmu: float, mlambda: float) -> Profile:
    """Stripe a [Kp, M] node-ordered cost table into the P7_OPROFILE layout."""
    Kp, M = costs.shape
    Q = nqb(M)
    rbv = np.full((Kp, Q, 16), 255, dtype=np.uint8)
    k = np.arange(M)
    rbv[:, k % Q, k // Q] = costs
    return Profile(M=M, rbv=rbv, tbm_b=tbm_b, tec_b=tec_b, base_b=base_b, bias_b=bias_b,
                   scale_b=float(np.float32(scale_b)), mmu=mmu, mlambda=mlambda)


def read_profile(path) -> Profile:
    b = open(path, "rb").read()
    if b[:8] != b"MSVPROF1":
        raise ValueError(f"{path}: not an MSVPROF1 file")
    M, Q, Kp, Lcfg = struct.unpack_from("<4i", b, 8)
    tbm, tec, tjb, base, bias = struct.unpack_from("<5B", b, 24)
    (scale,) = struct.unpack_from("<f", b, 32)
    mmu, mlambda = struct.unpack_from("<2d", b, 36)
    rbv = np.frombuffer(b, np.uint8, Kp * Q * 16, 52).reshape(Kp, Q, 16).copy()
    if Q != nqb(M):
        raise ValueError(f"{path}: Q={Q} but p7O_NQB({M})={nqb(M)}")
    return Profile(M=M, rbv=rbv, tbm_b=tbm, tec_b=tec, base_b=base, bias_b=bias, scale_b=scale,
                   mmu=mmu, mlambda=mlambda, tjb_cfg=tjb, Lcfg=Lcfg)


def write_profile(p: Profile, path) -> None:
    with open(path, "wb") as f:
        f.write(b"MSVPROF1")
        f.write(struct.pack("<4i", p.M, p.Q, p.Kp, p.Lcfg))
        f.write(struct.pack("<8B", p.tbm_b, p.tec_b, p.tjb_cfg, p.base_b, p.bias_b, 0, 0, 0))
        f.write(struct.pack("<f", p.scale_b))
        f.write(struct.pack("<2d", p.mmu, p.mlambda))
        f.write(np.ascontiguousarray(p.rbv, dtype=np.uint8).tobytes())


@dataclasses.dataclass
class SeqSet:
    codes: np.ndarray        # uint8 [total]
    off: np.ndarray          # int64 [n+1]

    @property
    def n(self) -> int:
        return int(self.off.shape[0] - 1)

    @property
    def lengths(self) -> np.ndarray:
        return np.diff(self.off)

    @property
    def total(self) -> int:
        return int(self.off[-1])

    def seq(self, i: int) -> np.ndarray:
        return self.codes[self.off[i]:self.off[i + 1]]

    def subset(self, idx) -> "SeqSet":
        idx = np.asarray(idx, dtype=np.int64)
        lens = self.lengths[idx]
        off = np.zeros(len(idx) + 1, np.int64)
        np.cumsum(lens, out=off[1:])
        codes = np.empty(int(off[-1]), np.uint8)
        for j, i in enumerate(idx):
            codes[off[j]:off[j + 1]] = self.codes[self.off[i]:self.off[i + 1]]
        return SeqSet(codes, off)

    @staticmethod
    def concat(sets) -> "SeqSet":
        sets = list(sets)
        codes = np.concatenate([s.codes for s in sets]) if sets else np.zeros(0, np.uint8)
        lens = np.concatenate([s.lengths for s in sets]) if sets else np.zeros(0, np.int64)
        off = np.zeros(len(lens) + 1, np.int64)
        np.cumsum(lens, out=off[1:])
        return SeqSet(codes.astype(np.uint8), off)

    @staticmethod
    def from_list(seqs) -> "SeqSet":
        seqs = [np.asarray(s, dtype=np.uint8) for s in seqs]
        lens = np.array([len(s) for s in seqs], dtype=np.int64)
        off = np.zeros(len(seqs) + 1, np.int64)
        np.cumsum(lens, out=off[1:])
        codes = np.concatenate(seqs) if seqs else np.zeros(0, np.uint8)
        return SeqSet(codes.astype(np.uint8), off)


def read_seqs(path) -> SeqSet:
    b = open(path, "rb").read()
    if b[:8] != b"MSVSEQS1":
        raise ValueError(f"{path}: not an MSVSEQS1 file")
    n, total = struct.unpack_from("<2q", b, 8)
    off = np.frombuffer(b, np.int64, n + 1, 24).copy()
    codes = np.frombuffer(b, np.uint8, total, 24 + 8 * (n + 1)).copy()
    return SeqSet(codes, off)


def write_seqs(s: SeqSet, path) -> None:
    with open(path, "wb") as f:
        f.write(b"MSVSEQS1")
        f.write(struct.pack("<2q", s.n, s.total))
        f.write(np.ascontiguousarray(s.off, dtype=np.int64).tobytes())
        f.write(np.ascontiguousarray(s.codes, dtype=np.uint8).tobytes())


@dataclasses.dataclass
class Results:
    status: np.ndarray       # int32
    sc: np.ndarray           # float32
    nullsc: np.ndarray       # float64 (float32 values)
    P: np.ndarray            # float64
    passed: np.ndarray       # uint8


def read_results(path) -> Results:
    b = open(path, "rb").read()
    if b[:8] != b"MSVRES01":
        raise ValueError(f"{path}: not an MSVRES01 file")
    (n,) = struct.unpack_from("<q", b, 8)
    o = 16
    st = np.frombuffer(b, np.int32, n, o).copy(); o += 4 * n
    sc = np.frombuffer(b, np.float32, n, o).copy(); o += 4 * n
    ns = np.frombuffer(b, np.float64, n, o).copy(); o += 8 * n
    P = np.frombuffer(b, np.float64, n, o).copy(); o += 8 * n
    ps = np.frombuffer(b, np.uint8, n, o).copy()
    return Results(st, sc, ns, P, ps)


@dataclasses.dataclass
class VProfile:
    """The ViterbiFilter part of a P7_OPROFILE (src/impl_sse/impl_sse.h:88-96),
    striped as the reference stores it: Q8 = max(2, ceil(M/8)); twv
    [8*Q8, 8] int16 (per vector q the 7 vectors BM MM IM DM MD MI II, then the
    Q8 DD vectors), rwv [Kp, Q8, 8] int16; element z of vector q is node
    q+1+z*Q8. xw [4, 2] int16 (E N J C x MOVE LOOP) as configured; the
    N/J/C MOVE costs are recomputed per target length."""
    M: int
    twv: np.ndarray
    rwv: np.ndarray
    xw: np.ndarray
    scale_w: float
    nj: float
    base_w: int
    ddbound_w: int
    vmu: float = 0.0
    vlambda: float = 0.0

    @property
    def Q8(self) -> int:
        return max(2, (self.M - 1) // 8 + 1)

    @property
    def Kp(self) -> int:
        return int(self.rwv.shape[0])


def read_vprofile(path) -> VProfile:
    """VITPROF1: int32 M, Q8, Kp; float scale_w, nj; int16 base_w, ddbound_w;
    int16 xw[4][2]; float vmu, vlambda; int16 twv[8*Q8][8]; int16 rwv[Kp][Q8][8]."""
    b = open(path, "rb").read()
    if b[:8] != b"VITPROF1":
        raise ValueError(f"{path}: not a VITPROF1 file")
    M, Q8, Kp = struct.unpack_from("<3i", b, 8)
    scale_w, nj = struct.unpack_from("<2f", b, 20)
    base_w, ddbound_w = struct.unpack_from("<2h", b, 28)
    xw = np.frombuffer(b, np.int16, 8, 32).reshape(4, 2).copy()
    vmu, vlambda = struct.unpack_from("<2f", b, 48)
    o = 56
    twv = np.frombuffer(b, np.int16, 8 * Q8 * 8, o).reshape(8 * Q8, 8).copy(); o += 8 * Q8 * 16
    rwv = np.frombuffer(b, np.int16, Kp * Q8 * 8, o).reshape(Kp, Q8, 8).copy()
    return VProfile(M=M, twv=twv, rwv=rwv, xw=xw, scale_w=scale_w, nj=nj, base_w=base_w, ddbound_w=ddbound_w,
                    vmu=vmu, vlambda=vlambda)


def read_vresults(path):
    """VITRES01: int64 n; int32 status[n] (-1: empty); float sc[n]."""
    b = open(path, "rb").read()
    if b[:8] != b"VITRES01":
        raise ValueError(f"{path}: not a VITRES01 file")
    (n,) = struct.unpack_from("<q", b, 8)
    st = np.frombuffer(b, np.int32, n, 16).copy()
    sc = np.frombuffer(b, np.float32, n, 16 + 4 * n).copy()
    return st, sc


@dataclasses.dataclass
class PipeResults:
    """The filter stages of p7_Pipeline on a sequence set (PIPERES1)."""
    M: int
    compo: np.ndarray          # float32[20], the model composition (P7_OPROFILE compo)
    mmu: float
    mlambda: float
    vmu: float
    vlambda: float
    F1: float
    F2: float
    nullsc: np.ndarray         # float32[n]
    usc: np.ndarray            # float32[n], MSV score
    fsc: np.ndarray            # float32[n], bias-filter score (every sequence)
    vfsc: np.ndarray           # float32[n], ViterbiFilter score (NaN where not run)
    stage: np.ndarray          # uint8[n]: 0 rejected by MSV, 1 by the bias filter, 2 by Viterbi, 3 passed, 255 empty


def read_pipe(path) -> PipeResults:
    """PIPERES1: int32 M; float compo[20]; float mmu, mlambda, vmu, vlambda;
    double F1, F2; int64 n; float nullsc[n], usc[n], fsc[n], vfsc[n]; uint8 stage[n]."""
    b = open(path, "rb").read()
    if b[:8] != b"PIPERES1":
        raise ValueError(f"{path}: not a PIPERES1 file")
    M = int(np.frombuffer(b, np.int32, 1, 8)[0])
    compo = np.frombuffer(b, np.float32, 20, 12).copy()
    ev = np.frombuffer(b, np.float32, 4, 92)
    F = np.frombuffer(b, np.float64, 2, 108)
    n = int(np.frombuffer(b, np.int64, 1, 124)[0])
    o = 132
    arr = [np.frombuffer(b, np.float32, n, o + 4 * n * k).copy() for k in range(4)]
    stage = np.frombuffer(b, np.uint8, n, o + 16 * n).copy()
    return PipeResults(M, compo, float(ev[0]), float(ev[1]), float(ev[2]), float(ev[3]), float(F[0]), float(F[1]),
                       arr[0], arr[1], arr[2], arr[3], stage)


def synth_sequences(n: int, *, seed: int, median: float = 300.0, sigma: float = 0.7,
                    lmin: int = 10, lmax: int = 5000, x_frac: float = 0.005,
                    uniform_frac: float = 0.0, uniform_range=(5000, 35000)) -> SeqSet:
    """Synthetic protein database: residues i.i.d. from the HMMER amino
    background with a fraction ``x_frac`` replaced by X (code 26), lengths
    lognormal(ln median, sigma) clipped to [lmin, lmax]; optionally a fraction
    of lengths uniform in ``uniform_range``. Residues are drawn through a
    65536-entry inverse-CDF table in chunks, so hundreds of millions of
    residues take seconds."""
    rng = np.random.default_rng(seed)
    lens = np.exp(rng.normal(np.log(median), sigma, size=n))
    lens = np.clip(np.rint(lens), lmin, lmax).astype(np.int64)
    if uniform_frac > 0:
        m = rng.random(n) < uniform_frac
        lens[m] = rng.integers(uniform_range[0], uniform_range[1] + 1, size=int(m.sum()))
    off = np.zeros(n + 1, np.int64)
    np.cumsum(lens, out=off[1:])
    total = int(off[-1])
    p = AMINO_BG.astype(np.float64) / AMINO_BG.astype(np.float64).sum() * (1.0 - x_frac)
    cdf = np.cumsum(np.concatenate([p, [x_frac]]))
    lut = np.searchsorted(cdf, (np.arange(65536) + 0.5) / 65536.0, side="right")
    lut = np.minimum(lut, K_AMINO).astype(np.uint8)
    lut[lut == K_AMINO] = CODE_X
    codes = np.empty(total, np.uint8)
    step = 1 << 26
    for a in range(0, total, step):
        b = min(total, a + step)
        codes[a:b] = lut[rng.integers(0, 65536, size=b - a, dtype=np.uint16)]
    return SeqSet(codes, off)


def emission_probs(p: Profile) -> np.ndarray:
    """Approximate match emission probabilities per node, float64 [M, 20]:
    e_k(x) proportional to f(x) * exp(msc(k,x)) with msc recovered from the
    quantised cost, msc ~ (bias - rbv) / scale (inverse of biased_byteify,
    src/impl_sse/p7_oprofile.c:495-503)."""
    costs = p.node_costs()[:K_AMINO].astype(np.float64).T          # [M, 20]
    msc = (p.bias_b - costs) / p.scale_b
    e = AMINO_BG[None, :].astype(np.float64) * np.exp(msc)
    return e / e.sum(axis=1, keepdims=True)


def emit_homologs(p: Profile, n: int, *, seed: int, flank_median: float = 150.0,
                  repeat: int = 1, lmax: int = 35000) -> SeqSet:
    """Synthetic homologs of a profile: a local, mostly ungapped walk through
    the model's match states (random start node and length, ~1% insert and
    ~1% delete events) emitting from emission_probs(), between background
    flanks. With repeat > 1 the emitted core is repeated (drives scores to
    overflow)."""
    rng = np.random.default_rng(seed)
    e = emission_probs(p)
    cdf = np.cumsum(e, axis=1)
    cdf /= cdf[:, -1:]
    bg = np.cumsum(AMINO_BG.astype(np.float64))
    bg /= bg[-1]
    out = []
    for _ in range(n):
        k0 = int(rng.integers(0, max(1, p.M // 3)))
        k1 = int(rng.integers(min(p.M, k0 + max(1, p.M // 2)), p.M + 1))
        ks = np.arange(k0, max(k1, k0 + 1))
        ks = ks[rng.random(len(ks)) >= 0.01]                   # deletions
        core = (cdf[ks] < rng.random(len(ks))[:, None]).sum(axis=1)
        ins = rng.random(len(core)) < 0.01                      # insertions after a node
        if ins.any():
            extra = np.searchsorted(bg, rng.random(int(ins.sum())), side="right")
            core = np.insert(core, np.nonzero(ins)[0] + 1, extra)
        core = np.minimum(core, K_AMINO - 1).astype(np.uint8)
        if repeat > 1:
            core = np.tile(core, repeat)
        fl = rng.exponential(flank_median, size=2).astype(np.int64)
        left = np.minimum(np.searchsorted(bg, rng.random(fl[0]), side="right"), K_AMINO - 1)
        right = np.minimum(np.searchsorted(bg, rng.random(fl[1]), side="right"), K_AMINO - 1)
        seq = np.concatenate([left.astype(np.uint8), core, right.astype(np.uint8)])[:lmax]
        out.append(seq if len(seq) else core[:1])
    return SeqSet.from_list(out)
