"""ctypes bindings for the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads oracle/libmsvoracle.so, the scalar C restatement of HMMER 3.1b1's
p7_MSVFilter (src/impl_sse/msvfilter.c:77-213, with the SSV fast path of
src/impl_sse/ssvfilter.c:1364-1413), of the MSV stage of p7_Pipeline
(src/p7_pipeline.c:662-677), of p7_ViterbiFilter
(src/impl_sse/vitfilter.c:84-250), of the bias filter p7_bg_FilterScore
(src/p7_bg.c:473) and of the filter-stage gates of p7_Pipeline
(src/p7_pipeline.c:666-705). Only tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py may import this module.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmsvoracle.so")


def build(force: bool = False) -> str:
    """Compiles the scalar oracle (msv_oracle.c) and the vectorized port used
    as the timed CPU baseline (msv_port.c) into one library."""
    srcs = [os.path.join(HERE, "msv_oracle.c"), os.path.join(HERE, "msv_port.c"), os.path.join(HERE, "vit_oracle.c"),
            os.path.join(HERE, "bias_oracle.c")]
    hdrs = [os.path.join(HERE, "msv_oracle.h"), os.path.join(HERE, "vit_oracle.h"), os.path.join(HERE, "bias_oracle.h")]
    if force or not os.path.exists(LIB_PATH) or any(os.path.getmtime(LIB_PATH) < os.path.getmtime(f)
                                                    for f in srcs + hdrs):
        subprocess.check_call(["cc", "-O3", "-std=gnu99", "-ffp-contract=off", "-fPIC", "-shared",
                               "-pthread"] + srcs + ["-o", LIB_PATH, "-lm"])
    return LIB_PATH


class _Prof(ctypes.Structure):
    _fields_ = [("M", ctypes.c_int), ("Q", ctypes.c_int), ("Kp", ctypes.c_int),
                ("rbv", ctypes.c_void_p),
                ("tbm_b", ctypes.c_uint8), ("tec_b", ctypes.c_uint8),
                ("base_b", ctypes.c_uint8), ("bias_b", ctypes.c_uint8),
                ("scale_b", ctypes.c_float), ("mmu", ctypes.c_double), ("mlambda", ctypes.c_double)]


class _VProf(ctypes.Structure):
    _fields_ = [("M", ctypes.c_int), ("Q8", ctypes.c_int), ("Kp", ctypes.c_int),
                ("scale_w", ctypes.c_float), ("nj", ctypes.c_float),
                ("base_w", ctypes.c_int16), ("ddbound_w", ctypes.c_int16),
                ("xw", ctypes.c_int16 * 8), ("twv", ctypes.c_void_p), ("rwv", ctypes.c_void_p)]


class _PipeRes(ctypes.Structure):
    _fields_ = [("usc", ctypes.c_float), ("nullsc", ctypes.c_float), ("filtersc", ctypes.c_float),
                ("vfsc", ctypes.c_float), ("stage", ctypes.c_int)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        _lib.orc_tjb_b.restype = ctypes.c_uint8
        _lib.orc_tjb_b.argtypes = [ctypes.c_float, ctypes.c_int]
        _lib.orc_msv_filter.restype = ctypes.c_int
        _lib.orc_msv_full.restype = ctypes.c_int
        _lib.orc_score_from_xj.restype = ctypes.c_float
        _lib.orc_score_from_xj.argtypes = [ctypes.c_uint8, ctypes.c_uint8, ctypes.c_uint8, ctypes.c_float]
        _lib.orc_f1_pass.restype = ctypes.c_int
        _lib.orc_f1_pass.argtypes = [ctypes.c_float, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_double, ctypes.POINTER(ctypes.c_float),
                                     ctypes.POINTER(ctypes.c_double)]
        _lib.port_msv_batch.restype = ctypes.c_int
        _lib.port_msv_batch.argtypes = [ctypes.POINTER(_Prof), ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_int64, ctypes.c_double, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]
        _lib.orc_vit_filter.restype = ctypes.c_int
        _lib.orc_vit_filter.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(_VProf),
                                        ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int)]
        _lib.orc_bias_filter.restype = ctypes.c_float
        _lib.orc_bias_filter.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_int]
        _lib.orc_gumbel_P.restype = ctypes.c_double
        _lib.orc_gumbel_P.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_double, ctypes.c_double]
        _lib.orc_pipe_stages.restype = None
        _lib.orc_pipe_stages.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_float, ctypes.c_void_p, ctypes.c_int,
                                         ctypes.POINTER(_VProf), ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.POINTER(_PipeRes)]
        _lib.orc_msv_batch.restype = ctypes.c_int
        _lib.orc_msv_batch.argtypes = [ctypes.POINTER(_Prof), ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_double, ctypes.c_int,
                                       ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                       ctypes.c_void_p, ctypes.c_void_p]
    return _lib


def _prof(p):
    rbv = np.ascontiguousarray(p.rbv, dtype=np.uint8)
    s = _Prof(p.M, p.Q, p.Kp, rbv.ctypes.data, p.tbm_b, p.tec_b, p.base_b, p.bias_b,
              p.scale_b, p.mmu, p.mlambda)
    return s, rbv


def tjb_b(scale_b: float, L: int) -> int:
    return int(lib().orc_tjb_b(scale_b, L))


def score_from_xj(xj: int, tjb: int, base_b: int, scale_b: float) -> float:
    return float(lib().orc_score_from_xj(xj, tjb, base_b, scale_b))


def f1_pass(usc: float, L: int, mmu: float, mlambda: float, F1: float = 0.02):
    ns = ctypes.c_float()
    P = ctypes.c_double()
    r = lib().orc_f1_pass(usc, L, mmu, mlambda, F1, ctypes.byref(ns), ctypes.byref(P))
    return bool(r), ns.value, P.value


def msv_filter(p, dsq_codes, *, full_only: bool = False):
    """One p7_MSVFilter call on a single sequence (codes without sentinels).
    Returns (status, xj, sc, path)."""
    L = len(dsq_codes)
    dsq = np.empty(L + 2, np.uint8)
    dsq[0] = dsq[-1] = 255
    dsq[1:L + 1] = dsq_codes
    s, keep = _prof(p)
    xj = ctypes.c_uint8()
    sc = ctypes.c_float()
    path = ctypes.c_int(1)
    tjb = tjb_b(p.scale_b, L)
    if full_only:
        st = lib().orc_msv_full(dsq.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(L), ctypes.byref(s),
                                ctypes.c_uint8(tjb), ctypes.byref(xj), ctypes.byref(sc))
    else:
        st = lib().orc_msv_filter(dsq.ctypes.data_as(ctypes.c_void_p), ctypes.c_int(L), ctypes.byref(s),
                                  ctypes.c_uint8(tjb), ctypes.byref(xj), ctypes.byref(sc),
                                  ctypes.byref(path))
    return int(st), int(xj.value), float(sc.value), int(path.value)


def msv_batch(p, seqs, *, F1: float = 0.02, nthreads: int = 0):
    """Oracle over a SeqSet. Returns dict of numpy arrays:
    status (int32, -1 = empty sequence), xj (uint8), sc (float32), pass (uint8), path (uint8)."""
    n = seqs.n
    out = {"status": np.zeros(n, np.int32), "xj": np.zeros(n, np.uint8), "sc": np.zeros(n, np.float32),
           "pass": np.zeros(n, np.uint8), "path": np.zeros(n, np.uint8)}
    s, keep = _prof(p)
    codes = np.ascontiguousarray(seqs.codes, dtype=np.uint8)
    off = np.ascontiguousarray(seqs.off, dtype=np.int64)
    if codes.size == 0:
        codes = np.zeros(1, np.uint8)
    lib().orc_msv_batch(ctypes.byref(s), codes.ctypes.data, off.ctypes.data, n, F1, nthreads,
                        out["status"].ctypes.data, out["xj"].ctypes.data, out["sc"].ctypes.data,
                        out["pass"].ctypes.data, out["path"].ctypes.data)
    return out


def port_batch(p, seqs, *, F1: float = 0.02, nthreads: int = 0):
    """The vectorized port of the reference's SSE2 MSV (16 uint8 lanes; NEON on
    aarch64) over a SeqSet: status, xj, sc, pass as msv_batch. Returns
    (outputs, threads used)."""
    n = seqs.n
    out = {"status": np.zeros(n, np.int32), "xj": np.zeros(n, np.uint8), "sc": np.zeros(n, np.float32),
           "pass": np.zeros(n, np.uint8)}
    s, keep = _prof(p)
    codes = np.ascontiguousarray(seqs.codes, dtype=np.uint8)
    off = np.ascontiguousarray(seqs.off, dtype=np.int64)
    if codes.size == 0:
        codes = np.zeros(1, np.uint8)
    used = lib().port_msv_batch(ctypes.byref(s), codes.ctypes.data, off.ctypes.data, n, F1, nthreads,
                                out["status"].ctypes.data, out["xj"].ctypes.data, out["sc"].ctypes.data,
                                out["pass"].ctypes.data)
    return out, used


def _vprof(vp):
    twv = np.ascontiguousarray(vp.twv, dtype=np.int16)
    rwv = np.ascontiguousarray(vp.rwv, dtype=np.int16)
    xw = (ctypes.c_int16 * 8)(*[int(v) for v in np.asarray(vp.xw).reshape(-1)])
    s = _VProf(vp.M, vp.Q8, vp.Kp, vp.scale_w, vp.nj, vp.base_w, vp.ddbound_w, xw,
               twv.ctypes.data, rwv.ctypes.data)
    return s, (twv, rwv)


def vit_filter(vp, dsq_codes):
    """p7_ViterbiFilter on one sequence (codes without sentinels). Returns (status, sc, xC)."""
    L = len(dsq_codes)
    dsq = np.empty(L + 2, np.uint8)
    dsq[0] = dsq[-1] = 255
    dsq[1:L + 1] = dsq_codes
    s, keep = _vprof(vp)
    sc = ctypes.c_float()
    xc = ctypes.c_int()
    st = lib().orc_vit_filter(dsq.ctypes.data, L, ctypes.byref(s), ctypes.byref(sc), ctypes.byref(xc))
    return int(st), float(sc.value), int(xc.value)


def vit_batch(vp, seqs):
    """vit_filter over a SeqSet: status (int32, -1 for empty), sc (float32), xc (int32)."""
    st = np.full(seqs.n, -1, np.int32)
    sc = np.zeros(seqs.n, np.float32)
    xc = np.zeros(seqs.n, np.int32)
    for i in range(seqs.n):
        if seqs.lengths[i] == 0:
            continue
        st[i], sc[i], xc[i] = vit_filter(vp, seqs.seq(i))
    return {"status": st, "sc": sc, "xc": xc}


def _dsq(codes):
    L = len(codes)
    dsq = np.empty(L + 2, np.uint8)
    dsq[0] = dsq[-1] = 255
    dsq[1:L + 1] = codes
    return dsq


def bias_filter(compo, M: int, dsq_codes) -> float:
    """p7_bg_FilterScore of one sequence with the filter HMM of the model
    composition compo[20] and length M."""
    c = np.ascontiguousarray(compo, dtype=np.float32)
    dsq = _dsq(dsq_codes)
    return float(lib().orc_bias_filter(c.ctypes.data, M, dsq.ctypes.data, len(dsq_codes)))


def bias_batch(compo, M: int, seqs):
    """bias_filter over a SeqSet (0 for empty sequences)."""
    out = np.zeros(seqs.n, np.float32)
    for i in range(seqs.n):
        if seqs.lengths[i]:
            out[i] = bias_filter(compo, M, seqs.seq(i))
    return out


def gumbel_P(sc: float, base: float, mu: float, lam: float) -> float:
    return float(lib().orc_gumbel_P(sc, base, mu, lam))


def pipe_batch(vp, seqs, usc, compo, *, mmu, mlambda, vmu, vlambda, F1=0.02, F2=1e-3, do_bias=True):
    """The filter stages of p7_Pipeline after the MSV score usc[i] of every
    sequence: dict of stage (uint8: 0 MSV, 1 bias, 2 Viterbi rejected, 3 passed,
    255 empty), nullsc, filtersc, vfsc (NaN where Viterbi did not run)."""
    s, keep = _vprof(vp)
    c = np.ascontiguousarray(compo, dtype=np.float32)
    out = {k: np.zeros(seqs.n, np.float32) for k in ("nullsc", "filtersc", "vfsc")}
    out["stage"] = np.zeros(seqs.n, np.uint8)
    r = _PipeRes()
    for i in range(seqs.n):
        dsq = _dsq(seqs.seq(i))
        lib().orc_pipe_stages(dsq.ctypes.data, int(seqs.lengths[i]), float(usc[i]), c.ctypes.data, int(do_bias),
                              ctypes.byref(s), mmu, mlambda, vmu, vlambda, F1, F2, ctypes.byref(r))
        out["stage"][i] = r.stage
        out["nullsc"][i], out["filtersc"][i], out["vfsc"][i] = r.nullsc, r.filtersc, r.vfsc
    return out
