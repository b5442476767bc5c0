"""Python mirror of the reference's MSV interface over the C ABI (include/msvgb.h).

The names follow HMMER's: ``MSVFilter(dsq, L, om, ox)`` is p7_MSVFilter
(src/impl_sse/msvfilter.c:78) and ``pipeline_msv_stage`` is the MSV stage of
p7_Pipeline (src/p7_pipeline.c:662-677). Everything runs through
libmsvgb.so; importing this module on a machine without it, or creating a
Context without a CUDA device, raises instead of falling back to the CPU.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import formats as F

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmsvgb.so")

eslOK, eslFAIL, eslEMEM, eslEINVAL, eslESYS, eslERANGE = 0, 1, 5, 11, 12, 16
eslEOF, eslENOTFOUND, eslEFORMAT, eslEINCOMPAT, eslEWRITE = 3, 6, 7, 10, 27
FLAG_ERANGE, FLAG_PASS, FLAG_FULL, FLAG_EMPTY = 0x01, 0x02, 0x04, 0x08

# Every function declared in include/msvgb.h.
EXPORTS = [
    "msvgb_ctx_create", "msvgb_ctx_destroy", "msvgb_ctx_set_stream", "msvgb_last_error",
    "msvgb_kernel_launches", "msvgb_MSVFilter", "msvgb_profile_create", "msvgb_profile_destroy",
    "msvgb_profile_M", "msvgb_profile_create_ex", "msvgb_profile_variant", "msvgb_profile_set_lanes",
    "msvgb_profile_lanes", "msvgb_profile_set_ssv_int8_words", "msvgb_profile_ssv_int8_words", "msvgb_db_create", "msvgb_db_destroy", "msvgb_db_nseq", "msvgb_db_residues",
    "msvgb_search", "msvgb_search_device", "msvgb_tjb_b", "msvgb_score", "msvgb_f1_pass",
    "msvgb_search_static", "msvgb_sample_om", "msvgb_calibrate",
    "msvgb_batch_create", "msvgb_batch_run", "msvgb_batch_items", "msvgb_batch_destroy", "msvgb_search_batch",
    "msvgb_server_create", "msvgb_server_slots", "msvgb_server_submit", "msvgb_server_wait",
    "msvgb_server_launches", "msvgb_server_solo_searches", "msvgb_server_destroy", "msvgb_pipeline_run",
    "msvgb_autotune", "msvgb_tune_save", "msvgb_tune_load", "msvgb_tune_lanes",
    "msvgb_h3f_open", "msvgb_h3f_read", "msvgb_h3f_close", "msvgb_h3f_write", "msvgb_fasta_read",
    "msvgb_seqs_n", "msvgb_seqs_codes", "msvgb_seqs_offsets", "msvgb_seqs_name", "msvgb_seqs_free",
    "msvgb_db_save", "msvgb_db_load", "msvgb_db_lengths", "msvgb_search_host",
    "msvgb_vprofile_create", "msvgb_vprofile_destroy", "msvgb_vitfilter", "msvgb_vit_score", "msvgb_vit_move_cost",
    "msvgb_biasfilter", "msvgb_bias_length_term", "msvgb_null_score", "msvgb_stage_pass", "msvgb_pipeline_filters",
    "msvgb_filter_collect", "msvgb_h3f_filter_params", "msvgb_h3p_open", "msvgb_h3p_read", "msvgb_h3p_close",
]


class MSVError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"status {code}: {msg}")
        self.code = code


class _Om(ctypes.Structure):
    _fields_ = [("M", ctypes.c_int), ("Kp", ctypes.c_int), ("rbv", ctypes.c_void_p),
                ("tbm_b", ctypes.c_uint8), ("tec_b", ctypes.c_uint8), ("tjb_b", ctypes.c_uint8),
                ("base_b", ctypes.c_uint8), ("bias_b", ctypes.c_uint8),
                ("scale_b", ctypes.c_float), ("mmu", ctypes.c_float), ("mlambda", ctypes.c_float)]


class _VOm(ctypes.Structure):
    _fields_ = [("M", ctypes.c_int), ("Kp", ctypes.c_int), ("twv", ctypes.c_void_p), ("rwv", ctypes.c_void_p),
                ("xw", ctypes.c_int16 * 8), ("scale_w", ctypes.c_float), ("nj", ctypes.c_float),
                ("base_w", ctypes.c_int16), ("ddbound_w", ctypes.c_int16)]


def _vom_struct(vp: F.VProfile):
    twv = np.ascontiguousarray(vp.twv, dtype=np.int16)
    rwv = np.ascontiguousarray(vp.rwv, dtype=np.int16)
    xw = (ctypes.c_int16 * 8)(*[int(v) for v in np.asarray(vp.xw).reshape(-1)])
    return _VOm(vp.M, vp.Kp, twv.ctypes.data, rwv.ctypes.data, xw, vp.scale_w, vp.nj, vp.base_w, vp.ddbound_w), (twv, rwv)


class _Filters(ctypes.Structure):
    _fields_ = [("om", ctypes.POINTER(_Om)), ("vom", ctypes.POINTER(_VOm)), ("compo", ctypes.c_void_p),
                ("vmu", ctypes.c_float), ("vlambda", ctypes.c_float), ("F1", ctypes.c_double), ("F2", ctypes.c_double)]


class FilterHit(ctypes.Structure):
    _fields_ = [("seq_index", ctypes.c_int64), ("usc", ctypes.c_float), ("nullsc", ctypes.c_float),
                ("filtersc", ctypes.c_float), ("vfsc", ctypes.c_float)]


class _FilterSink(ctypes.Structure):
    _fields_ = [("hits", ctypes.c_void_p), ("cap", ctypes.c_int64), ("n", ctypes.c_int64)]


class FilterStats(ctypes.Structure):
    _fields_ = [("nseqs", ctypes.c_int64), ("nres", ctypes.c_int64), ("n_past_msv", ctypes.c_int64),
                ("n_past_bias", ctypes.c_int64), ("n_past_vit", ctypes.c_int64)]


class _Omx(ctypes.Structure):
    _fields_ = [("allocQ16", ctypes.c_int), ("M", ctypes.c_int)]


_lib = None


def lib():
    """Loads libmsvgb.so (built by cudahmmsearch_gb300/build.py or __graft_entry__.build())."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    L = ctypes.CDLL(LIB_PATH)
    vp, i32, i64, u8, f32, f64 = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint8,
                                  ctypes.c_float, ctypes.c_double)
    sig = {
        "msvgb_ctx_create": (i32, [i32, ctypes.POINTER(vp)]),
        "msvgb_ctx_destroy": (i32, [vp]),
        "msvgb_ctx_set_stream": (i32, [vp, vp]),
        "msvgb_last_error": (ctypes.c_char_p, []),
        "msvgb_kernel_launches": (ctypes.c_uint64, []),
        "msvgb_MSVFilter": (i32, [vp, vp, i32, ctypes.POINTER(_Om), ctypes.POINTER(_Omx), ctypes.POINTER(f32)]),
        "msvgb_profile_create": (i32, [vp, ctypes.POINTER(_Om), ctypes.POINTER(vp)]),
        "msvgb_profile_create_ex": (i32, [vp, ctypes.POINTER(_Om), i32, ctypes.POINTER(vp)]),
        "msvgb_profile_variant": (i32, [vp]),
        "msvgb_profile_set_lanes": (i32, [vp, ctypes.POINTER(_Om), i32]),
        "msvgb_profile_set_ssv_int8_words": (i32, [vp, ctypes.POINTER(_Om), i32]),
        "msvgb_profile_ssv_int8_words": (i32, [vp]),
        "msvgb_autotune": (i32, [vp, ctypes.c_double]),
        "msvgb_tune_save": (i32, [vp, ctypes.c_char_p]),
        "msvgb_tune_load": (i32, [vp, ctypes.c_char_p]),
        "msvgb_tune_lanes": (i32, [vp, i32, i32, ctypes.POINTER(i32)]),
        "msvgb_h3f_open": (i32, [ctypes.c_char_p, ctypes.POINTER(vp)]),
        "msvgb_h3f_read": (i32, [vp, ctypes.POINTER(_Om), ctypes.c_char_p, i32]),
        "msvgb_h3f_close": (i32, [vp]),
        "msvgb_h3f_write": (i32, [ctypes.c_char_p, ctypes.POINTER(_Om), ctypes.c_char_p, i32]),
        "msvgb_fasta_read": (i32, [ctypes.c_char_p, ctypes.POINTER(vp)]),
        "msvgb_seqs_n": (ctypes.c_int64, [vp]),
        "msvgb_seqs_codes": (vp, [vp]),
        "msvgb_seqs_offsets": (vp, [vp]),
        "msvgb_seqs_name": (ctypes.c_char_p, [vp, ctypes.c_int64]),
        "msvgb_seqs_free": (i32, [vp]),
        "msvgb_db_save": (i32, [vp, ctypes.c_char_p]),
        "msvgb_db_load": (i32, [vp, ctypes.c_char_p, ctypes.POINTER(vp)]),
        "msvgb_db_lengths": (i32, [vp, vp]),
        "msvgb_search_host": (i32, [vp, vp, vp, vp, ctypes.c_int64, ctypes.c_double, ctypes.c_int64, vp, vp]),
        "msvgb_vprofile_create": (i32, [vp, ctypes.POINTER(_VOm), ctypes.POINTER(vp)]),
        "msvgb_vprofile_destroy": (i32, [vp]),
        "msvgb_vitfilter": (i32, [vp, vp, vp, vp, ctypes.c_int64, vp, vp]),
        "msvgb_vit_score": (ctypes.c_float, [i32, i32, i32, ctypes.POINTER(_VOm)]),
        "msvgb_vit_move_cost": (ctypes.c_int16, [ctypes.c_float, ctypes.c_float, i32]),
        "msvgb_profile_lanes": (i32, [vp]),
        "msvgb_profile_destroy": (i32, [vp]),
        "msvgb_profile_M": (i32, [vp]),
        "msvgb_db_create": (i32, [vp, vp, vp, i64, ctypes.POINTER(vp)]),
        "msvgb_db_destroy": (i32, [vp]),
        "msvgb_db_nseq": (i64, [vp]),
        "msvgb_db_residues": (i64, [vp]),
        "msvgb_search": (i32, [vp, vp, vp, f64, vp, vp]),
        "msvgb_search_device": (i32, [vp, vp, vp, f64, vp, vp]),
        "msvgb_tjb_b": (u8, [f32, i32]),
        "msvgb_score": (f32, [u8, u8, i32, u8, f32]),
        "msvgb_f1_pass": (i32, [f32, i32, f32, f32, f64, ctypes.POINTER(f64)]),
        "msvgb_search_static": (i32, [vp, vp, f64, vp, vp, vp]),
        "msvgb_sample_om": (i32, [ctypes.c_uint32, i32, vp, ctypes.POINTER(_Om), ctypes.POINTER(f64)]),
        "msvgb_calibrate": (i32, [vp, ctypes.POINTER(_Om), f64]),
        "msvgb_batch_create": (i32, [vp, vp, i32, vp, f64, vp, vp, ctypes.POINTER(vp)]),
        "msvgb_batch_run": (i32, [vp]),
        "msvgb_batch_items": (i64, [vp]),
        "msvgb_batch_destroy": (i32, [vp]),
        "msvgb_search_batch": (i32, [vp, vp, i32, vp, f64, vp, vp]),
        "msvgb_server_create": (i32, [vp, vp, f64, i32, ctypes.c_size_t, ctypes.POINTER(vp)]),
        "msvgb_server_slots": (i32, [vp]),
        "msvgb_server_submit": (i32, [vp, ctypes.POINTER(_Om), ctypes.POINTER(ctypes.c_uint64)]),
        "msvgb_server_wait": (i32, [vp, ctypes.c_uint64, vp, vp, f64]),
        "msvgb_server_launches": (ctypes.c_uint64, [vp]),
        "msvgb_server_solo_searches": (ctypes.c_uint64, [vp]),
        "msvgb_server_destroy": (i32, [vp]),
        "msvgb_pipeline_run": (i32, [vp, ctypes.POINTER(_Om), vp, vp, i64, i64, f64, i32, vp, vp,
                                     ctypes.POINTER(i64)]),
        "msvgb_biasfilter": (i32, [vp, vp, i32, vp, vp, i64, vp]),
        "msvgb_bias_length_term": (f32, [f32, i32]),
        "msvgb_null_score": (f32, [i32]),
        "msvgb_stage_pass": (i32, [f32, f32, f64, f64, f64, ctypes.POINTER(f64)]),
        "msvgb_pipeline_filters": (i32, [vp, ctypes.POINTER(_Filters), vp, vp, i64, i64, i32, vp, vp,
                                         ctypes.POINTER(FilterStats)]),
        "msvgb_filter_collect": (i32, [vp, vp]),
        "msvgb_h3f_filter_params": (i32, [vp, vp, ctypes.POINTER(f32), ctypes.POINTER(f32)]),
        "msvgb_h3p_open": (i32, [ctypes.c_char_p, ctypes.POINTER(vp)]),
        "msvgb_h3p_read": (i32, [vp, ctypes.POINTER(_VOm), ctypes.c_char_p, i32]),
        "msvgb_h3p_close": (i32, [vp]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype, fn.argtypes = res, args
    _lib = L
    return L


def _check(code):
    if code != eslOK:
        raise MSVError(code, lib().msvgb_last_error().decode())
    return code


def kernel_launches() -> int:
    return int(lib().msvgb_kernel_launches())


def _om_struct(p: F.Profile, tjb_b: int = 0):
    rbv = np.ascontiguousarray(p.rbv, dtype=np.uint8)
    om = _Om(p.M, p.Kp, rbv.ctypes.data, p.tbm_b, p.tec_b, tjb_b, p.base_b, p.bias_b,
             p.scale_b, p.mmu, p.mlambda)
    return om, rbv


class Context:
    """One GPU and one CUDA stream (msvgb_ctx)."""

    def __init__(self, device: int = 0):
        h = ctypes.c_void_p()
        _check(lib().msvgb_ctx_create(device, ctypes.byref(h)))
        self.h = h

    def set_stream(self, stream_handle: int | None):
        _check(lib().msvgb_ctx_set_stream(self.h, ctypes.c_void_p(stream_handle or 0)))

    def close(self):
        if self.h:
            lib().msvgb_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- lane-count autotuner ---------------------------------------------------
    def autotune(self, budget_s: float = 0.0, cache: str | None = None) -> str:
        """Lanes per sequence per (model length, target-length bin) for this GPU.
        With cache: load it when it was measured on this GPU model, else measure
        and write it. Returns "loaded" or "measured"."""
        if cache and os.path.exists(cache):
            st = lib().msvgb_tune_load(self.h, cache.encode())
            if st == eslOK:
                return "loaded"
            if st not in (eslEFORMAT, eslEINCOMPAT):
                _check(st)
        _check(lib().msvgb_autotune(self.h, budget_s))
        if cache:
            _check(lib().msvgb_tune_save(self.h, cache.encode()))
        return "measured"

    def tune_save(self, path: str):
        _check(lib().msvgb_tune_save(self.h, path.encode()))

    def tune_load(self, path: str):
        _check(lib().msvgb_tune_load(self.h, path.encode()))

    def tune_lanes(self, M: int, L: int = -1):
        """(lanes, variant) the context picks for model length M and target length L (-1: mix)."""
        v = ctypes.c_int()
        g = lib().msvgb_tune_lanes(self.h, M, L, ctypes.byref(v))
        return int(g), int(v.value)

    # -- p7_MSVFilter drop-in --------------------------------------------------
    def MSVFilter(self, dsq: np.ndarray, L: int, om: F.Profile, tjb_b: int, allocQ16: int | None = None):
        """p7_MSVFilter(dsq, L, om, ox, &sc): dsq holds sentinels at 0 and L+1.
        Returns (status, sc). status is eslOK or eslERANGE; raises on eslEINVAL."""
        dsq = np.ascontiguousarray(dsq, dtype=np.uint8)
        o, keep = _om_struct(om, tjb_b)
        ox = _Omx(om.Q if allocQ16 is None else allocQ16, 0)
        sc = ctypes.c_float()
        st = lib().msvgb_MSVFilter(self.h, dsq.ctypes.data, L, ctypes.byref(o), ctypes.byref(ox), ctypes.byref(sc))
        if st not in (eslOK, eslERANGE):
            raise MSVError(st, lib().msvgb_last_error().decode())
        return st, float(sc.value)


class DeviceProfile:
    """A profile resident in HBM (msvgb_profile)."""

    def __init__(self, ctx: Context, p: F.Profile, variant: int | None = None):
        o, keep = _om_struct(p)
        h = ctypes.c_void_p()
        if variant is None:
            _check(lib().msvgb_profile_create(ctx.h, ctypes.byref(o), ctypes.byref(h)))
        else:
            _check(lib().msvgb_profile_create_ex(ctx.h, ctypes.byref(o), variant, ctypes.byref(h)))
        self.h, self.ctx, self.profile = h, ctx, p
        self.variant = int(lib().msvgb_profile_variant(h))

    def set_lanes(self, lanes: int):
        """Lanes per sequence of the SSV pass (32, 16 or 8)."""
        o, keep = _om_struct(self.profile)
        _check(lib().msvgb_profile_set_lanes(self.h, ctypes.byref(o), lanes))

    @property
    def lanes(self) -> int:
        return int(lib().msvgb_profile_lanes(self.h))

    def set_int8_words(self, words: int):
        """DP words per lane of the 16/8-lane SSV pass whose costs are bytes (mixed-width table)."""
        o, keep = _om_struct(self.profile)
        _check(lib().msvgb_profile_set_ssv_int8_words(self.h, ctypes.byref(o), words))

    @property
    def int8_words(self) -> int:
        return int(lib().msvgb_profile_ssv_int8_words(self.h))

    def close(self):
        if self.h:
            lib().msvgb_profile_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class DeviceDB:
    """A packed, length-sorted sequence database resident in HBM (msvgb_db)."""

    def __init__(self, ctx: Context, seqs: F.SeqSet):
        codes = np.ascontiguousarray(seqs.codes, dtype=np.uint8)
        if codes.size == 0:
            codes = np.zeros(1, np.uint8)
        off = np.ascontiguousarray(seqs.off, dtype=np.int64)
        h = ctypes.c_void_p()
        _check(lib().msvgb_db_create(ctx.h, codes.ctypes.data, off.ctypes.data, seqs.n, ctypes.byref(h)))
        self.h, self.ctx, self.n, self.lengths = h, ctx, seqs.n, seqs.lengths.copy()
        self.residues = int(seqs.total)

    def save(self, path: str):
        """Writes the packed layout (msvgb_db_save)."""
        _check(lib().msvgb_db_save(self.h, path.encode()))

    @classmethod
    def load(cls, ctx: Context, path: str) -> "DeviceDB":
        """A database from a packed file (msvgb_db_load)."""
        h = ctypes.c_void_p()
        _check(lib().msvgb_db_load(ctx.h, path.encode(), ctypes.byref(h)))
        self = cls.__new__(cls)
        self.h, self.ctx = h, ctx
        self.n = int(lib().msvgb_db_nseq(h))
        self.residues = int(lib().msvgb_db_residues(h))
        self.lengths = np.zeros(self.n, np.int32)
        if self.n:
            _check(lib().msvgb_db_lengths(h, self.lengths.ctypes.data))
        return self

    def close(self):
        if self.h:
            lib().msvgb_db_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_h3f(path: str, filter_params: bool = False):
    """Every record of a pressed MSV profile file: [(name, Profile)]; with
    filter_params, [(name, Profile, compo float32[20], vmu, vlambda)] -- the
    composition and Viterbi Gumbel parameters the later filter stages use."""
    h = ctypes.c_void_p()
    _check(lib().msvgb_h3f_open(path.encode(), ctypes.byref(h)))
    out = []
    try:
        name = ctypes.create_string_buffer(1024)
        while True:
            o = _Om()
            st = lib().msvgb_h3f_read(h, ctypes.byref(o), name, 1024)
            if st == eslEOF:
                break
            _check(st)
            Q = F.nqb(o.M)
            rbv = np.ctypeslib.as_array(ctypes.cast(o.rbv, ctypes.POINTER(ctypes.c_uint8)),
                                        shape=(o.Kp * Q * 16,)).reshape(o.Kp, Q, 16).copy()
            prof = F.Profile(M=o.M, rbv=rbv, tbm_b=o.tbm_b, tec_b=o.tec_b, base_b=o.base_b, bias_b=o.bias_b,
                             scale_b=o.scale_b, mmu=o.mmu, mlambda=o.mlambda, tjb_cfg=o.tjb_b)
            if filter_params:
                compo = np.zeros(20, np.float32)
                vmu, vlam = ctypes.c_float(), ctypes.c_float()
                _check(lib().msvgb_h3f_filter_params(h, compo.ctypes.data, ctypes.byref(vmu), ctypes.byref(vlam)))
                out.append((name.value.decode(), prof, compo, vmu.value, vlam.value))
            else:
                out.append((name.value.decode(), prof))
    finally:
        lib().msvgb_h3f_close(h)
    return out


def read_h3p(path: str):
    """Every record of a pressed profile's .h3p file, its ViterbiFilter part:
    [(name, VProfile)]."""
    h = ctypes.c_void_p()
    _check(lib().msvgb_h3p_open(path.encode(), ctypes.byref(h)))
    out = []
    try:
        name = ctypes.create_string_buffer(1024)
        while True:
            v = _VOm()
            st = lib().msvgb_h3p_read(h, ctypes.byref(v), name, 1024)
            if st == eslEOF:
                break
            _check(st)
            Q8 = max(2, (v.M - 1) // 8 + 1)
            twv = np.ctypeslib.as_array(ctypes.cast(v.twv, ctypes.POINTER(ctypes.c_int16)), shape=(8 * Q8 * 8,))
            rwv = np.ctypeslib.as_array(ctypes.cast(v.rwv, ctypes.POINTER(ctypes.c_int16)), shape=(v.Kp * Q8 * 8,))
            xw = np.array(list(v.xw), np.int16).reshape(4, 2)
            out.append((name.value.decode(), F.VProfile(M=v.M, twv=twv.reshape(8 * Q8, 8).copy(),
                                                         rwv=rwv.reshape(v.Kp, Q8, 8).copy(), xw=xw,
                                                         scale_w=v.scale_w, nj=v.nj, base_w=v.base_w,
                                                         ddbound_w=v.ddbound_w)))
    finally:
        lib().msvgb_h3p_close(h)
    return out


def write_h3f(path: str, named_profiles):
    """Writes [(name, Profile)] as a pressed MSV profile file."""
    for i, (name, p) in enumerate(named_profiles):
        o, keep = _om_struct(p, p.tjb_cfg)
        _check(lib().msvgb_h3f_write(path.encode(), ctypes.byref(o), name.encode(), 1 if i else 0))


def read_fasta(path: str):
    """(SeqSet of digital amino codes, names) of a FASTA file."""
    h = ctypes.c_void_p()
    _check(lib().msvgb_fasta_read(path.encode(), ctypes.byref(h)))
    try:
        n = int(lib().msvgb_seqs_n(h))
        off = np.ctypeslib.as_array(ctypes.cast(lib().msvgb_seqs_offsets(h), ctypes.POINTER(ctypes.c_int64)),
                                    shape=(n + 1,)).copy()
        total = int(off[-1])
        codes = (np.ctypeslib.as_array(ctypes.cast(lib().msvgb_seqs_codes(h), ctypes.POINTER(ctypes.c_uint8)),
                                       shape=(total,)).copy() if total else np.zeros(0, np.uint8))
        names = [lib().msvgb_seqs_name(h, i).decode() for i in range(n)]
    finally:
        lib().msvgb_seqs_free(h)
    return F.SeqSet(codes, off), names


def search_host(ctx: Context, prof: DeviceProfile, seqs: F.SeqSet, F1: float = 0.02, chunk_residues: int = 0,
                out=None):
    """End to end from host buffers (msvgb_search_host): chunked upload and
    packing overlapped with the search. Returns (xj, flags) as search();
    out: optional (xj, flags) uint8 arrays of n entries to write them to
    (pinned ones make the results' copy a direct DMA)."""
    codes = np.ascontiguousarray(seqs.codes, dtype=np.uint8)
    if codes.size == 0:
        codes = np.zeros(1, np.uint8)
    off = np.ascontiguousarray(seqs.off, dtype=np.int64)
    if out is not None:
        xj, fl = out
        if (xj.dtype != np.uint8 or fl.dtype != np.uint8 or xj.size != seqs.n or fl.size != seqs.n
                or not xj.flags.c_contiguous or not fl.flags.c_contiguous):
            raise ValueError("out must be two contiguous uint8 arrays of n entries")
    else:
        xj = np.zeros(seqs.n, np.uint8)
        fl = np.zeros(seqs.n, np.uint8)
    _check(lib().msvgb_search_host(ctx.h, prof.h, codes.ctypes.data, off.ctypes.data, seqs.n, F1,
                                   chunk_residues, xj.ctypes.data, fl.ctypes.data))
    return xj, fl


class DeviceVProfile:
    """The ViterbiFilter part of a profile resident on the GPU (msvgb_vprofile)."""

    def __init__(self, ctx: Context, vp: F.VProfile):
        o, keep = _vom_struct(vp)
        h = ctypes.c_void_p()
        _check(lib().msvgb_vprofile_create(ctx.h, ctypes.byref(o), ctypes.byref(h)))
        self.h, self.ctx, self.vp = h, ctx, vp

    def close(self):
        if self.h:
            lib().msvgb_vprofile_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def vitfilter(ctx: Context, vprof: DeviceVProfile, db: DeviceDB, ids=None):
    """p7_ViterbiFilter on the listed sequences (original indices; all by
    default). Returns (status uint8 [0 ok, 1 overflow, 2 empty], score
    float32 nats) per listed sequence."""
    ids = np.arange(db.n, dtype=np.int64) if ids is None else np.ascontiguousarray(ids, dtype=np.int64)
    xc = np.zeros(ids.size, np.int32)
    st = np.zeros(ids.size, np.uint8)
    _check(lib().msvgb_vitfilter(ctx.h, vprof.h, db.h, ids.ctypes.data if ids.size else None, ids.size,
                                 xc.ctypes.data, st.ctypes.data))
    # msvgb_vit_score's float expression (vitfilter.c:240-247), vectorized: the
    # integer sums are exact in float32, the division is IEEE, and subtracting
    # 3.0 in double then rounding equals the float32 subtraction here
    vp = vprof.vp
    L = db.lengths[ids].astype(np.int64)
    uniq, inv = np.unique(L, return_inverse=True)
    move = np.array([lib().msvgb_vit_move_cost(vp.scale_w, vp.nj, int(x)) for x in uniq], np.float32)[inv]
    with np.errstate(over="ignore", invalid="ignore"):
        sc = (xc.astype(np.float32) + move - np.float32(vp.base_w)) / np.float32(vp.scale_w) - np.float32(3.0)
    sc = np.where(xc <= -32768, np.float32(-np.inf), sc).astype(np.float32)
    sc = np.where(st == 1, np.float32(np.inf), sc).astype(np.float32)
    return st, sc


def biasfilter(ctx: Context, compo, M: int, db: DeviceDB, ids=None):
    """p7_bg_FilterScore on the listed sequences (original indices; all by
    default) with the filter HMM of model composition compo[20] and length M.
    Returns float32 scores in nats."""
    ids = np.arange(db.n, dtype=np.int64) if ids is None else np.ascontiguousarray(ids, dtype=np.int64)
    c = np.ascontiguousarray(compo, dtype=np.float32)
    out = np.zeros(ids.size, np.float32)
    _check(lib().msvgb_biasfilter(ctx.h, c.ctypes.data, M, db.h, ids.ctypes.data if ids.size else None, ids.size,
                                  out.ctypes.data))
    return out


def stage_pass(sc: float, base: float, mu: float, lam: float, F: float):
    """The pipeline gate: (passes, P) for P = esl_gumbel_surv((sc - base) / log 2, mu, lambda)."""
    P = ctypes.c_double()
    r = lib().msvgb_stage_pass(sc, base, mu, lam, F, ctypes.byref(P))
    return bool(r), P.value


def search(ctx: Context, prof: DeviceProfile, db: DeviceDB, F1: float = 0.02):
    """Plain path: one profile, one launch. Returns (xj uint8[n], flags uint8[n])."""
    xj = np.zeros(db.n, np.uint8)
    fl = np.zeros(db.n, np.uint8)
    _check(lib().msvgb_search(ctx.h, prof.h, db.h, F1, xj.ctypes.data, fl.ctypes.data))
    return xj, fl


def search_device(ctx: Context, prof: DeviceProfile, db: DeviceDB, d_xj: int, d_flags: int, F1: float = 0.02):
    """Asynchronous search writing to device pointers (on the context's stream)."""
    _check(lib().msvgb_search_device(ctx.h, prof.h, db.h, F1, ctypes.c_void_p(d_xj), ctypes.c_void_p(d_flags)))


def sample_profile(M: int, seed: int, ctx: "Context | None" = None) -> F.Profile:
    """A profile sampled as HMMER's p7_hmm_Sample(seed) + p7_ProfileConfig +
    p7_oprofile_Convert would make it; with a context, also calibrated
    (p7_MSVMu on the GPU), else mmu = 0."""
    Q = F.nqb(M)
    rbv = np.zeros((F.KP_AMINO, Q, 16), np.uint8)
    om = _Om()
    lam = ctypes.c_double()
    _check(lib().msvgb_sample_om(seed, M, rbv.ctypes.data, ctypes.byref(om), ctypes.byref(lam)))
    if ctx is not None:
        _check(lib().msvgb_calibrate(ctx.h, ctypes.byref(om), lam.value))
    return F.Profile(M=M, rbv=rbv, tbm_b=om.tbm_b, tec_b=om.tec_b, base_b=om.base_b, bias_b=om.bias_b,
                     scale_b=float(np.float32(om.scale_b)), mmu=float(np.float32(om.mmu)),
                     mlambda=float(np.float32(om.mlambda)))


def _om_array(profiles):
    structs, keep = [], []
    for p in profiles:
        o, k = _om_struct(p)
        structs.append(o)
        keep.append(k)
    arr = (ctypes.POINTER(_Om) * len(structs))(*[ctypes.pointer(o) for o in structs])
    return arr, (structs, keep)


def search_batch(ctx: Context, profiles, db: DeviceDB, F1: float = 0.02):
    """Many profiles in one persistent launch. Returns (xj, flags) as uint8 [nprof, n]."""
    arr, keep = _om_array(profiles)
    xj = np.zeros((len(profiles), db.n), np.uint8)
    fl = np.zeros((len(profiles), db.n), np.uint8)
    _check(lib().msvgb_search_batch(ctx.h, ctypes.cast(arr, ctypes.c_void_p), len(profiles), db.h, F1,
                                    xj.ctypes.data, fl.ctypes.data))
    return xj, fl


class Batch:
    """A captured batched search (msvgb_batch): run() replays the CUDA graph."""

    def __init__(self, ctx: Context, profiles, db: DeviceDB, d_xj: int, d_flags: int, F1: float = 0.02):
        arr, keep = _om_array(profiles)
        h = ctypes.c_void_p()
        _check(lib().msvgb_batch_create(ctx.h, ctypes.cast(arr, ctypes.c_void_p), len(profiles), db.h, F1,
                                        ctypes.c_void_p(d_xj), ctypes.c_void_p(d_flags), ctypes.byref(h)))
        self.h = h
        self.items = int(lib().msvgb_batch_items(h))

    def run(self):
        _check(lib().msvgb_batch_run(self.h))

    def close(self):
        if self.h:
            lib().msvgb_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Continuous-batching serving loop over a resident database (msvgb_server).
    submit() admits a query (blocking while all device slots are busy) and
    returns a ticket; wait() returns its (xj, flags). Thread-safe."""

    def __init__(self, ctx: Context, db: DeviceDB, F1: float = 0.02, max_slots: int = 64,
                 mem_budget: int = 2 << 30):
        h = ctypes.c_void_p()
        _check(lib().msvgb_server_create(ctx.h, db.h, F1, max_slots, mem_budget, ctypes.byref(h)))
        self.h, self.db = h, db
        self.slots = int(lib().msvgb_server_slots(h))

    def submit(self, p: F.Profile) -> int:
        o, keep = _om_struct(p)
        t = ctypes.c_uint64()
        _check(lib().msvgb_server_submit(self.h, ctypes.byref(o), ctypes.byref(t)))
        return t.value

    def wait(self, ticket: int, timeout_s: float = 120.0, want=True):
        xj = np.zeros(self.db.n, np.uint8) if want else None
        fl = np.zeros(self.db.n, np.uint8) if want else None
        _check(lib().msvgb_server_wait(self.h, ticket, xj.ctypes.data if want else None,
                                       fl.ctypes.data if want else None, timeout_s))
        return xj, fl

    @property
    def launches(self) -> int:
        """Launches of the persistent serving kernel."""
        return int(lib().msvgb_server_launches(self.h))

    @property
    def solo_searches(self) -> int:
        """Requests run as their own single-query searches (M x residues >= 40e9)."""
        return int(lib().msvgb_server_solo_searches(self.h))

    def close(self):
        if self.h:
            lib().msvgb_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


SURVIVOR_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int64, ctypes.c_float,
                               ctypes.c_uint8, ctypes.c_uint8)


def pipeline_run(ctx: Context, p: F.Profile, seqs: F.SeqSet, on_survivor=None, *, block_size: int = 100_000,
                 F1: float = 0.02, n_workers: int = 4):
    """hmmsearch-style driver: blocks scored on the GPU, survivors of the F1
    gate handed to on_survivor(index, usc, xj, flags) on CPU worker threads.
    Returns n_past_msv."""
    o, keep = _om_struct(p)
    codes = np.ascontiguousarray(seqs.codes, dtype=np.uint8)
    if codes.size == 0:
        codes = np.zeros(1, np.uint8)
    off = np.ascontiguousarray(seqs.off, dtype=np.int64)
    cb = None
    if on_survivor is not None:
        def _cb(user, i, usc, xj, fl):
            return 1 if on_survivor(int(i), float(usc), int(xj), int(fl)) else 0
        cb = SURVIVOR_FN(_cb)
    n_past = ctypes.c_int64()
    _check(lib().msvgb_pipeline_run(ctx.h, ctypes.byref(o), codes.ctypes.data, off.ctypes.data, seqs.n,
                                    block_size, F1, n_workers, ctypes.cast(cb, ctypes.c_void_p) if cb else None,
                                    None, ctypes.byref(n_past)))
    return n_past.value


FILTER_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.POINTER(FilterHit))


def pipeline_filters(ctx: Context, p: F.Profile, seqs: F.SeqSet, *, vprof: F.VProfile | None = None, compo=None,
                     vmu: float = 0.0, vlambda: float = 0.0, on_hit=None, block_size: int = 100_000,
                     F1: float = 0.02, F2: float = 1e-3, n_workers: int = 4):
    """The filter stages of p7_Pipeline on the GPU (msvgb_pipeline_filters):
    MSV, bias filter (when compo is given), ViterbiFilter (when vprof is
    given). on_hit(seq_index, usc, nullsc, filtersc, vfsc) runs on the worker
    threads for every sequence past the last stage; without on_hit the hits
    are collected natively (msvgb_filter_collect). Returns (hits: structured
    array sorted by seq_index, empty with on_hit; stats: FilterStats)."""
    o, keep = _om_struct(p)
    vo, vkeep = _vom_struct(vprof) if vprof is not None else (None, None)
    c = np.ascontiguousarray(compo, dtype=np.float32) if compo is not None else None
    f = _Filters(ctypes.pointer(o), ctypes.pointer(vo) if vo is not None else None,
                 c.ctypes.data if c is not None else None, vmu, vlambda, F1, F2)
    codes = np.ascontiguousarray(seqs.codes, dtype=np.uint8)
    if codes.size == 0:
        codes = np.zeros(1, np.uint8)
    off = np.ascontiguousarray(seqs.off, dtype=np.int64)
    dt = np.dtype([("seq_index", np.int64), ("usc", np.float32), ("nullsc", np.float32),
                   ("filtersc", np.float32), ("vfsc", np.float32)])
    stats = FilterStats()
    args = (ctx.h, ctypes.byref(f), codes.ctypes.data, off.ctypes.data, seqs.n, block_size, n_workers)
    if on_hit is not None:
        def _cb(user, h):
            h = h.contents
            return 1 if on_hit(int(h.seq_index), h.usc, h.nullsc, h.filtersc, h.vfsc) else 0
        cb = FILTER_FN(_cb)
        _check(lib().msvgb_pipeline_filters(*args, ctypes.cast(cb, ctypes.c_void_p), None, ctypes.byref(stats)))
        return np.zeros(0, dt), stats
    cap = max(16, seqs.n // 8)
    while True:                                   # the native collector; rerun larger if it overflowed
        buf = np.zeros(cap, dt)
        sink = _FilterSink(buf.ctypes.data, cap, 0)
        _check(lib().msvgb_pipeline_filters(*args, ctypes.cast(lib().msvgb_filter_collect, ctypes.c_void_p),
                                            ctypes.byref(sink), ctypes.byref(stats)))
        if sink.n <= cap:
            break
        cap = sink.n
    hits = buf[:sink.n]
    hits = hits[np.argsort(hits["seq_index"], kind="stable")]   # a structured-array sort compares whole records
    return hits, stats


def tjb_b(scale_b: float, L: int) -> int:
    return int(lib().msvgb_tjb_b(scale_b, L))


def scores(p: F.Profile, lengths: np.ndarray, xj: np.ndarray, flags: np.ndarray) -> np.ndarray:
    """Float MSV scores (nats) from xJ, as p7_MSVFilter writes them (msvfilter.c:205-210)."""
    out = np.empty(len(xj), np.float32)
    f = lib().msvgb_score
    for i in range(len(xj)):
        out[i] = f(int(xj[i]), int(flags[i]), int(lengths[i]), p.base_b, p.scale_b)
    return out


def pipeline_msv_stage(ctx: Context, prof: DeviceProfile, db: DeviceDB, F1: float = 0.02):
    """MSV stage of p7_Pipeline over a whole database (p7_pipeline.c:662-677):
    returns (passed indices, their float scores usc, xj, flags). Sequences of
    length 0 are skipped as the reference does."""
    xj, fl = search(ctx, prof, db, F1)
    idx = np.nonzero(fl & FLAG_PASS)[0]
    usc = scores(prof.profile, db.lengths[idx], xj[idx], fl[idx])
    return idx, usc, xj, fl
