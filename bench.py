"""Benchmark: MSV GCUPS on one GB300 (HMMER3 hmmsearch stage 1).

Default workload (N=1): one sampled profile of M=400 (HMMER p7_hmm_Sample,
seed 1, reference-generated: tests/golden/m400_s1.prof) against 2,000,000
synthetic protein sequences (lognormal lengths, median 300, sigma 0.7,
clipped to [10, 35000], 0.5% X, 2% homologs of the profile) -- the
"one query at throughput scale" configuration. A step is one full search of
the database by the profile. GCUPS = M * residues / seconds.

  value : device-timed (CUDA events on the launching stream), database and
          profile resident in HBM, outputs left on the device.
  e2e   : the same search through the public API from host buffers, every
          step: pinned host sequences -> device (packing included), search,
          per-sequence results back to the host (host wall clock).
  --impl reference : the reference's MSV algorithm on the host cores: a
          vectorized port of its SSE2 code (oracle/msv_port.c, NEON), since
          the reference's own SSE2 build cannot run on the aarch64 host.

The default line also carries, measured after the timed region:
  parity  : the timed outputs against the oracle on 50,000 random sequences
          of the timed database (status, xJ, float score bits, pass flag);
  batched : 256 profiles (M~U[50,1500]) vs 1,000,000 sequences in one
          persistent launch (CUDA graph) next to 256 single-query launches,
          with the batched-over-plain ratio and an oracle sample;
  serving : Poisson query streams at 50 and 500 queries/s on the resident
          database, with p50/p99 latency and offered vs achieved load.

The database (~770 MB) is larger than L2 (129 MB), so no flush is needed.
For N>1 (torchrun), the database is the concatenation of one block per rank
(each rank's block is its residue-balanced shard, generated by that rank);
every rank searches its shard (weak scaling: per-GPU work fixed) and the
per-sequence results are gathered once with a tensor all_gather.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

from cudahmmsearch_gb300 import formats as F  # noqa: E402

INT_LANE_OPS_PER_CLK_PER_SM = 128   # 4 SM sub-partitions x 32 lanes: nominal issue width
# DRAM bytes per residue of the hot kernel (the lane-group SSV pass), from the
# ncu capture of the lane-group SSV kernel on 400,000 sequences (summary under profiles/)
# (168.8 MB for 154.56 M residues); the pass reads each residue once, so
# traffic scales with the residue count.
DRAM_BYTES_PER_RESIDUE = 168.8e6 / 154.56e6
SMEM_BYTES_PER_CLK_PER_SM = 128     # one 128-byte shared-memory wavefront per clock


def ssv_table_bytes_per_cell(M, lanes, int8_words):
    """Shared-memory bytes of SSV cost read per DP cell: 2 (f16) for every
    word of a lane's row, 1 for the words of a mixed-width table that hold
    8-bit costs (lane groups: Cg = M / (2 lanes) + 1 words per lane)."""
    if lanes >= 32 or int8_words <= 0:
        return 2.0
    cg = M // (2 * lanes) + 1
    return (4.0 * (cg - int8_words) + 2.0 * int8_words) / (2.0 * cg)


def workload(name, rank=0, args=None):
    if name == "m400_2M":
        p = F.read_profile(os.path.join(ROOT, "tests", "golden", "m400_s1.prof"))
        n_total, n_hom = 2_000_000, 40_000
        bg = F.synth_sequences(n_total - n_hom, seed=1000 + rank, lmax=35000)
        hom = F.emit_homologs(p, n_hom, seed=2000 + rank, lmax=35000)
        s = F.SeqSet.concat([bg, hom])
        cfg = {"workload": "plain MSV, 1 profile M=400 (p7_hmm_Sample seed 1) vs 2,000,000 seqs "
                           "(lognormal median 300 sigma 0.7 clipped [10,35000], 0.5% X, 2% homologs)",
               "M": p.M, "n_seqs": s.n, "residues": s.total, "l2_flush": "inputs larger than L2 (129 MB)"}
        return p, s, cfg
    if name == "m400_400k":   # smaller case of the same distribution (profiling: > L2, few GB)
        p = F.read_profile(os.path.join(ROOT, "tests", "golden", "m400_s1.prof"))
        s = F.SeqSet.concat([F.synth_sequences(392_000, seed=1000 + rank, lmax=35000),
                             F.emit_homologs(p, 8_000, seed=2000 + rank, lmax=35000)])
        cfg = {"workload": "plain MSV, M=400 vs 400,000 seqs (same distribution as m400_2M)",
               "M": p.M, "n_seqs": s.n, "residues": s.total, "l2_flush": "inputs larger than L2 (129 MB)"}
        return p, s, cfg
    if name == "m2400_200k":  # length extremes: long targets and overflow-to-infinity
        p = F.read_profile(os.path.join(ROOT, "tests", "golden", "m2400_s1.prof"))
        s = F.SeqSet.concat([F.synth_sequences(199_000, seed=7000 + rank, lmax=35000, uniform_frac=0.1),
                             F.emit_homologs(p, 1_000, seed=7100 + rank, repeat=20, lmax=60000)])
        cfg = {"workload": "length extremes: M=2400 (p7_hmm_Sample seed 1) vs 200,000 seqs (90% lognormal "
                           "median 300, 10% uniform [5000,35000]) + 1,000 saturation seqs (emitted core x20)",
               "M": p.M, "n_seqs": s.n, "residues": s.total, "l2_flush": "inputs larger than L2 (129 MB)"}
        return p, s, cfg
    if name == "m200_20k":
        p = F.read_profile(os.path.join(ROOT, "tests", "golden", "m200_s1.prof"))
        s = F.SeqSet.concat([F.synth_sequences(19800, seed=11 + rank, lmax=5000), F.emit_homologs(p, 200, seed=12)])
        cfg = {"workload": "plain MSV, 1 profile M=200 vs 20,000 seqs (lognormal clipped [10,5000], 1% homologs)",
               "M": p.M, "n_seqs": s.n, "residues": s.total, "l2_flush": "none (inputs fit in L2)"}
        return p, s, cfg
    if name == "sampled":     # any model length: p7_hmm_Sample-style profile of length M, m400_2M's sequence law
        from cudahmmsearch_gb300 import api
        p = api.sample_profile(args.M, 1, api.Context(0))
        n_hom = args.nseq // 50
        s = F.SeqSet.concat([F.synth_sequences(args.nseq - n_hom, seed=1000 + rank, lmax=35000),
                             F.emit_homologs(p, n_hom, seed=2000 + rank, lmax=35000)])
        cfg = {"workload": f"plain MSV, 1 sampled profile M={args.M} (seed 1) vs {s.n:,} seqs "
                           "(lognormal median 300 sigma 0.7 clipped [10,35000], 0.5% X, 2% homologs)",
               "M": p.M, "n_seqs": s.n, "residues": s.total,
               "l2_flush": "inputs larger than L2 (129 MB)" if s.total > 129e6 else "none (inputs fit in L2)"}
        return p, s, cfg
    raise SystemExit(f"unknown workload {name}")


def measure_peak(name, device):
    """One of the probe library's peaks (include/msvgb_probe.h), measured now
    on this GPU: msvgb_measure_int_peak (32-bit integer ops/s) or
    msvgb_measure_smem_peak (shared-memory bytes/s)."""
    import ctypes
    L = ctypes.CDLL(os.path.join(ROOT, "cudahmmsearch_gb300", "libmsvgb_probe.so"))
    fn = getattr(L, name)
    fn.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    fn.restype = ctypes.c_int
    L.msvgb_probe_last_error.restype = ctypes.c_char_p
    v = ctypes.c_double()
    if fn(device, ctypes.byref(v)) != 0:
        raise RuntimeError(L.msvgb_probe_last_error().decode())
    return v.value


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.rows = []
        if self.proc is None:
            return
        time.sleep(0.25)
        self.proc.terminate()
        out, _ = self.proc.communicate(timeout=10)
        for line in out.strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                self.rows.append(f)

    def summary(self):
        rows = getattr(self, "rows", [])
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def cpu_baseline(p, s, budget_s=12.0, nthreads=0):
    """The reference's MSV algorithm (SSV first, full MSV when undecided) on
    all host cores: the vectorized port of its SSE2 code (oracle/msv_port.c,
    16 uint8 lanes on NEON here; bit-exact with the reference's golden
    vectors), on a bounded random sample of the workload's sequences."""
    from oracle import oracle as O
    rng = np.random.default_rng(7)
    cores = os.cpu_count() if nthreads <= 0 else nthreads
    # calibrate on a small sample, then size the timed sample to ~budget_s
    idx = rng.choice(s.n, size=min(s.n, 4000), replace=False)
    sub = s.subset(np.sort(idx))
    t0 = time.perf_counter()
    O.port_batch(p, sub, nthreads=cores)
    rate = sub.total * p.M / max(1e-6, time.perf_counter() - t0)
    want = int(min(s.n, max(4000, budget_s * rate / (p.M * max(1.0, s.total / s.n)))))
    idx = rng.choice(s.n, size=want, replace=False)
    sub = s.subset(np.sort(idx))
    reps = 0
    t0 = time.perf_counter()
    while True:                      # repeat a sample smaller than the budget until it is spent
        _, used = O.port_batch(p, sub, nthreads=cores)
        reps += 1
        if time.perf_counter() - t0 >= budget_s or reps >= 200:
            break
    dt = time.perf_counter() - t0
    return {"value": reps * sub.total * p.M / dt / 1e9, "unit": "GCUPS", "cores": used, "kind": "port",
            "sample": f"{sub.n} random sequences of the workload ({sub.total} residues, M={p.M}) x{reps}, {dt:.1f} s; "
                      f"vectorized port of the reference SSE2 p7_MSVFilter "
                      f"({'NEON' if os.uname().machine == 'aarch64' else 'GCC vector extensions'}; "
                      "SSV in register sweeps of diagonals as the reference), "
                      "bit-exact with its golden vectors",
            "seconds": dt}


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    p, s, cfg = workload(args.workload, 0, args)
    vals = []
    for i in range(args.warmup + args.steps):
        cb = cpu_baseline(p, s, budget_s=max(2.0, 60.0 / (args.steps + args.warmup)))
        if i >= args.warmup:
            vals.append(cb["value"])
    v = float(np.mean(vals))
    cb["value"] = v
    line = {"metric": "MSV GCUPS", "value": v, "unit": "GCUPS", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic", "config": cfg, "impl": "reference",
            "cpu_baseline": cb, "e2e": {"value": v, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


ORACLE_NOTE = ("oracle/msv_oracle.c: scalar C restatement of p7_MSVFilter (SSV decision, full MSV) and the "
               "p7_Pipeline F1 gate, pinned bit-exact to the reference's golden vectors")


def oracle_parity(api, p, s, xj, fl, n_check=50_000, seed=11):
    """Compares a GPU search's outputs (xj, flags over the whole SeqSet s) with
    the oracle on a random sample of s: the status (ERANGE or not), xJ where
    the status is eslOK, the float score's bit pattern and the F1 pass flag.
    Runs outside any timed region, on all host cores."""
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(s.n, size=min(n_check, s.n), replace=False))
    sub = s.subset(idx)
    t = time.perf_counter()
    o = O.msv_batch(p, sub)
    o_s = time.perf_counter() - t
    gx, gf = xj[idx], fl[idx]
    nonempty = sub.lengths > 0
    ok = o["status"] == 0
    mism = np.zeros(idx.size, bool)
    mism |= ((gf & api.FLAG_ERANGE) != 0) != (o["status"] == 16)
    mism[ok] |= gx[ok] != o["xj"][ok]
    mism[nonempty] |= ((gf & api.FLAG_PASS) != 0)[nonempty] != (o["pass"][nonempty] == 1)
    mism[~nonempty] |= (gf[~nonempty] & api.FLAG_EMPTY) == 0
    sc = api.scores(p, sub.lengths, gx, gf)
    mism[nonempty] |= sc.view(np.uint32)[nonempty] != o["sc"].view(np.uint32)[nonempty]
    return {"checked": int(idx.size), "mismatches": int(mism.sum()),
            "erange": int((o["status"] == 16).sum()), "passed": int((o["pass"] == 1).sum()),
            "compared": "status, xJ, float score bits, F1 pass flag", "oracle": ORACLE_NOTE,
            "oracle_s": round(o_s, 2)}


def batch_record(args, api, torch, ctx, stream, local, steps, warmup):
    """256 profiles (p7_hmm_Sample seeds 1..256, M uniform in [50, 1500],
    calibrated on the GPU) against 1,000,000 sequences in one persistent
    launch (a replayed CUDA graph), next to 256 back-to-back single-query
    launches on the same GPU (the reference's one-launch-per-query pattern).
    Returns (record, clock summary, launches, per-step ms)."""
    rng = np.random.default_rng(4)
    n_prof = args.nprof
    Ms = rng.integers(50, 1501, size=n_prof)
    t0 = time.perf_counter()
    profs = [api.sample_profile(int(M), i + 1, ctx) for i, M in enumerate(Ms)]
    prep_s = time.perf_counter() - t0
    n_seq = args.nseq
    n_hom = n_seq // 100
    bg = F.synth_sequences(n_seq - n_hom, seed=3000, lmax=35000)
    homs = [F.emit_homologs(profs[i % n_prof], 1, seed=5000 + i) for i in range(n_hom)]
    s = F.SeqSet.concat([bg] + homs)
    cells = float(sum(p.M for p in profs)) * float(s.total)
    db = api.DeviceDB(ctx, s)
    out = torch.empty(2 * n_prof * s.n, dtype=torch.uint8, device="cuda")
    d_xj, d_fl = out.data_ptr(), out.data_ptr() + n_prof * s.n
    batch = api.Batch(ctx, profs, db, d_xj, d_fl)
    for _ in range(warmup):
        batch.run()
    torch.cuda.synchronize()
    launches0 = api.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with ClockSampler(local) as clk:
        for i in range(steps):
            ev[i][0].record(stream)
            batch.run()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    launches = api.kernel_launches() - launches0
    per = [a.elapsed_time(b) for a, b in ev]
    total_ms = float(sum(per))
    value = cells * steps / (total_ms * 1e-3) / 1e9
    batched = out.cpu().numpy().copy()
    # the plain path: one single-query launch per profile, back to back
    dprofs = [api.DeviceProfile(ctx, p) for p in profs]
    plain = torch.empty(2 * s.n, dtype=torch.uint8, device="cuda")
    for dp in dprofs[:2]:
        api.search_device(ctx, dp, db, plain.data_ptr(), plain.data_ptr() + s.n)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for i, dp in enumerate(dprofs):
        api.search_device(ctx, dp, db, plain.data_ptr(), plain.data_ptr() + s.n)
    b.record(stream)
    torch.cuda.synchronize()
    plain_ms = a.elapsed_time(b)
    plain_value = cells / (plain_ms * 1e-3) / 1e9
    # identical per-pair xJ and flags (checked on a sample of profiles)
    mismatches, checked = 0, []
    for i in range(0, n_prof, max(1, n_prof // 16)):
        api.search_device(ctx, dprofs[i], db, plain.data_ptr(), plain.data_ptr() + s.n)
        torch.cuda.synchronize()
        pl = plain.cpu().numpy()
        mismatches += int((pl[:s.n] != batched[i * s.n:(i + 1) * s.n]).sum())
        mismatches += int((pl[s.n:] != batched[(n_prof + i) * s.n:(n_prof + i + 1) * s.n]).sum())
        checked.append(i)
    # the oracle on a sample of (profile, sequence) pairs: four profiles
    # spread over the model lengths, 2,000 random sequences each
    order = np.argsort(Ms)
    par = {"checked": 0, "mismatches": 0, "oracle": ORACLE_NOTE, "profiles_M": []}
    for j, pi in enumerate(order[np.linspace(0, n_prof - 1, 4).astype(int)]):
        r = oracle_parity(api, profs[pi], s, batched[pi * s.n:(pi + 1) * s.n],
                          batched[(n_prof + pi) * s.n:(n_prof + pi + 1) * s.n], n_check=2000, seed=100 + j)
        par["checked"] += r["checked"]
        par["mismatches"] += r["mismatches"]
        par["profiles_M"].append(int(Ms[pi]))
    del out, plain
    db.close()
    rec = {"workload": f"batched MSV: {n_prof} profiles (p7_hmm_Sample seeds 1..{n_prof}, M~U[50,1500], "
                       f"GPU-calibrated) vs {s.n} seqs (lognormal median 300, 1% homologs), one persistent "
                       "launch replayed as a CUDA graph",
           "value": value, "unit": "GCUPS", "steps": steps, "warmup": warmup, "ms_per_step": total_ms / steps,
           "n_profiles": n_prof, "n_seqs": s.n, "residues": s.total, "sum_M": int(sum(p.M for p in profs)),
           "work_items": batch.items, "profile_prep_s": round(prep_s, 2),
           "plain": {"value": plain_value, "unit": "GCUPS", "ms": plain_ms,
                     "what": f"{n_prof} back-to-back msvgb_search_device launches, one per profile"},
           "batched_over_plain": value / plain_value,
           "mismatches_vs_plain": mismatches, "profiles_checked_vs_plain": len(checked),
           "parity": par}
    batch.close()
    return rec, clk.summary(), launches, per


def run_batch(args, api, torch, ctx, stream, local):
    rec, clocks, launches, per = batch_record(args, api, torch, ctx, stream, local, args.steps, args.warmup)
    peak_tops = measure_peak("msvgb_measure_int_peak", local) / 1e12
    cells = float(rec["sum_M"]) * float(rec["residues"])
    achieved = cells / (np.mean(per) * 1e-3) / 1e12
    line = {"metric": "MSV GCUPS", "value": rec["value"], "unit": "GCUPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": rec["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": rec["workload"], "n_profiles": rec["n_profiles"], "n_seqs": rec["n_seqs"],
                       "residues": rec["residues"], "sum_M": rec["sum_M"], "work_items": rec["work_items"],
                       "profile_prep_s": rec["profile_prep_s"]},
            "plain_256_launches": rec["plain"],
            "batched_over_plain": rec["batched_over_plain"], "mismatches_vs_plain": rec["mismatches_vs_plain"],
            "parity": rec["parity"], "gpu_launches": int(launches), "clocks": clocks,
            "roofline": {"bound": "int32-pipe", "achieved": achieved, "peak": peak_tops, "unit": "Tops/s",
                         "frac": achieved / peak_tops, "traffic": None,
                         "peak_note": "measured: msvgb_measure_int_peak"}}
    print(json.dumps(line))


def run_filters(args, api, torch, ctx, stream, local):
    """The filter stages after MSV (p7_Pipeline, src/p7_pipeline.c:662-705) on
    the GPU. The model is the M=400 sampled HMM (seed 1) in hmmsearch's local
    configuration with the composition hmmbuild gives it (tests/golden/
    pipe_m400_s1.*, vit_m400_s1.vprof); the sequences follow m400_2M's law.
    Timed per step: (a) the ViterbiFilter kernel stage on 200,000 listed
    sequences (cells = M x residues), (b) the bias filter on the same list,
    each with CUDA events on the launching stream (the calls include the id
    upload and the result copy); (c) the whole filter pipeline (database
    blocks uploaded, MSV, bias, ViterbiFilter, gates) through
    msvgb_pipeline_filters from pinned host buffers, host wall clock."""
    G = os.path.join(ROOT, "tests", "golden")
    p = F.read_profile(os.path.join(G, "pipe_m400_s1.prof"))
    vp = F.read_vprofile(os.path.join(G, "vit_m400_s1.vprof"))
    pr = F.read_pipe(os.path.join(G, "pipe_m400_s1.pres"))
    n_seq = args.nseq
    n_hom = n_seq // 50
    s = F.SeqSet.concat([F.synth_sequences(n_seq - n_hom, seed=1000, lmax=35000),
                         F.emit_homologs(p, n_hom, seed=2000, lmax=35000)])
    db = api.DeviceDB(ctx, s)
    dvp = api.DeviceVProfile(ctx, vp)
    ids = np.arange(min(200_000, s.n), dtype=np.int64)
    res_ids = float(s.lengths[ids].sum())
    xc = np.zeros(ids.size, np.int32)
    vst = np.zeros(ids.size, np.uint8)
    fsc = np.zeros(ids.size, np.float32)
    c = np.ascontiguousarray(pr.compo, np.float32)
    L = api.lib()

    def vit():
        api._check(L.msvgb_vitfilter(ctx.h, dvp.h, db.h, ids.ctypes.data, ids.size, xc.ctypes.data, vst.ctypes.data))

    def bias():
        api._check(L.msvgb_biasfilter(ctx.h, c.ctypes.data, vp.M, db.h, ids.ctypes.data, ids.size, fsc.ctypes.data))

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        ms = []
        for _ in range(args.steps):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            fn()
            b.record(stream)
            torch.cuda.synchronize()
            ms.append(a.elapsed_time(b))
        return float(np.median(ms))
    # the pipeline reads the residues and offsets from pinned host memory
    hs = F.SeqSet(torch.from_numpy(s.codes).pin_memory().numpy(), torch.from_numpy(s.off).pin_memory().numpy())
    launches0 = api.kernel_launches()
    with ClockSampler(local) as clk:
        vit_ms = timed(vit)
        bias_ms = timed(bias)
        pipe_s = []
        for i in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t = time.perf_counter()
            hits, st = api.pipeline_filters(ctx, p, hs, vprof=vp, compo=pr.compo, vmu=pr.vmu, vlambda=pr.vlambda,
                                            block_size=500_000, n_workers=4)
            if i >= args.warmup:
                pipe_s.append(time.perf_counter() - t)
    launches = api.kernel_launches() - launches0
    cells = float(p.M) * float(s.total)
    value = cells / float(np.median(pipe_s)) / 1e9
    line = {"metric": "filter pipeline GCUPS", "value": value, "unit": "GCUPS", "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": float(np.median(pipe_s)) * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8/s16/f32", "data": "synthetic",
            "config": {"workload": f"p7_Pipeline filter stages (MSV, bias, ViterbiFilter) on the GPU, M=400 local "
                                   f"(p7_hmm_Sample seed 1) vs {s.n:,} seqs (m400_2M's law), blocks of 500,000, "
                                   f"from pinned host buffers",
                       "M": p.M, "n_seqs": s.n, "residues": s.total,
                       "n_past_msv": st.n_past_msv, "n_past_bias": st.n_past_bias, "n_past_vit": st.n_past_vit},
            "stages": {"vitfilter": {"ms": vit_ms, "gcups": vp.M * res_ids / (vit_ms * 1e-3) / 1e9,
                                     "n_seqs": int(ids.size), "residues": int(res_ids)},
                       "biasfilter": {"ms": bias_ms, "gres_per_s": res_ids / (bias_ms * 1e-3) / 1e9,
                                      "n_seqs": int(ids.size)},
                       "pipeline_s": [round(t, 4) for t in pipe_s]},
            "gpu_launches": int(launches), "clocks": clk.summary()}
    print(json.dumps(line))


def run_dropin(args, api, torch, ctx, local):
    """Per-call latency of the drop-in msvgb_MSVFilter (one sequence per call,
    as p7_Pipeline calls p7_MSVFilter, src/p7_pipeline.c:671) at L=300 for
    M = 200, 400, 2400, beside the reference's per-call cost on one host core
    (the vectorized port of its SSE2 filter) and the per-sequence cost of the
    batched search of the same sequences from a resident database. Host wall
    clock; the drop-in figure includes the ctypes call (its overhead alone,
    measured on a host-only C ABI function, is reported)."""
    import ctypes
    from oracle import oracle as O
    n = args.dropin_calls
    L = 300
    s = F.synth_sequences(n, seed=61, sigma=1e-9, lmin=L, lmax=L)
    assert int(s.lengths.min()) == L == int(s.lengths.max())
    f = api.lib().msvgb_tjb_b
    t = time.perf_counter()
    for _ in range(n):
        f(ctypes.c_float(4.328), L)
    ctypes_us = (time.perf_counter() - t) / n * 1e6
    rows = []
    for name in ("m200_s1", "m400_s1", "m2400_s1"):
        p = F.read_profile(os.path.join(ROOT, "tests", "golden", name + ".prof"))
        tjb = api.tjb_b(p.scale_b, L)
        dsqs = [np.concatenate([[255], s.seq(i), [255]]).astype(np.uint8) for i in range(n)]
        for i in range(min(50, n)):
            ctx.MSVFilter(dsqs[i], L, p, tjb)
        got = np.zeros(n, np.float32)
        t = time.perf_counter()
        for i in range(n):
            got[i] = ctx.MSVFilter(dsqs[i], L, p, tjb)[1]
        gpu_us = (time.perf_counter() - t) / n * 1e6
        o = O.msv_batch(p, s)
        mism = int((got.view(np.uint32) != o["sc"].view(np.uint32)).sum())
        O.port_batch(p, s, nthreads=1)
        t = time.perf_counter()
        O.port_batch(p, s, nthreads=1)
        cpu_us = (time.perf_counter() - t) / n * 1e6
        dp, db = api.DeviceProfile(ctx, p), api.DeviceDB(ctx, s)
        api.search(ctx, dp, db)
        t = time.perf_counter()
        api.search(ctx, dp, db)
        batch_us = (time.perf_counter() - t) / n * 1e6
        dp.close()
        db.close()
        rows.append({"M": p.M, "L": L, "dropin_us_per_call": gpu_us, "cpu_port_1core_us_per_call": cpu_us,
                     "resident_search_us_per_seq": batch_us, "dropin_over_cpu": cpu_us / gpu_us,
                     "score_mismatches_vs_oracle": mism})
    line = {"metric": "drop-in p7_MSVFilter latency", "value": rows[1]["dropin_us_per_call"], "unit": "us/call",
            "n_gpus": 1, "steps": n, "warmup": 50, "ms_per_step": rows[1]["dropin_us_per_call"] / 1e3,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": f"msvgb_MSVFilter one call per sequence, {n} sequences of L={L}, "
                                   "M = 200, 400, 2400 (reference-sampled golden profiles)",
                       "ctypes_call_us": ctypes_us},
            "rows": rows}
    print(json.dumps(line))


def serve_record(args, api, ctx, s, db, loads):
    """Serving: a resident database receives query profiles (p7_hmm_Sample
    with per-request seeds, M log-uniform in [50, 2000], calibrated
    beforehand) as Poisson streams at the given (rate q/s, window s) loads;
    admission is bounded by a device-memory budget. Latency = completion -
    arrival (admission wait included). The first two requests of every
    window are also searched alone on the plain path afterwards: their
    served results must be identical. Requests that fill the GPU alone
    (M x residues >= 40e9: all but the smallest models here) run as their own
    single-query searches, the others in the persistent serving kernel.
    Returns (windows, kernel launches, own searches, prep s, checks)."""
    import threading
    import concurrent.futures as cf
    rng = np.random.default_rng(9)
    n_req_total = sum(int(r * t * 1.5) + 8 for r, t in loads)
    Ms = np.exp(rng.uniform(np.log(50), np.log(2000), size=n_req_total)).astype(int)
    t0 = time.perf_counter()
    profs = [api.sample_profile(int(M), 10000 + i, ctx) for i, M in enumerate(Ms)]
    prep_s = time.perf_counter() - t0
    srv = api.Server(ctx, db, max_slots=args.slots, mem_budget=args.mem_budget)
    # warm-up: one query end to end
    srv.wait(srv.submit(profs[0]), want=False)
    results, kept = [], {}
    used = 1
    for rate, dur in loads:
        arr = np.cumsum(rng.exponential(1.0 / rate, size=int(rate * dur * 1.5) + 8))
        arr = arr[arr < dur]
        reqs = list(range(used, used + len(arr)))
        used += len(arr)
        keep_ids = set(reqs[:2])
        lat, done_t, cells = [], [], []
        lock = threading.Lock()
        pool = cf.ThreadPoolExecutor(max_workers=max(8, args.slots))
        start = time.perf_counter()

        def finish(tk, a_time, pi):
            xj, fl = srv.wait(tk, want=True)
            t = time.perf_counter() - start
            with lock:
                lat.append(t - a_time)
                done_t.append(t)
                cells.append(float(profs[pi].M) * s.total)
                if pi in keep_ids:
                    kept[pi] = (xj, fl)

        futs = []
        for a_time, pi in zip(arr, reqs):
            now = time.perf_counter() - start
            if a_time > now:
                time.sleep(a_time - now)
            tk = srv.submit(profs[pi])                     # blocks while no slot is free
            futs.append(pool.submit(finish, tk, float(a_time), pi))
        for f in futs:
            f.result()
        pool.shutdown()
        span = max(done_t) if done_t else 0.0
        mean_cells = float(np.mean([profs[i].M for i in reqs])) * s.total if reqs else 0.0
        results.append({"offered_qps": rate, "window_s": dur, "requests": len(reqs),
                        "offered_gcups": rate * mean_cells / 1e9,
                        "achieved_qps": len(reqs) / span if span else 0.0,
                        "achieved_gcups": sum(cells) / span / 1e9 if span else 0.0,
                        "latency_p50_ms": float(np.percentile(lat, 50) * 1e3) if lat else None,
                        "latency_p99_ms": float(np.percentile(lat, 99) * 1e3) if lat else None,
                        "latency_max_ms": float(np.max(lat) * 1e3) if lat else None})
    launches, solo = srv.launches, srv.solo_searches
    srv.close()
    mism = 0
    for pi, (xj, fl) in kept.items():                       # served in the mix == searched alone
        dp = api.DeviceProfile(ctx, profs[pi])
        xa, fa = api.search(ctx, dp, db)
        mism += int((xa != xj).sum() + (fa != fl).sum())
        dp.close()
    checks = {"requests_checked": len(kept), "mismatches_vs_alone": mism}
    return results, launches, solo, prep_s, checks


def run_serve(args, api, torch, ctx, local):
    s = F.synth_sequences(args.nseq if args.nseq != 1_000_000 else 2_000_000, seed=8000, lmax=35000)
    db = api.DeviceDB(ctx, s)
    loads = [(float(r), float(t)) for r, t in (x.split(":") for x in args.loads.split(","))]
    k0 = api.kernel_launches()
    results, launches, solo, prep_s, checks = serve_record(args, api, ctx, s, db, loads)
    k1 = api.kernel_launches() - k0
    best = max(r["achieved_gcups"] for r in results)
    line = {"metric": "MSV GCUPS (serving)", "value": best, "unit": "GCUPS", "n_gpus": 1, "steps": len(loads),
            "warmup": 1, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": {"workload": f"serving: resident {s.n} seqs (lognormal median 300, {s.total} residues), "
                                   "Poisson query streams, M log-uniform [50,2000] (p7_hmm_Sample per-request seeds)",
                       "slots": args.slots, "mem_budget_bytes": args.mem_budget, "profile_prep_s": prep_s},
            "serving": results, "checks": checks, "serve_kernel_launches": int(launches),
            "own_searches": int(solo), "gpu_launches": int(k1)}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="m400_2M")
    ap.add_argument("--variant", type=int, default=None, help="SSV arithmetic: 0 int8 table, 1 f16 table")
    ap.add_argument("--lanes", type=int, default=None, help="lanes per sequence of the SSV pass (32, 16, 8)")
    ap.add_argument("--int8-words", type=int, default=None,
                    help="lane-group SSV pass: DP words per lane with 8-bit costs (mixed-width table)")
    ap.add_argument("--M", type=int, default=100, help="sampled workload: model length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--nprof", type=int, default=256, help="batch workload: number of profiles")
    ap.add_argument("--nseq", type=int, default=1_000_000, help="batch/serve workload: database size")
    ap.add_argument("--loads", default="10:3,50:3,500:0.5", help="serve workload: rate:seconds,...")
    ap.add_argument("--slots", type=int, default=32, help="serve workload: max concurrent queries")
    ap.add_argument("--mem-budget", type=int, default=1 << 30, help="serve workload: device bytes for slots")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the batched and serving sub-records")
    ap.add_argument("--batch-steps", type=int, default=2, help="batched sub-record: timed replays")
    ap.add_argument("--serve-loads", default="50:2,500:0.4",
                    help="serving sub-record: rate:seconds,... on the default workload's database")
    ap.add_argument("--dropin-calls", type=int, default=2000, help="dropin workload: calls per model")
    ap.add_argument("--parity-seqs", type=int, default=50_000,
                    help="default workload: random sequences of the timed database checked against the oracle")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import torch.distributed as dist
    from cudahmmsearch_gb300 import api
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if args.workload == "batch256":
        ctx = api.Context(local)
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        ctx.set_stream(stream.cuda_stream)
        return run_batch(args, api, torch, ctx, stream, local)
    if args.workload == "serve":
        return run_serve(args, api, torch, api.Context(local), local)
    if args.workload == "dropin":
        return run_dropin(args, api, torch, api.Context(local), local)
    if args.workload == "filters":
        ctx = api.Context(local)
        stream = torch.cuda.Stream()
        torch.cuda.set_stream(stream)
        ctx.set_stream(stream.cuda_stream)
        return run_filters(args, api, torch, ctx, stream, local)

    p, s, cfg = workload(args.workload, rank, args)
    cells = float(p.M) * float(s.total)
    ctx = api.Context(local)
    # A dedicated (non-default) stream: its handle is non-NULL, so the library
    # launches on it and the CUDA events below time exactly those launches.
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx.set_stream(stream.cuda_stream)
    prof = api.DeviceProfile(ctx, p, args.variant)
    if args.lanes:
        prof.set_lanes(args.lanes)
    if args.int8_words is not None:
        prof.set_int8_words(args.int8_words)
    db = api.DeviceDB(ctx, s)
    out = torch.empty(2 * s.n, dtype=torch.uint8, device="cuda")
    d_xj, d_fl = out.data_ptr(), out.data_ptr() + s.n

    def step():
        api.search_device(ctx, prof, db, d_xj, d_fl)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    launches0 = api.kernel_launches()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        t0.record(stream)
        for i in range(args.steps):
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        t1.record(stream)
        torch.cuda.synchronize()
    launches = api.kernel_launches() - launches0
    if world > 1:
        dist.barrier()
    total_ms = t0.elapsed_time(t1)
    per = [a.elapsed_time(b) for a, b in ev]
    t_max = torch.tensor([total_ms], device="cuda")
    if world > 1:
        dist.all_reduce(t_max, op=dist.ReduceOp.MAX)
    total_ms = float(t_max.item())
    value = cells * world * args.steps / (total_ms * 1e-3) / 1e9

    # the timed outputs (the last step's) against the oracle on 50,000 random
    # sequences of the timed database (outside the timed region)
    xj_all = out[:s.n].cpu().numpy()
    fl_all = out[s.n:].cpu().numpy()
    parity = oracle_parity(api, p, s, xj_all, fl_all, n_check=args.parity_seqs) if rank == 0 else None

    # e2e through the public API from pinned host buffers
    codes_pin = torch.from_numpy(s.codes).pin_memory()
    off_pin = torch.from_numpy(s.off).pin_memory()
    res_pin = torch.zeros(2, s.n, dtype=torch.uint8).pin_memory()   # results come back by direct DMA
    e2e_times, e2e_parts = [], []
    seqset = F.SeqSet(codes_pin.numpy(), off_pin.numpy())
    for i in range(args.e2e_steps + 1 if args.e2e_steps > 0 else 0):
        torch.cuda.synchronize()
        t = time.perf_counter()
        xj, fl = api.search_host(ctx, prof, seqset,            # chunks searched as their residues arrive
                                 out=(res_pin[0].numpy(), res_pin[1].numpy()))
        dt = time.perf_counter() - t
        if i > 0:
            e2e_times.append(dt)
    if e2e_times:
        assert np.array_equal(xj, xj_all) and np.array_equal(fl, fl_all)
        # the same work as two separate calls (database upload, then search), for the breakdown
        torch.cuda.synchronize()
        t = time.perf_counter()
        db2 = api.DeviceDB(ctx, seqset)
        t_db = time.perf_counter()
        xj2, fl2 = api.search(ctx, prof, db2)
        t_search = time.perf_counter()
        db2.close()
        dt2 = time.perf_counter() - t
        assert np.array_equal(xj2, xj_all) and np.array_equal(fl2, fl_all)
        e2e_parts.append({"db_create_ms": (t_db - t) * 1e3, "search_ms": (t_search - t_db) * 1e3,
                          "destroy_ms": (t + dt2 - t_search) * 1e3,
                          "separate_calls_gcups": cells / dt2 / 1e9})
    e2e_val = cells / float(np.median(e2e_times)) / 1e9 if e2e_times else None

    clocks = clk.summary()
    sm_mhz = clocks["sm_mhz"] or 2070.0
    nsm = torch.cuda.get_device_properties(local).multi_processor_count
    peak_tops = measure_peak("msvgb_measure_int_peak", local) / 1e12    # measured now, same GPU and clock regime
    smem_peak = measure_peak("msvgb_measure_smem_peak", local) / 1e9
    tb = ssv_table_bytes_per_cell(p.M, prof.lanes, prof.int8_words)
    hbm_peak, hbm_note = 6800.0, "of fallback (6.8 TB/s: no measured peaks file)"
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm_peak, hbm_note = float(json.load(f)["hbm_gbs"]), "of measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, KeyError, ValueError):
        pass
    kern_ms = float(np.mean(per))
    achieved_tops = cells / (kern_ms * 1e-3) / 1e12          # 1 cell = 1 packed int32 op (4 uint8 lane-ops)
    roofline = {"bound": "int32-pipe", "achieved": achieved_tops, "peak": peak_tops, "unit": "Tops/s",
                "frac": achieved_tops / peak_tops,
                "traffic": DRAM_BYTES_PER_RESIDUE * s.total,
                "traffic_note": "DRAM bytes of the SSV pass scaled by residues from an ncu capture of the same "
                                "kernel on 400,000 sequences (summary under profiles/)",
                "peak_note": f"measured: msvgb_measure_int_peak (independent max.s32/xor over {nsm} SMs); "
                             f"nominal {nsm} SMs x {INT_LANE_OPS_PER_CLK_PER_SM} lane-ops/clk x {sm_mhz:.0f} MHz = "
                             f"{nsm * INT_LANE_OPS_PER_CLK_PER_SM * sm_mhz * 1e6 / 1e12:.1f} Tops/s",
                "smem": {"achieved": tb * cells / (kern_ms * 1e-3) / 1e9,
                         "peak": smem_peak, "unit": "GB/s",
                         "frac": tb * cells / (kern_ms * 1e-3) / 1e9 / smem_peak,
                         "nominal": nsm * SMEM_BYTES_PER_CLK_PER_SM * sm_mhz * 1e6 / 1e9,
                         "peak_note": "measured: msvgb_measure_smem_peak (conflict-free 16-byte loads over "
                                      f"{nsm} SMs); nominal {nsm} SMs x 128 B/clk x {sm_mhz:.0f} MHz. "
                                      f"{tb:.3f} B of SSV cost per cell ({prof.int8_words} of each lane's words "
                                      "8-bit, the rest f16): with issue, the bound the SSV pass runs "
                                      "against"},
                "hbm": {"achieved": (s.total + 2 * s.n) / (kern_ms * 1e-3) / 1e9, "peak": hbm_peak,
                        "unit": "GB/s", "frac": (s.total + 2 * s.n) / (kern_ms * 1e-3) / 1e9 / hbm_peak,
                        "peak_note": hbm_note}}
    fullfrac = float(((fl_all & api.FLAG_FULL) != 0).mean())
    line = {"metric": "MSV GCUPS", "value": value, "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "u8", "data": "synthetic",
            "config": dict(cfg, variant=prof.variant, lanes=prof.lanes, int8_words=prof.int8_words,
                           full_msv_fraction=fullfrac,
                           pass_fraction=float(((fl_all & api.FLAG_PASS) != 0).mean())),
            "e2e": {"value": e2e_val, "unit": "GCUPS", "h2d_bytes_per_step": int(s.total + 28 * s.n),
                    "d2h_bytes_per_step": int(2 * s.n),
                    "path": "msvgb_search_host from pinned host memory (residues and offsets) into pinned "
                            "result buffers: the offsets go up and the whole input is sorted on the GPU chunk "
                            "by chunk while every chunk's residues follow on the copy engine; each chunk is "
                            "packed and searched as it arrives, one full-MSV list pass at the end",
                    "separate_calls": e2e_parts[-1] if e2e_parts else None,
                    "steps_ms": [round(t * 1e3, 2) for t in e2e_times], "statistic": "median of the timed steps"},
            "gpu_launches": int(launches), "clocks": clocks, "roofline": roofline, "parity": parity}
    if world > 1:
        # the one exchange of the sharded search: every rank's per-sequence
        # bytes, concatenated in rank (= database) order on every rank
        from cudahmmsearch_gb300 import shard as S
        t = time.perf_counter()
        gx, gf = S.gather_results(xj_all, fl_all, device=torch.device("cuda", local))
        line["gather"] = {"seqs": int(gx.size), "ms": (time.perf_counter() - t) * 1e3,
                          "how": "torch.distributed all_gather of fixed-size uint8 tensors (NCCL)"}
    if rank == 0 and world == 1 and not args.no_extras:
        # the metric's other halves: batched vs plain, and serving latency
        del out
        torch.cuda.empty_cache()
        bsteps, bwarm = args.batch_steps, max(3, min(args.warmup, 3))
        brec, bclk, _, _ = batch_record(args, api, torch, ctx, stream, local, bsteps, bwarm)
        brec["clocks"] = bclk
        line["batched"] = brec
        loads = [(float(r), float(t)) for r, t in (x.split(":") for x in args.serve_loads.split(","))]
        sres, slaunch, ssolo, sprep, schecks = serve_record(args, api, ctx, s, db, loads)
        line["serving"] = {"workload": f"serving: the resident {s.n:,}-sequence database above, Poisson query "
                                       "streams, M log-uniform [50,2000] (p7_hmm_Sample per-request seeds)",
                           "windows": sres, "slots": args.slots, "mem_budget_bytes": args.mem_budget,
                           "profile_prep_s": round(sprep, 2), "kernel_launches": int(slaunch),
                           "own_searches": int(ssolo), **schecks}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(p, s)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
