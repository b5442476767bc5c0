"""Builds libmsvgb.so (the CUDA kernels and the C ABI of include/msvgb.h) in-tree.

nvcc for sm_103a only, one -gencode, translation units compiled in parallel.
Host code is compiled with -ffp-contract=off so the score/P-value expressions
round exactly as the reference's (FMA-free) x86 build does.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmsvgb.so")
# the benchmark's peak probes: a library of their own (include/msvgb_probe.h)
PROBE_SRC = "msv_probe.cu"
PROBE_LIB = os.path.join(HERE, "libmsvgb_probe.so")

SOURCES = ["msv_batch.cu", "msv_serve.cu", "inst_g16.cu", "inst_g8.cu", "inst_hyb0.cu", "inst_l8.cu", "inst_l16.cu", "inst_w32.cu", "inst_hyb1.cu", "inst_hyb2.cu", "msv_api.cu", "msv_tune.cu", "msv_io.cu", "msv_vit.cu", "msv_noalloc.cu", "msv_pack.cu", "msv_sample.cu", "msv_pipeline.cu", "msv_bias.cu", "inst_a.cu", "inst_b.cu", "inst_c.cu", "inst_d.cu",
           "inst_e.cu", "inst_f.cu", "inst_h.cu", "inst_i.cu"]
HEADERS = ["msv_device.cuh", "msv_kernel_impl.cuh", "msv_internal.h", "msv_multi.cuh", "msv_group.cuh",
           "msv_hyb_list.h",
           os.path.join("..", "..", "include", "msvgb.h"), os.path.join("..", "..", "include", "msvgb_probe.h")]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.abspath(__file__)]
    jobs = []
    for s in SOURCES + [PROBE_SRC]:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        if force or _stale(obj, [src] + hdrs):
            jobs.append([nvcc()] + NVCC_FLAGS + ["-c", src, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            futs = [ex.submit(subprocess.run, j, capture_output=True, text=True) for j in jobs]
            for j, f in zip(jobs, futs):
                r = f.result()
                if verbose or r.returncode != 0:
                    sys.stderr.write(r.stdout + r.stderr)
                if r.returncode != 0:
                    raise RuntimeError(f"nvcc failed: {' '.join(j)}")
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    probe_obj = [os.path.join(BUILD, PROBE_SRC.replace(".cu", ".o"))]
    for lib, o in ((LIB, objs), (PROBE_LIB, probe_obj)):
        if force or jobs or _stale(lib, o):
            cmd = [nvcc()] + ARCH + ["-shared", "-o", lib] + o
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                sys.stderr.write(r.stdout + r.stderr)
                raise RuntimeError("link failed")
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
