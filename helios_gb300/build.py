"""Build libhrt.so (CUDA, sm_103a) in-tree with nvcc.

Translation units are compiled in parallel and linked into
``helios_gb300/_build/libhrt.so``.  Geometry code relies on IEEE single
precision without contraction, so every unit is compiled with --fmad=false,
-prec-div=true and -prec-sqrt=true (no --use_fast_math).
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
LIB = os.path.join(BUILD, "libhrt.so")
SOURCES = ["hrt_bvh.cu", "hrt_bvh4.cu", "hrt_trace.cu", "hrt_ps_accumulate.cu", "hrt_ps_special.cu", "hrt_ps_w4.cu", "hrt_camera.cu", "hrt_energy.cu", "hrt_ingest.cpp", "hrt_api.cu",
           "hrt_static.cu", "hrt_serve.cu"]
HEADERS = ["hrt_device.cuh", "hrt_internal.h", "hrt_trace.cuh", "hrt_trace_w4.cuh", os.path.join("..", "..", "include", "hrt.h")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-Xcompiler", "-ffp-contract=off",
           "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, h) for h in HEADERS]
    cc = nvcc()
    objs, jobs = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s, *headers, __file__]):
            cmd = [cc, *ARCH, *NVFLAGS, *(extra or []), "-c", s, "-o", o]
            jobs.append(cmd)
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if verbose or r.returncode:
            sys.stderr.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
        if r.returncode:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stderr}")
    with cf.ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fPIC"]
        run(cmd)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
