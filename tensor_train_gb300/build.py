"""Compile libttgpu.so (sm_103a) in-tree with nvcc.

Translation units compiled in parallel, one -gencode, no cmake.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libttgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC"]

SOURCES = ["ttg_kernels.cu", "ttg_wide.cu", "ttg_api.cpp", "ttg_host.cpp", "ttg_noalloc.cu",
           "ttg_mlp.cu", "ttg_tc_gemm.cu", "ttg_shard.cpp"]
HEADERS = ["ttg_device.cuh", "ttg_device_df.cuh", "ttg_df64.cuh", "ttg_job.h", "ttg_kernels.h",
           "ttg_tc.cuh", "ttg_sweep_common.cuh", "ttg_ozaki.cuh", "ttg_wy_df.cuh", "ttg_gemm_live.h"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    inc = os.path.join(os.path.dirname(HERE), "include")
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(inc, "ttg.h")]
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _stale(o, [s] + hdrs):
            jobs.append([nvcc, *ARCH, *COMMON, "-I", inc, "-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        subprocess.check_call(cmd)

    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(run, jobs))
    if force or jobs or _stale(LIB, objs):
        tmp = LIB + f".tmp{os.getpid()}"
        run([nvcc, "-shared", *ARCH, *objs, "-o", tmp])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
