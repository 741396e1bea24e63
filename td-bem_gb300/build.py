"""Build libtdbem.so (CUDA kernels + C ABI) for sm_103a, in-tree.

    python td-bem_gb300/build.py [--verbose] [--ptxas-info]

Each translation unit is compiled in parallel with nvcc and linked into
td-bem_gb300/_build/libtdbem.so.  Objects are rebuilt when a source or header
is newer.  No CMake, no torch extension machinery: plain nvcc.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
LIB = os.path.join(OUT, "libtdbem.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


RUN = os.path.join(OUT, "tdbem_run")
RUN_SRC = os.path.join(CSRC, "host", "tdbem_run.cpp")


def _sources():
    host = [p for p in glob.glob(os.path.join(CSRC, "host", "*.cpp")) if p != RUN_SRC]
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")) +
                  host)


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
            glob.glob(os.path.join(ROOT, "include", "*.h")) +
            glob.glob(os.path.join(ROOT, "include", "*.hpp")))


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _compile(src, verbose, ptxas_info):
    sub = "host_" if os.path.basename(os.path.dirname(src)) == "host" else ""
    obj = os.path.join(OUT, sub + os.path.splitext(os.path.basename(src))[0] + ".o")
    if not _stale(obj, [src] + _headers()) and not ptxas_info:
        return obj, ""
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + (["-Xptxas", "-v"] if ptxas_info else []) + \
        ["-c", src, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj, r.stderr


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        results = list(ex.map(lambda s: _compile(s, verbose, ptxas_info), srcs))
    objs = [o for o, _ in results]
    if ptxas_info:
        for _, log in results:
            sys.stderr.write(log)
    if _stale(LIB, objs):
        cuda_lib = os.path.join(os.path.dirname(os.path.dirname(os.path.realpath(nvcc()))), "lib64")
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + \
            ["-lcudart", "-lpthread", "-Xlinker", "-rpath=" + cuda_lib]
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
    # tdbem_run: main.cpp's sequence over the host classes, linked to the library
    if _stale(RUN, [RUN_SRC, LIB] + _headers()):
        cmd = [nvcc()] + ARCH + ["-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                                 RUN_SRC, "-o", RUN, "-L" + OUT, "-ltdbem", "-lcudart",
                                 "-Xlinker", "-rpath=$ORIGIN"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {RUN_SRC}:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--verbose", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true")
    a = ap.parse_args()
    print(build(a.verbose, a.ptxas_info))
