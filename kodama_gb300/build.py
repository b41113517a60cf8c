"""Build the CUDA library libkodama_gb300.so in-tree (kodama_gb300/_lib/).

nvcc compiles every translation unit for sm_103a only, in parallel, and links
one shared library exporting the C ABI of include/kodama_gb300.h.  Exact
float/double reproduction of the reference requires that no multiply-add is
contracted: device code is built with --fmad=false and host code with
-ffp-contract=off.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libkodama_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "evolve.cu", "kmeans.cu", "graph_ops.cu", "knn.cu", "knn_tc.cu", "noalloc.cu", "pls.cu", "mlp.cu", "plan.cu", "host_plan.cpp"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(src: str) -> list[str]:
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", CSRC]
    if src.endswith(".cu"):
        return ARCH + ["-lineinfo", "--fmad=false", "--expt-relaxed-constexpr"] + common
    return ["-x", "c++"] + common


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(HERE, "..", "include", "kodama_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT_DIR, src + ".o")
        objs.append(obj)
        if _stale(obj, path):
            jobs.append([nvcc] + _flags(src) + ["-c", path, "-o", obj])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=len(jobs)) as ex:
            results = list(ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs))
        for cmd, r in zip(jobs, results):
            if r.returncode != 0:
                raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
            if verbose and (r.stdout or r.stderr):
                print(r.stdout + r.stderr)
    if jobs or not os.path.exists(LIB):
        tmp = LIB + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
