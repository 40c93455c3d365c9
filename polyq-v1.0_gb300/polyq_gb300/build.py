"""Build recipe for the in-tree native library (sm_103a only).

Two translation units compiled in parallel -- the host producer (g++) and the CUDA runtime
and kernels (nvcc, ``-gencode arch=compute_103a,code=sm_103a``) -- linked by nvcc into
``_lib/libpolyq_gb300.so`` with the CUDA runtime linked statically.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # polyq-v1.0_gb300/
REPO = os.path.dirname(ROOT)                     # repository root
CSRC = os.path.join(ROOT, "csrc")
INCLUDE = os.path.join(REPO, "include")
LIB_DIR = os.path.join(PKG, "_lib")
LIB_PATH = os.path.join(LIB_DIR, "libpolyq_gb300.so")
OBJ_DIR = os.path.join(ROOT, "_build")

GENCODE = "arch=compute_103a,code=sm_103a"
SOURCES_CU = ["pq_device.cu", "pq_peak.cu"]
SOURCES_CPP = ["pq_host.cpp"]
HEADERS = ["pq_core.cuh", "pq_kernels.cuh", "pq_host.hpp"]


def _nvcc() -> str:
    for p in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if p and (os.path.isabs(p) and os.path.exists(p) or not os.path.isabs(p)):
            return p
    return "nvcc"


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in SOURCES_CU + SOURCES_CPP + HEADERS]
    deps.append(os.path.join(INCLUDE, "polyq_gb300.h"))
    deps.append(os.path.abspath(__file__))
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(LIB_DIR, exist_ok=True)
    os.makedirs(OBJ_DIR, exist_ok=True)
    nvcc = _nvcc()
    inc = ["-I", INCLUDE, "-I", CSRC]
    jobs = []
    objs = []
    for f in SOURCES_CU:
        o = os.path.join(OBJ_DIR, f + ".o")
        objs.append(o)
        jobs.append([nvcc, "-std=c++17", "-O3", "-gencode", GENCODE, "-lineinfo", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-fvisibility=hidden", *inc, "-c", os.path.join(CSRC, f), "-o", o])
    for f in SOURCES_CPP:
        o = os.path.join(OBJ_DIR, f + ".o")
        objs.append(o)
        jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-fvisibility=hidden", "-pthread", *inc,
                     "-c", os.path.join(CSRC, f), "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))
    tmp = LIB_PATH + ".tmp%d" % os.getpid()
    run([nvcc, "-shared", "-gencode", GENCODE, "-Xcompiler", "-pthread", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
