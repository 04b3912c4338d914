"""Builds the native library libresvg_gb300.so in-tree (resvg_gb300/_native/).

Host C++ is compiled with g++; CUDA sources with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``).  Translation units compile in
parallel and are linked with nvcc.  Floating-point contraction is disabled on
both sides (``-ffp-contract=off`` / ``--fmad=false``): the raster and filter
kernels reproduce the CPU restatement's f32 arithmetic operation by operation,
and an FMA would change the rounding.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_native")
LIB = os.path.join(OUT_DIR, "libresvg_gb300.so")
BUILD_DIR = os.path.join(OUT_DIR, "obj")

NVCC = os.environ.get("NVCC", shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
INCLUDES = ["-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
CXXFLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math", "-fwrapv", "-Wall",
            "-Wno-unused-function"]
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "--fmad=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-fwrapv",
           "-Xptxas", "-O3"] + ARCH


def _sources():
    srcs = []
    for sub in ("host", "kernels", ""):
        d = os.path.join(CSRC, sub)
        if not os.path.isdir(d):
            continue
        for f in sorted(os.listdir(d)):
            p = os.path.join(d, f)
            if os.path.isfile(p) and (f.endswith(".cpp") or f.endswith(".cu")):
                srcs.append(p)
    return srcs


def _headers_digest():
    h = hashlib.sha1()
    for d, _, files in os.walk(CSRC):
        for f in sorted(files):
            if f.endswith((".h", ".cuh")):
                with open(os.path.join(d, f), "rb") as fh:
                    h.update(fh.read())
    for f in sorted(os.listdir(os.path.join(ROOT, "include"))):
        with open(os.path.join(ROOT, "include", f), "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def _compile(src, hdr_digest):
    with open(src, "rb") as fh:
        digest = hashlib.sha1(fh.read() + hdr_digest.encode() + " ".join(NVFLAGS + CXXFLAGS).encode()).hexdigest()[:16]
    obj = os.path.join(BUILD_DIR, os.path.basename(src) + "." + digest + ".o")
    if os.path.exists(obj):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC, "-c", src, "-o", obj + ".tmp"] + NVFLAGS + INCLUDES
    else:
        cmd = ["g++", "-c", src, "-o", obj + ".tmp"] + CXXFLAGS + INCLUDES + ["-I/usr/local/cuda/include"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD_DIR, exist_ok=True)
    srcs = _sources()
    hd = _headers_digest()
    with cf.ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, hd), srcs))
    key = hashlib.sha1("".join(objs).encode()).hexdigest()[:16]
    stamp = LIB + ".stamp"
    if os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == key:
        return LIB
    cmd = [NVCC, "-shared", "-o", LIB + ".tmp"] + objs + ARCH + ["-lcudart", "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    os.replace(LIB + ".tmp", LIB)
    with open(stamp, "w") as fh:
        fh.write(key)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
