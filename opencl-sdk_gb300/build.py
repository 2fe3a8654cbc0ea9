"""Builds libgbcompute.so in-tree: every CUDA/C++ source compiled for sm_103a
only, in parallel, then linked into one shared library with the CUDA runtime
linked statically (the library loads on a machine without a GPU; the C ABI
then reports no device).

Usage: python opencl-sdk_gb300/build.py [-v] [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbcompute.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

SOURCES = [
    "runtime.cpp",
    "capi.cpp",
    "autotune.cpp",
    "elementwise.cu",
    "sort.cu",
    "scan.cu",
    "reduce.cu",
    "histogram.cu",
    "segmented.cu",
    "segscan.cu",
    "learned.cu",
    "reduce_by_key.cu",
    "select.cu",
    "transform.cu",
    "bitpack.cu",
    "static_map.cu",
]

COMMON = [
    "-O3",
    "-std=c++17",
    "-lineinfo",
    "-Xcompiler",
    "-fPIC,-fvisibility=hidden,-Wall,-Wno-unused-function",
    "--expt-relaxed-constexpr",
    "-I" + CSRC,
]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build gbcompute")


def _headers_digest() -> str:
    h = hashlib.sha256()
    for name in sorted(os.listdir(CSRC)):
        if name.endswith((".hpp", ".cuh", ".h")):
            with open(os.path.join(CSRC, name), "rb") as f:
                h.update(name.encode() + f.read())
    with open(os.path.join(HERE, "..", "include", "compute_c.h"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(COMMON + ARCH).encode())
    return h.hexdigest()[:16]


def _compile(src: str, force: bool, digest: str, verbose: bool) -> str:
    path = os.path.join(CSRC, src)
    obj = os.path.join(OUT_DIR, src + "." + digest + ".o")
    if not force and os.path.exists(obj) and os.path.getmtime(obj) >= os.path.getmtime(path):
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else []
    cmd = [nvcc()] + COMMON + ARCH + lang + ["-c", path, "-o", obj]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, flush=True)
    return obj


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    digest = _headers_digest()
    workers = min(len(SOURCES), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, digest, verbose), SOURCES))
    # objects of earlier header digests are never used again
    keep = {os.path.basename(o) for o in objs}
    for name in os.listdir(OUT_DIR):
        if name.endswith(".o") and name not in keep:
            os.remove(os.path.join(OUT_DIR, name))
    newest = max(os.path.getmtime(o) for o in objs)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < newest:
        tmp = LIB + ".tmp"
        cmd = [nvcc(), "-shared", "-o", tmp] + ARCH + objs + ["-cudart", "static", "-lpthread", "-ldl", "-lrt"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
