"""Build libwavedm.so in-tree with nvcc for sm_103a (no cmake, parallel TUs).

    python wavedm.jl_gb300/build.py            # build if sources are newer
    python wavedm.jl_gb300/build.py --force    # rebuild everything

The library lands next to this file (``wavedm.jl_gb300/libwavedm.so``); the
object files go to ``wavedm.jl_gb300/_build/``.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwavedm.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
         "-Xptxas", "-O3", "-I", CSRC, "-I", INCLUDE]


def nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libwavedm")


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(INCLUDE, "wavedm.h"))
    return hs


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def needs_build():
    if not os.path.exists(LIB):
        return True
    return _newest(sources() + headers()) > os.path.getmtime(LIB)


def _compile(src, verbose=False, extra=(), build_dir=BUILD):
    obj = os.path.join(build_dir, os.path.basename(src)[:-3] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and (r.stdout or r.stderr):
        print(r.stdout + r.stderr, file=sys.stderr)
    return obj


def build(force=False, verbose=False, ptxas_info=False, defines=(), out=None):
    """Compile every csrc/*.cu for sm_103a and link libwavedm.so; returns its path.

    ``defines`` (e.g. ["WDM_X_MINB=6"]) and ``out`` build a tuning variant of
    the library at another path, with objects in a directory beside it.
    """
    lib = os.path.abspath(out) if out else LIB
    if not force and not defines and out is None and not needs_build():
        return LIB
    build_dir = BUILD if out is None else lib + ".objs"
    os.makedirs(build_dir, exist_ok=True)
    extra = tuple(("-Xptxas", "-v") if ptxas_info else ()) + tuple("-D" + d for d in defines)
    srcs = sources()
    workers = min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(workers) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose or ptxas_info, extra, build_dir), srcs))
    tmp = lib + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib)
    return lib


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas-info", action="store_true", help="print registers/spills per kernel")
    ap.add_argument("--define", "-D", action="append", default=[], help="extra preprocessor define (variant build)")
    ap.add_argument("--out", default=None, help="output path of a variant library")
    a = ap.parse_args()
    print(build(force=a.force or a.ptxas_info, verbose=True, ptxas_info=a.ptxas_info, defines=a.define, out=a.out))
