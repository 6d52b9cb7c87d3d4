"""Build the native parts of axbc_gb300 in-tree with nvcc (sm_103a only).

Outputs (git-ignored):
  axbc_gb300/libaxbc_gb300.so   the C-ABI library (include/axbc.h, include/axbc_compat.h)
  axbc_gb300/axbc               the command-line driver (the reference's CLI surface)

Usage: python -m axbc_gb300.build [--force] [--verbose]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libaxbc_gb300.so")
CLI = os.path.join(HERE, "axbc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xcompiler", "-Wno-unused-function", "-I", os.path.join(ROOT, "include")]
LIB_SOURCES = ["api.cu", "graph.cu", "single.cu", "batch.cu", "sampler.cu", "serve.cu", "compat.cu",
               "tune.cu", "noalloc.cu", "kron.cu", "host_graph.cpp"]
# the Graph500 generator's binomial draws round every product and sum apart,
# as the host code they restate does
FILE_FLAGS = {"kron.cu": ["-fmad=false"]}
CLI_SOURCES = ["cli.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build axbc_gb300")


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def _compile(src: str, force: bool, verbose: bool) -> str:
    out = os.path.join(OBJ, os.path.basename(src) + ".o")
    deps = [src] + _headers()
    if not force and not _stale(out, deps):
        return out
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, *FILE_FLAGS.get(os.path.basename(src), []), "-c", src, "-o", out]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++", *NVCC_FLAGS, "-c", src, "-o", out]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr.strip():
        print(r.stderr, file=sys.stderr)
    return out


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = [os.path.join(CSRC, s) for s in LIB_SOURCES]
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, force, verbose), srcs))
    if force or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fPIC"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    cli_src = [os.path.join(CSRC, s) for s in CLI_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    if cli_src and (force or _stale(CLI, cli_src + [LIB])):
        cmd = ["g++", "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), *cli_src,
               "-o", CLI, "-L", HERE, "-laxbc_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"CLI build failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose="--verbose" in sys.argv)
    print(LIB)
