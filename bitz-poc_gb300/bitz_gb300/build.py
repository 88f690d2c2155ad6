"""In-tree build of the CUDA library (libbitzgpu.so) for sm_103a.

Each translation unit is compiled by nvcc in parallel into
``bitz-poc_gb300/build/`` and linked into ``bitz_gb300/libbitzgpu.so`` (both
paths are git-ignored).  Nothing here needs a GPU.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)                      # bitz-poc_gb300/
CSRC = os.path.join(ROOT, "csrc")
BUILD = os.path.join(ROOT, "build")
LIB = os.path.join(PKG, "libbitzgpu.so")
INCLUDE = os.path.join(os.path.dirname(ROOT), "include")

SOURCES = ["ntt.cu", "merkle.cu", "fold.cu", "runtime.cu", "batch.cu", "serve.cu", "pipeline.cu", "noalloc.cu",
           "transcript.cu", "pow.cu", "open.cu", "codec.cpp", "ligerito.cu",
           "pcs_open.cu", "ingest.cu", "shard.cu", "gkr.cu", "persist.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _deps() -> list[str]:
    out = []
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h", ".cpp")):
                out.append(os.path.join(d, f))
    return out


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-I", CSRC, "-I", INCLUDE, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def sources() -> list[str]:
    return [os.path.join(CSRC, s) for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]


def build(force: bool = False, extra: list[str] | None = None, verbose: bool = False) -> str:
    srcs = sources()
    newest = max(os.path.getmtime(p) for p in _deps())
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    if verbose:
        print("built", LIB)
    return LIB


def ptxas_report() -> str:
    """Register / shared-memory usage of every kernel (-Xptxas -v)."""
    lines = []
    for s in sources():
        cmd = [nvcc(), *ARCH, *FLAGS, "-Xptxas", "-v", "-I", CSRC, "-I", INCLUDE, "-c", s,
               "-o", os.devnull]
        r = subprocess.run(cmd, capture_output=True, text=True)
        lines.append(r.stderr)
    return "\n".join(lines)


if __name__ == "__main__":
    build(force=True, verbose=True)
