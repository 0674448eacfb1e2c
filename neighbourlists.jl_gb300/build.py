"""Builds libnlgpu.so (the C-ABI library) for sm_103a with nvcc.

Each .cu translation unit is compiled in parallel, then linked into a shared
library next to this file.  Host code is compiled with -ffp-contract=off so
that the restated cell analysis rounds every operation like Julia does.
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
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libnlgpu.so")
SOURCES = ["nl_build.cu", "nl_pairs.cu", "nl_api.cu", "nl_static.cu", "nl_legacy.cu", "nl_f32.cu", "nl_query.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    p = shutil.which("nvcc")
    if p:
        return p
    for cand in ("/usr/local/cuda/bin/nvcc",):
        if os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnlgpu.so")


def flags(extra=()):
    return ARCH + [
        "-O3",
        "-lineinfo",
        "-std=c++17",
        "-Xcompiler", "-fPIC",
        "-Xcompiler", "-ffp-contract=off",
        "-Xcompiler", "-fno-fast-math",
        "-I", CSRC,
        "-I", INCLUDE,
        *extra,
    ]


def _headers_mtime() -> float:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cuh")]
    hs.append(os.path.join(INCLUDE, "nlgpu.h"))
    return max(os.path.getmtime(h) for h in hs)


def _compile(src: str, verbose: bool, ptxas_v: bool) -> str:
    obj = os.path.join(BUILD, src.replace(".cu", ".o"))
    extra = os.environ.get("NLGPU_EXTRA_FLAGS", "").split()
    cmd = [nvcc(), "-c", os.path.join(CSRC, src), "-o", obj] + flags(extra + (["-Xptxas", "-v"] if ptxas_v else []))
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose or ptxas_v:
        sys.stderr.write(r.stdout + r.stderr)
    return obj


def build(force: bool = False, verbose: bool = False, ptxas_v: bool = False) -> str:
    """Compiles libnlgpu.so when a source is newer.  NLGPU_EXTRA_FLAGS (e.g.
    "-DNL_EMIT_FLAT=1") rebuilds with extra compile flags, for trying the
    kernels' compile-time variants."""
    os.makedirs(BUILD, exist_ok=True)
    extra = os.environ.get("NLGPU_EXTRA_FLAGS", "").split()
    if extra:
        force = True
    newest = max(_headers_mtime(), *(os.path.getmtime(os.path.join(CSRC, s)) for s in SOURCES),
                 os.path.getmtime(__file__))
    if not force and not ptxas_v and os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose, ptxas_v), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), "-shared", "-o", tmp, *objs] + ARCH + ["-Xcompiler", "-fPIC", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True, ptxas_v="-v" in sys.argv)
    print(LIB)
