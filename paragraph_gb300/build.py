"""Builds paragraph_gb300/_lib/libparagraph_gb300.so with nvcc for sm_103a (in-tree).

Each translation unit compiles in its own process (in parallel), then one link step.  The
library is rebuilt only when a source or header is newer than it, and then only the objects
older than their source or a shared header are recompiled.
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
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libparagraph_gb300.so")
SOURCES = ["pg_api.cu", "pg_graph.cu", "pg_search.cu", "pg_screen.cu", "pg_prune_tc.cu",
           "pg_noalloc.cu", "pg_roar.cu", "pg_gt.cu"]
HEADERS = ["pg_device.cuh", "pg_kernels.h", "pg_tc.cuh"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "--expt-relaxed-constexpr"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in SOURCES + HEADERS]
    deps.append(os.path.join(ROOT, "include", "paragraph_gb300.h"))
    deps.append(__file__)
    return any(os.path.getmtime(p) > t for p in deps if os.path.exists(p))


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and not _stale():
        return LIB
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    extra = list(extra or [])
    objs = []

    common = [os.path.join(CSRC, f) for f in HEADERS]
    common += [os.path.join(ROOT, "include", "paragraph_gb300.h"), __file__]
    newest_common = max(os.path.getmtime(p) for p in common if os.path.exists(p))

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        if (not force and not extra and os.path.exists(obj)
                and os.path.getmtime(obj) > max(newest_common,
                                                os.path.getmtime(os.path.join(CSRC, src)))):
            return obj  # object newer than its source and every shared header
        cmd = [cc, *ARCH, *FLAGS, *extra, "-I", os.path.join(ROOT, "include"), "-c",
               os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + ".tmp"
    cudalib = os.path.join(os.path.dirname(os.path.dirname(cc)), "lib64")
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs, "-lcudart", "-Xlinker", "-rpath",
           "-Xlinker", cudalib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
