"""Compile libgbhf.so (CUDA sources in ../csrc) for sm_103a with nvcc.

Each translation unit is compiled in parallel, then linked into
``gbhf/_build/libgbhf.so``.  No CMake, no PyTorch extension machinery: the
library exposes a plain C ABI (include/gbhf.h).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libgbhf.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cu", "setup.cu", "eri_canon.cu", "jk.cu", "linalg.cu", "scf.cu", "measure.cu", "noalloc.cu", "grad.cu", "batch.cu",
           "sad.cu", "bscf.cu", "jkd.cu", "gradd.cu", "uhf.cu",
           "tune.cu", "tridiag.cu"]
HEADERS = ["gbhf_common.cuh", "gbhf_internal.h", "gbhf_md.cuh", "eri_gen.cuh", "grad_gen.cuh", "jacobi.cuh",
           "dense.cuh", "mdwarp.cuh"]


def nvcc():
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra=()):
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                   "-I", str(CSRC), "-I", str(PKG.parent.parent / "include")] + list(extra)


def _stale():
    if not LIB.exists():
        return True
    t = LIB.stat().st_mtime
    deps = [CSRC / s for s in SOURCES + HEADERS] + [PKG.parent.parent / "include" / "gbhf.h"]
    return any(d.stat().st_mtime > t for d in deps if d.exists())


def build(force=False, verbose=False, extra_flags=()):
    """Build libgbhf.so if any source is newer; returns its path."""
    if not force and not _stale():
        return LIB
    BUILD.mkdir(exist_ok=True)
    cc = nvcc()

    def compile_one(src):
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [cc, "-c", str(CSRC / src), "-o", str(obj)] + _flags(extra_flags)
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, SOURCES))
    objs = [str(o) for o, _ in results]
    tmp = BUILD / f"libgbhf.so.tmp{os.getpid()}"
    cmd = [cc, "-shared", "-o", str(tmp)] + objs + ARCH + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose=True))
