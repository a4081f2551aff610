"""Build the CUDA library ``libfdtd_gb300.so`` in-tree with nvcc (sm_103a only).

Each ``csrc/*.cu`` compiles to an object in parallel, then nvcc links them
into ``simulation_gb300/_build/libfdtd_gb300.so`` (CUDA runtime linked
statically, so the library needs only the driver at run time).  A stamp of
the sources and flags skips the build when nothing changed.

    python -m simulation_gb300.build [--force] [--debug]
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.environ.get("FDTD_BUILD_DIR", os.path.join(PKG, "_build"))
LIB = os.path.join(OUT, "libfdtd_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
         "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libfdtd_gb300.so")


def _sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stamp(flags: list[str]) -> str:
    h = hashlib.sha256()
    for f in sorted(os.listdir(CSRC)) + ["../../include/fdtd.h"]:
        p = os.path.normpath(os.path.join(CSRC, f))
        if os.path.isfile(p):
            h.update(f.encode())
            with open(p, "rb") as fh:
                h.update(fh.read())
    h.update(" ".join(flags).encode())
    h.update(os.uname().machine.encode())
    return h.hexdigest()


def build(force: bool = False, debug: bool = False, verbose: bool = False) -> str:
    flags = FLAGS + (["-DFDTD_BOUNDS_CHECK"] if debug else [])
    flags += os.environ.get("FDTD_NVCC_EXTRA", "").split()
    os.makedirs(OUT, exist_ok=True)
    stamp_path = os.path.join(OUT, "stamp.txt")
    stamp = _stamp(flags)
    if not force and os.path.exists(LIB) and os.path.exists(stamp_path):
        with open(stamp_path) as fh:
            if fh.read().strip() == stamp:
                return LIB
    cc = nvcc()
    srcs = _sources()
    objs = [os.path.join(OUT, os.path.basename(s)[:-3] + ".o") for s in srcs]

    def compile_one(src_obj):
        src, obj = src_obj
        cmd = [cc] + ARCH + flags + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr.strip():
            sys.stderr.write(r.stderr)
        return obj

    workers = max(1, min(len(srcs), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(workers) as ex:
        list(ex.map(compile_one, zip(srcs, objs)))
    tmp = LIB + ".tmp"
    cmd = [cc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp_path, "w") as fh:
        fh.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, debug="--debug" in sys.argv, verbose=True))
