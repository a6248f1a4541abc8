"""Build recipe for libcc3d_gpu.so (sm_103a).

Every translation unit under ../csrc is compiled by nvcc in parallel and
linked into cc3d_gb300/_lib/libcc3d_gpu.so.  A stamp file holding the hash of
the sources and flags makes repeated builds free.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
PROJECT = os.path.dirname(PKG)
CSRC = os.path.join(PROJECT, "csrc")
INCLUDE = os.path.join(os.path.dirname(PROJECT), "include")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libcc3d_gpu.so")
OBJDIR = os.path.join(PROJECT, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build cc3d_gb300")


def _sources():
    units = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    headers = sorted(f for f in os.listdir(CSRC) if f.endswith((".cuh", ".h")))
    return units, headers


def _stamp(units, headers) -> str:
    h = hashlib.sha256()
    for name in units + headers:
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(name.encode() + f.read())
    with open(os.path.join(INCLUDE, "cc3d_gpu.h"), "rb") as f:
        h.update(f.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    """Compile the library if its sources changed; return its path."""
    units, headers = _sources()
    stamp = _stamp(units, headers)
    stamp_file = os.path.join(LIBDIR, "libcc3d_gpu.stamp")
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read().strip() == stamp:
                return LIB
    os.makedirs(OBJDIR, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(unit):
        obj = os.path.join(OBJDIR, unit[:-3] + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-c", os.path.join(CSRC, unit), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    jobs = jobs or max(1, min(len(units), os.cpu_count() or 4))
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(compile_one, units))
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
