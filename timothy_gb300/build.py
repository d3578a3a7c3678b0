"""Build libtimothy_gb300.so in place (sm_103a only).

Every CUDA translation unit is compiled in parallel with nvcc, the C drop-in
layer with gcc, and everything is linked into timothy_gb300/libtimothy_gb300.so.
No CMake, no torch extension machinery: the library is a plain C-ABI shared
object.

    python -m timothy_gb300.build
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libtimothy_gb300.so")
# the reference-signature drop-ins as a static archive: a program links them
# as regular objects, so their definitions replace the reference's (weakened)
# ones, which a shared library's definitions cannot do
DROPIN_LIB = os.path.join(PKG, "libtimothy_gb300_dropin.a")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-I", INCLUDE, "-I", CSRC]
CC_FLAGS = ["-O2", "-fPIC", "-std=gnu11", "-ffp-contract=off", "-Wall", "-I", INCLUDE]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stderr


def _stale(out: str, deps) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(INCLUDE, "*.h"))
    jobs = []
    objs = []
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers) or ptxas_info:
            extra = ["-Xptxas", "-v"] if ptxas_info else []
            jobs.append([nvcc()] + ARCH + NVCC_FLAGS + extra + ["-c", src, "-o", obj])
    for src in sorted(glob.glob(os.path.join(CSRC, "*.c"))):
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if _stale(obj, [src] + headers):
            jobs.append(["gcc"] + CC_FLAGS + ["-c", src, "-o", obj])
    logs = []
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for err in ex.map(_run, jobs):
            logs.append(err)
    if jobs or not os.path.exists(LIB):
        _run([nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"])
    dropin_obj = os.path.join(BUILD, "tm_dropin.c.o")
    if jobs or not os.path.exists(DROPIN_LIB):
        if os.path.exists(DROPIN_LIB):
            os.remove(DROPIN_LIB)
        _run(["ar", "rcs", DROPIN_LIB, dropin_obj])
    if verbose or ptxas_info:
        for l in logs:
            if l:
                sys.stderr.write(l)
    return LIB


if __name__ == "__main__":
    build(verbose=True, ptxas_info="--ptxas" in sys.argv)
    print(LIB)
