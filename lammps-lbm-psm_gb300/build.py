"""In-tree build of liblbmpsm_gb300.so for sm_103a (nvcc, no cmake).

Each translation unit compiles in parallel; the FP64 units that must keep
the reference's operand order are compiled with -fmad=false.

    python lammps-lbm-psm_gb300/build.py [--force]
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liblbmpsm_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I",
          os.path.join(ROOT, "include")]
# units whose FP64 arithmetic must not be contracted into FMAs
NO_FMA = {"collide_f64", "particles", "layout"}
UNITS = ["collide_f64", "collide_lowp", "particles", "layout", "adjoint", "capi"]


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbmpsm_gb300.so")
    return exe


def _deps(unit: str) -> list[str]:
    return [os.path.join(CSRC, unit + ".cu"), os.path.join(CSRC, "lbmpsm_internal.cuh"),
            os.path.join(ROOT, "include", "lbmpsm.h")]


def _stale(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(unit: str, force: bool) -> str:
    src = os.path.join(CSRC, unit + ".cu")
    obj = os.path.join(BUILD, unit + ".o")
    if force or _stale(obj, _deps(unit)):
        cmd = [nvcc(), *ARCH, *COMMON, "-c", src, "-o", obj]
        if unit in NO_FMA:
            cmd.insert(1, "-fmad=false")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {unit}.cu:\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    units = [u for u in UNITS if os.path.exists(os.path.join(CSRC, u + ".cu"))]
    with cf.ThreadPoolExecutor(max_workers=len(units)) as ex:
        objs = list(ex.map(lambda u: _compile(u, force), units))
    if force or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    build_driver(force)
    return LIB


HOST = os.path.join(PKG, "host")
DRIVER = os.path.join(PKG, "lbmpsm_driver")


def build_driver(force: bool = False) -> str:
    """The C++ host side (host/lbmpsm_fix.cpp) and its standalone driver,
    linked against liblbmpsm_gb300.so (found next to the binary at run time)."""
    srcs = [os.path.join(HOST, f) for f in ("lbmpsm_fix.cpp", "lbmpsm_driver.cpp")]
    deps = srcs + [os.path.join(HOST, "lbmpsm_fix.h"), os.path.join(ROOT, "include", "lbmpsm.h"), LIB]
    if force or _stale(DRIVER, deps):
        cxx = shutil.which("g++") or "g++"
        cmd = [cxx, "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"), "-I", HOST,
               *srcs, "-o", DRIVER, "-L", PKG, "-llbmpsm_gb300", "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"host driver build failed:\n{r.stdout}\n{r.stderr}")
    return DRIVER


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
