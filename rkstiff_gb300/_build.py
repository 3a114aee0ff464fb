"""Compile the CUDA sources of rkstiff_gb300 into an in-tree shared library.

``build()`` runs nvcc once per translation unit (in parallel) for sm_103a and links
``rkstiff_gb300/_lib/librkstiff_gb300.so``.  A stamp with the hash of the sources,
the compiler version and the host machine skips the work when nothing changed.
"""

from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIBNAME = "librkstiff_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rkstiff_gb300")


def _sources():
    cu = sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))
    deps = sorted(f for f in os.listdir(CSRC) if f.endswith((".cuh", ".h")))
    return cu, deps


def _stamp(nvcc: str) -> str:
    h = hashlib.sha256()
    cu, deps = _sources()
    for name in cu + deps:
        with open(os.path.join(CSRC, name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    for name in sorted(os.listdir(INCLUDE)):
        with open(os.path.join(INCLUDE, name), "rb") as f:
            h.update(name.encode() + b"\0" + f.read())
    ver = subprocess.run([nvcc, "--version"], capture_output=True, text=True).stdout
    h.update(ver.encode())
    h.update(platform.machine().encode())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False) -> str:
    """Build (if needed) and return the path of the shared library."""
    nvcc = _nvcc()
    stamp = _stamp(nvcc)
    stamp_file = os.path.join(LIBDIR, "build.stamp")
    if not force and os.path.exists(lib_path()) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read().strip() == stamp:
                return lib_path()
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cu, _ = _sources()

    def compile_one(name):
        obj = os.path.join(BUILD, name[:-3] + ".o")
        cmd = [nvcc, *ARCH, *NVCC_FLAGS, "-I", INCLUDE, "-c", os.path.join(CSRC, name), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        if verbose:
            print(f"[rkstiff_gb300] compiled {name}", file=sys.stderr)
        return obj

    workers = max(1, min(len(cu), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        objs = list(ex.map(compile_one, cu))
    tmp = lib_path() + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, lib_path())
    with open(stamp_file, "w") as f:
        f.write(stamp + "\n")
    if verbose:
        print(f"[rkstiff_gb300] linked {lib_path()}", file=sys.stderr)
    return lib_path()


if __name__ == "__main__":
    print(build(verbose=True, force="--force" in sys.argv))
