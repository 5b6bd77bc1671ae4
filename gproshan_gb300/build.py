"""Build libgp_ptp.so in-tree with nvcc for sm_103a (GB300).

Every translation unit is compiled in parallel, then linked into
``gproshan_gb300/libgp_ptp.so``.  Nothing is installed: the library is loaded
from this directory by ``gproshan_gb300._capi``.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgp_ptp.so")
STAMP = LIB + ".stamp"  # fingerprint of what LIB was built from (see _fingerprint)

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
              "--expt-relaxed-constexpr"]
SOURCES = ["gp_mesh.cu", "gp_toplesets.cu", "gp_ptp.cu", "gp_mlp.cu", "gp_capi.cpp", "gp_off.cpp"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgp_ptp.so")


def _compile(src: str, verbose_ptxas: bool) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-I", os.path.join(HERE, "..", "include"), "-c",
           os.path.join(CSRC, src), "-o", obj]
    if verbose_ptxas and src.endswith(".cu"):
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    if verbose_ptxas:
        sys.stderr.write(r.stderr)
    return obj


def _fingerprint() -> str:
    """sha256 of everything the library is built from: every source under
    csrc/, the public header, this script (flags and source list), the nvcc
    version and the machine type."""
    h = hashlib.sha256()
    files = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC))
    files += [os.path.join(HERE, "..", "include", "gp_ptp.h"), os.path.abspath(__file__)]
    for p in files:
        if os.path.isfile(p):
            h.update(os.path.basename(p).encode())
            with open(p, "rb") as f:
                h.update(f.read())
    r = subprocess.run([nvcc(), "--version"], capture_output=True, text=True)
    h.update(r.stdout.encode())
    h.update(platform.machine().encode())
    return h.hexdigest()


def _stale(fp: str) -> bool:
    """The library is rebuilt unless it exists beside a stamp holding the
    fingerprint of the sources, flags, toolchain and machine it came from (a
    copy built elsewhere, or from other sources, is never reused)."""
    if not os.path.exists(LIB) or not os.path.exists(STAMP):
        return True
    with open(STAMP) as f:
        return f.read().strip() != fp


def build(force: bool = False, verbose_ptxas: bool = False) -> str:
    """Compile libgp_ptp.so unless its stamp matches the current fingerprint;
    return its path."""
    fp = _fingerprint()
    if not force and not _stale(fp):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose_ptxas), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(fp + "\n")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    print(LIB)
