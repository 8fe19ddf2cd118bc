"""Builds the native library nekbone_gb300/libnekbone_gb300.so for sm_103a.

Every translation unit is compiled in parallel with nvcc (one -gencode,
compute_103a -> sm_103a) and linked into one shared library with the C ABI
declared in include/nekbone_gb300.h.  Objects go to nekbone_gb300/_build/.

Usage:  python nekbone_gb300/build.py [--force] [--jobs N]
(run by path: importing the package requires the library this builds)
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libnekbone_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is built without floating-point contraction so that the set-up
# math (GLL points, derivative matrices, multigrid operators) rounds the same
# way on x86-64 and aarch64 (gcc contracts a*b+c into fma by default on
# aarch64).  Device code spells every fused multiply-add out explicitly.
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off",
              "--expt-relaxed-constexpr", "-Xptxas", "-warn-spills"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists() and not shutil.which(cand):
        raise RuntimeError("nvcc not found; the CUDA toolkit is required to build nekbone_gb300")
    return cand


def sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers_mtime() -> float:
    hs = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    return max((h.stat().st_mtime for h in hs), default=0.0)


def _compile(src: Path, force: bool) -> tuple[Path, str]:
    obj = BUILD / (src.name + ".o")
    if (not force and obj.exists() and obj.stat().st_mtime >= src.stat().st_mtime
            and obj.stat().st_mtime >= _headers_mtime()):
        return obj, ""
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)]
    if src.suffix == ".cpp":
        cmd = [nvcc(), "-x", "cu", *ARCH, *NVCC_FLAGS, "-I", str(ROOT / "include"), "-c", str(src),
               "-o", str(obj)]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    return obj, p.stderr


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        results = list(ex.map(lambda s: _compile(s, force), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for o, err in results:
            if err.strip():
                print(f"[{o.name}]\n{err}", file=sys.stderr)
    newest = max(o.stat().st_mtime for o in objs)
    if force or not LIB.exists() or LIB.stat().st_mtime < newest:
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
        os.replace(tmp, LIB)
    build_driver(force)
    return LIB


DRIVER_SRC = PKG / "driver" / "nekbone.cpp"
DRIVER = PKG / "bin" / "nekbone"


def build_driver(force: bool = False) -> Path:
    """The reference's driver program over the C ABI (host C++ only)."""
    DRIVER.parent.mkdir(exist_ok=True)
    if (not force and DRIVER.exists() and DRIVER.stat().st_mtime >= LIB.stat().st_mtime
            and DRIVER.stat().st_mtime >= DRIVER_SRC.stat().st_mtime):
        return DRIVER
    cxx = os.environ.get("CXX") or shutil.which("g++") or "g++"
    cmd = [cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(ROOT / "include"),
           "-o", str(DRIVER), str(DRIVER_SRC), "-L", str(PKG), "-lnekbone_gb300",
           "-Wl,-rpath,$ORIGIN/.."]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"driver build failed: {' '.join(cmd)}\n{p.stdout}\n{p.stderr}")
    return DRIVER


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--jobs", type=int, default=None)
    ap.add_argument("-v", "--verbose", action="store_true")
    a = ap.parse_args()
    print(build(force=a.force, jobs=a.jobs, verbose=a.verbose))


if __name__ == "__main__":
    main()
