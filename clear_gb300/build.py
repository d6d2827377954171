"""Compile the CUDA sources into ``clear_gb300/libclear_gb300.so`` (sm_103a).

Each ``csrc/*.cu`` (nvcc) and host-only ``csrc/*.cpp`` (the host compiler) is
compiled to an object in parallel, then linked into one
shared library whose exported symbols are the C ABI of
``include/clear_cuda.h``.  Only nvcc and the host compiler are needed.
"""
from __future__ import annotations

import os
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libclear_gb300.so"
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = [
    *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    # The reference's arithmetic is defined without fused multiply-add and with
    # IEEE division/sqrt; the kernels also spell that out with __f*_rn.
    "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
    f"-I{ROOT / 'include'}", f"-I{CSRC}",
]


CXX = os.environ.get("CXX", "g++")
# Host-only sources (no device code): the host compiler directly.
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-fvisibility=hidden", f"-I{ROOT / 'include'}", f"-I{CSRC}"]


def _sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted((ROOT / "include").glob("*.h"))


def _compile(src: Path) -> Path:
    obj = BUILD / (src.stem + ".o")
    deps = [src, *_headers(), Path(__file__)]
    if obj.exists() and all(obj.stat().st_mtime >= d.stat().st_mtime for d in deps):
        return obj
    if src.suffix == ".cpp":
        cmd = [CXX, *CXX_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = [NVCC, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"{cmd[0]} failed for {src.name}:\n{res.stderr}")
    return obj


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    srcs = _sources()
    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    if not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-Xcompiler", "-fPIC", *map(str, objs), "-o", str(LIB), "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed:\n{res.stderr}")
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(verbose=True)
