"""Builds libspkgpu.so (the C-ABI library with the sm_103a kernels) in-tree.

Each translation unit is compiled by nvcc in parallel for sm_103a only, then
linked into ``spparks_gb300/_lib/libspkgpu.so``.  Rebuilds only what changed.
"""

from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
OBJ = OUT / "obj"
LIB = OUT / "libspkgpu.so"
INCLUDE = PKG.parent / "include"

SOURCES = [
    "spkgpu_api.cpp",
    "sweep_generic.cu",
    "sweep_fused2d.cu",
    "sweep_resident.cu",
    "kmc.cu",
    "ensemble.cu",
    "noalloc.cu",
    "packed.cu",
    "sweep_rows.cu",
    "diag.cu",
    "calib.cu",
    "driver.cpp",
]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              f"-I{INCLUDE}", f"-I{CSRC}"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or "/usr/local/cuda/bin/nvcc"
    return cand if Path(cand).exists() else "nvcc"


def _headers():
    return list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))


def _compile(src: str, verbose: bool) -> Path:
    s = CSRC / src
    o = OBJ / (src + ".o")
    newest_dep = max([s.stat().st_mtime] + [h.stat().st_mtime for h in _headers()])
    if o.exists() and o.stat().st_mtime >= newest_dep:
        return o
    cmd = [nvcc(), *ARCH, *NVCC_FLAGS, "-c", str(s), "-o", str(o) + ".tmp"]
    if src.endswith(".cu"):
        cmd.insert(1, "-Xptxas=-warn-spills")
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr.strip():
        print(res.stderr, file=sys.stderr)
    os.replace(str(o) + ".tmp", o)
    return o


def build(verbose: bool = False) -> Path:
    OBJ.mkdir(parents=True, exist_ok=True)
    srcs = [s for s in SOURCES if (CSRC / s).exists()]
    with ThreadPoolExecutor(max_workers=max(2, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if LIB.exists() and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return LIB
    tmp = OUT / f"libspkgpu.{os.getpid()}.so"
    cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-lcudart"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
