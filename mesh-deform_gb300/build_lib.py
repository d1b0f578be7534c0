"""Builds libarap_gb300.so (the C ABI of include/arap_gpu.h) for sm_103a.

Six translation units compiled in parallel, then linked with the static CUDA
runtime:
  csrc/arap_kernels.cu   the sm_103a kernels (nvcc)
  csrc/arap_context.cu   context state and the C ABI (nvcc)
  csrc/arap_noalloc.cu   cotan weights with static scratch (nvcc)
  csrc/arap_batch.cu     many poses of one mesh in one pass (nvcc)
  csrc/arap_symbolic.cpp host symbolic analysis (g++)
  csrc/arap_server.cpp   the request scheduler of arap_srv_* (g++)
The library is built in-tree (next to this file) and is git-ignored.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
ROOT = PKG.parent
BUILD = PKG / "_build"
LIB = PKG / "libarap_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
                     f"-I{ROOT / 'include'}", "--expt-relaxed-constexpr"]
def cuda_include() -> str:
    return str(Path(nvcc()).resolve().parent.parent / "include")


GXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-pthread", f"-I{ROOT / 'include'}"]

SOURCES = [
    ("nvcc", CSRC / "arap_kernels.cu"),
    ("nvcc", CSRC / "arap_context.cu"),
    ("nvcc", CSRC / "arap_noalloc.cu"),
    ("nvcc", CSRC / "arap_batch.cu"),
    ("g++", CSRC / "arap_symbolic.cpp"),
    ("g++", CSRC / "arap_server.cpp"),
]
HEADERS = [CSRC / "arap_kernels.h", CSRC / "arap_symbolic.h", CSRC / "arap_device.cuh", CSRC / "arap_server.h",
           ROOT / "include" / "arap_gpu.h"]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _needs(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return any(p.stat().st_mtime > t for p in [src] + HEADERS)


def _compile(kind: str, src: Path, extra: list[str]) -> Path:
    obj = BUILD / (src.stem + ".o")
    if not _needs(obj, src):
        return obj
    if kind == "nvcc":
        cmd = [nvcc()] + NVCC_FLAGS + extra + ["-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++"] + GXX_FLAGS + [f"-I{cuda_include()}", "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    if r.stderr.strip():
        sys.stderr.write(r.stderr)
    return obj


def build(force: bool = False, verbose_ptxas: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    if force:
        for o in BUILD.glob("*.o"):
            o.unlink()
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    with ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda ks: _compile(ks[0], ks[1], extra), SOURCES))
    if LIB.exists() and not force and all(LIB.stat().st_mtime >= o.stat().st_mtime for o in objs):
        return LIB
    tmp = LIB.with_suffix(f".so.tmp{os.getpid()}")
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-Xcompiler", "-pthread", "-o", str(tmp)] + \
        [str(o) for o in objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))
