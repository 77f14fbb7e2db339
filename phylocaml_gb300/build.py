"""Builds libphylo_gpu.so in-tree with nvcc for sm_103a.

Every translation unit under ``csrc/`` is compiled in parallel to an object
file under ``_build/`` and linked into ``phylocaml_gb300/_lib/libphylo_gpu.so``.
Objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIBDIR = PKG / "_lib"
LIB = LIBDIR / "libphylo_gpu.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
    "--expt-relaxed-constexpr", "-I", str(INCLUDE),
]


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libphylo_gpu")
    return cand


def _sources() -> list[Path]:
    return sorted(list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cpp")))


def _headers() -> list[Path]:
    return sorted(list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h")))


def _stale(obj: Path, src: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return t < src.stat().st_mtime or t < newest_header


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compiles the CUDA library; returns the path of the shared object."""
    BUILD.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    cc = nvcc()
    hdr_t = max((h.stat().st_mtime for h in _headers()), default=0.0)
    srcs = _sources()
    objs = [BUILD / (s.name + ".o") for s in srcs]

    def compile_one(pair):
        src, obj = pair
        if not _stale(obj, src, hdr_t):
            return None
        cmd = [cc] + NVFLAGS + ["-c", str(src), "-o", str(obj)]
        if src.suffix == ".cpp":
            cmd = [cc, "-x", "cu"] + NVFLAGS + ["-c", str(src), "-o", str(obj)]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src.name}:\n{r.stdout}\n{r.stderr}")
        return r.stderr

    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with ThreadPoolExecutor(max_workers=max(jobs, 1)) as ex:
        for msg in ex.map(compile_one, zip(srcs, objs)):
            if verbose and msg:
                print(msg, flush=True)

    newest_obj = max(o.stat().st_mtime for o in objs)
    if not LIB.exists() or LIB.stat().st_mtime < newest_obj:
        cmd = [cc] + ARCH + ["-shared", "-o", str(LIB)] + [str(o) for o in objs] + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link of libphylo_gpu.so failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
