"""Build libctraj.so with nvcc for sm_103a (GB300), in-tree.

    python -m ctraj.build            # from centrex-molecule-trajectories_gb300/

The library is a plain shared object with a C ABI (include/ctraj.h), linked
against the static CUDA runtime, so it needs no PyTorch at build or load time.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG.parent / "csrc"
INCLUDE = PKG.parent.parent / "include"
OUT = PKG / "_lib" / "libctraj.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xptxas", "-warn-spills"]
OBJ = PKG / "_lib" / "obj"


def sources():
    return sorted(CSRC.glob("*.cu"))


def headers():
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def nvcc() -> str:
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(exe).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libctraj.so")
    return exe


def _newest_dependency() -> float:
    return max(p.stat().st_mtime for p in headers() + [Path(__file__)])


def up_to_date() -> bool:
    if not OUT.exists():
        return False
    t = OUT.stat().st_mtime
    return all(p.stat().st_mtime <= t for p in sources() + headers() + [Path(__file__)])


def build_library(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> Path:
    """Every translation unit compiled to an object in parallel (one nvcc each),
    then linked into the shared library; an object is rebuilt when its source,
    any header or this script is newer."""
    from concurrent.futures import ThreadPoolExecutor

    if not force and up_to_date():
        return OUT
    OBJ.mkdir(parents=True, exist_ok=True)
    dep = _newest_dependency()
    jobs = []
    for src in sources():
        obj = OBJ / (src.stem + ".o")
        if force or not obj.exists() or obj.stat().st_mtime < max(dep, src.stat().st_mtime):
            tmp = obj.with_name(obj.name + f".tmp{os.getpid()}")
            jobs.append(([nvcc(), *ARCH, *NVCC_FLAGS, f"-I{INCLUDE}", f"-I{CSRC}", *(extra or []), "-c", str(src),
                          "-o", str(tmp)], tmp, obj))

    def compile_one(job):
        cmd, tmp, obj = job
        if verbose:
            print(" ".join(cmd), flush=True)
        subprocess.run(cmd, check=True)
        tmp.replace(obj)

    with ThreadPoolExecutor(max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for f in [ex.submit(compile_one, j) for j in jobs]:
            f.result()
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_name(OUT.name + f".tmp{os.getpid()}")
    link = [nvcc(), *ARCH, "-shared", *[str(OBJ / (s.stem + ".o")) for s in sources()], "-o", str(tmp)]
    if verbose:
        print(" ".join(link), flush=True)
    subprocess.run(link, check=True)
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True,
                  extra=["-Xptxas", "-v"] if "-v" in sys.argv else None)
