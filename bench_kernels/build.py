"""Build libctraj_probes.so: measurement probes for bench.py and the tests.

    python bench_kernels/build.py [--force]

Not part of the engine: an FMA-chain kernel that measures the FP32 peak (the
denominator of the lens pass's roofline fraction), the production FP32 lens
RK4 step in a loop (its one-warp latency and isolated throughput), and a check
of the lens kernels' table-interval arithmetic against the conversions it
replaces.  They include the engine's device headers, so they measure the code
the engine runs.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
CSRC = ROOT / "centrex-molecule-trajectories_gb300" / "csrc"
INCLUDE = ROOT / "include"
SRC = sorted(HERE.glob("*.cu"))
OUT = HERE / "_build" / "libctraj_probes.so"


def build(force: bool = False) -> Path:
    sys.path.insert(0, str(ROOT / "centrex-molecule-trajectories_gb300"))
    from ctraj.build import ARCH, headers, nvcc

    deps = SRC + headers() + [Path(__file__)]
    if not force and OUT.exists() and all(p.stat().st_mtime <= OUT.stat().st_mtime for p in deps):
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_name(OUT.name + f".tmp{os.getpid()}")
    subprocess.run([nvcc(), *ARCH, "-O3", "-std=c++17", "-Xcompiler", "-fPIC", "-shared", f"-I{INCLUDE}",
                    f"-I{CSRC}", *map(str, SRC), "-o", str(tmp)], check=True)
    tmp.replace(OUT)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
