"""TEST INFRASTRUCTURE, NOT PRODUCT CODE: ctypes wrapper of the FP64 oracle.

``ctraj_oracle.c`` restates the reference's propagation path on the CPU (see
its header for the file:line map).  Only tests/, ``__graft_entry__.smoke()``
and bench.py's CPU-baseline leg import this module, and only as the checker
or the timed CPU baseline; the product path never calls it.

The oracle takes the same element / force-table structs as the CUDA library
(``include/ctraj.h``), produced by the product's beamline compiler, so a
fixture test exercises compiler + oracle against the reference's outputs.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SRC = HERE / "ctraj_oracle.c"
LIB = HERE / "_build" / "libctraj_oracle.so"
G = 9.80665  # scipy.constants.g, bound into molecule.py:15-16,58

CFLAGS = ["-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def build(force: bool = False) -> Path:
    """Compile the oracle with gcc (recipe also in oracle/Makefile)."""
    LIB.parent.mkdir(parents=True, exist_ok=True)
    hdr = HERE.parent / "include" / "ctraj.h"
    if force or not LIB.exists() or LIB.stat().st_mtime < max(SRC.stat().st_mtime, hdr.stat().st_mtime):
        tmp = LIB.with_suffix(".so.tmp")
        subprocess.run(["gcc", *CFLAGS, str(SRC), "-o", str(tmp), "-lm"], check=True)
        tmp.replace(LIB)
    return LIB


_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        lib = ctypes.CDLL(str(build()))
        P = ctypes.c_void_p
        lib.ctraj_oracle_run.restype = ctypes.c_int
        lib.ctraj_oracle_run.argtypes = [P, ctypes.c_int, P, ctypes.c_int, ctypes.c_double, P,
                                         ctypes.c_int64, ctypes.c_int, ctypes.c_int, P, P, P, P, P, P]
        lib.ctraj_oracle_trace.restype = ctypes.c_int64
        lib.ctraj_oracle_trace.argtypes = [P, ctypes.c_int, P, ctypes.c_int, ctypes.c_double, P, P,
                                           ctypes.c_int64, P]
        _lib = lib
    return _lib


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def run(compiled, ics: np.ndarray, g: float = G, threads: int = 1, outputs: bool = True) -> dict:
    """Propagate ics (6, n) float64 through a compiled beamline on the CPU."""
    lib = load()
    ics = np.ascontiguousarray(ics, dtype=np.float64)
    n = ics.shape[1]
    nl = len(compiled.labels)
    label = np.empty(n, np.int32) if outputs else None
    fin = np.empty((10, n)) if outputs else None
    rows = np.empty(n, np.int32) if outputs else None
    margin = np.empty(n) if outputs else None
    counts = np.zeros(nl + 1, np.int64)
    stats = np.zeros(5, np.int64)
    tabs = compiled.table_structs()
    status = lib.ctraj_oracle_run(ctypes.addressof(compiled.elements), compiled.n_elements,
                                  ctypes.addressof(tabs), len(compiled.tables), g, _ptr(ics), n, nl,
                                  threads, _ptr(label), _ptr(fin), _ptr(rows), _ptr(margin),
                                  _ptr(counts), _ptr(stats))
    return dict(status=status, label=label, final=fin, rows=rows, margin=margin, counts=counts,
                steps=int(stats[0]), lens_steps=int(stats[1]), edge_band=int(stats[2]),
                table_range=int(stats[3]), errors=int(stats[4]))


def trace(compiled, ic, g: float = G, max_rows: int = 100000):
    """All stored rows (including the initial one) of one molecule: (rows (k, 10), label)."""
    lib = load()
    ic = np.ascontiguousarray(ic, dtype=np.float64)
    out = np.empty((max_rows, 10))
    lab = np.zeros(1, np.int32)
    tabs = compiled.table_structs()
    k = lib.ctraj_oracle_trace(ctypes.addressof(compiled.elements), compiled.n_elements,
                               ctypes.addressof(tabs), len(compiled.tables), g, _ptr(ic), _ptr(out),
                               max_rows, _ptr(lab))
    return out[:min(k, max_rows)].copy(), int(lab[0])
