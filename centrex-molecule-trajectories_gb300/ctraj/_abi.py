"""ctypes mirror of ``include/ctraj.h`` and the loader for ``libctraj.so``.

The structs here must match the header byte for byte; ``tests/test_abi.py``
checks the sizes and the exported symbol list without a GPU.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_DIR = PKG_DIR / "_lib"
LIB_PATH = LIB_DIR / "libctraj.so"

ABI_VERSION = 2

# status codes
OK = 0
EINVAL = -1
ECUDA = -2
ENOMEM = -3
ERANGE = -4
ESTEPS = -5
EOVERFLOW = -6
ESTATE = -7

MAX_ELEMENTS = 64
MAX_LABELS = 64
MAX_TABLES = 8
MAX_LENS_STEPS = 10_000_000

# element types
CIRCULAR_APERTURE = 1
RECTANGULAR_APERTURE = 2
FIELD_PLATES = 3
ELECTROSTATIC_LENS = 4
HONEYCOMB = 5

STEP_DZ = 0
STEP_DT = 1
RK4_REFERENCE = 0
RK4_CLASSIC = 1

TABLE_STARK_SPLINE = 1
TABLE_RADIAL_LINEAR = 2
TABLE_MESH = 3

DIST_NONE = 0
DIST_GAUSSIAN_POSITION = 1
DIST_DISC_POSITION = 2
DIST_GAUSSIAN_VELOCITY = 3

IC_DEVICE_DRAW = 0
IC_HOST = 1
IC_DEVICE = 2

OUT_NONE = 0
OUT_HOST = 1
OUT_DEVICE = 2

LABEL_DETECTED = -1


class Element(ctypes.Structure):
    _fields_ = [
        ("type", ctypes.c_int32),
        ("label", ctypes.c_int32),
        ("label_inside", ctypes.c_int32),
        ("table", ctypes.c_int32),
        ("step_mode", ctypes.c_int32),
        ("scheme", ctypes.c_int32),
        ("field_order", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("z0", ctypes.c_double),
        ("z1", ctypes.c_double),
        ("x0", ctypes.c_double),
        ("y0", ctypes.c_double),
        ("p", ctypes.c_double * 8),
    ]


class ForceTable(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("n_knots", ctypes.c_int32),
        ("knots", ctypes.POINTER(ctypes.c_double)),
        ("coef", ctypes.POINTER(ctypes.c_double)),
        ("values", ctypes.POINTER(ctypes.c_double)),
    ]


class Distribution(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("p", ctypes.c_double * 6),
    ]


class RunArgs(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("precision", ctypes.c_int32),
        ("ic_mode", ctypes.c_int32),
        ("ics", ctypes.c_void_p),
        ("xdist", Distribution),
        ("vdist", Distribution),
        ("seed", ctypes.c_uint64),
        ("offset", ctypes.c_uint64),
        ("g", ctypes.c_double),
        ("out_mode", ctypes.c_int32),
        ("timing", ctypes.c_int32),
        ("out_label", ctypes.c_void_p),
        ("out_final", ctypes.c_void_p),
        ("out_rows", ctypes.c_void_p),
        ("out_margin", ctypes.c_void_p),
        ("counts", ctypes.c_void_p),
    ]


class RunStats(ctypes.Structure):
    _fields_ = [
        ("molecules", ctypes.c_int64),
        ("molecule_steps", ctypes.c_int64),
        ("lens_steps", ctypes.c_int64),
        ("edge_band", ctypes.c_int64),
        ("table_range", ctypes.c_int64),
        ("bad_steps", ctypes.c_int64),
        ("kernels", ctypes.c_int32),
        ("timed", ctypes.c_int32),
        ("front_ms", ctypes.c_float),
        ("lens_ms", ctypes.c_float),
        ("max_lens_steps", ctypes.c_int32),
        ("linear_tables", ctypes.c_int32),
    ]


class Tuning(ctypes.Structure):
    _fields_ = [
        ("chunk_first", ctypes.c_int32),
        ("chunk_growth", ctypes.c_int32),
        ("chunk_max", ctypes.c_int32),
        ("front_waves", ctypes.c_int32),
        ("lens_mode", ctypes.c_int32),
        ("lens_interval", ctypes.c_int32),
        ("front_threads", ctypes.c_int32),
        ("batch_group", ctypes.c_int32),
        ("lens_threads", ctypes.c_int32),
        ("lens_molecules", ctypes.c_int32),
        ("batch_lens_threads", ctypes.c_int32),
        ("lens_service", ctypes.c_int32),
    ]


LENS_PERSISTENT = 0
LENS_CHUNKED = 1


class Sweep(ctypes.Structure):
    _fields_ = [
        ("n_configs", ctypes.c_int32),
        ("use_graph", ctypes.c_int32),
        ("n_molecules", ctypes.c_void_p),  # int64[n_configs]
        ("alpha", ctypes.c_void_p),        # double[n_configs]
        ("table", ctypes.c_void_p),        # int32[n_configs]
    ]


MAX_SWEEP_CONFIGS = 65536


class RingEntry(ctypes.Structure):
    _fields_ = [
        ("molecule", ctypes.c_int64),
        ("first_row", ctypes.c_uint64),
        ("rows", ctypes.c_int32),
        ("label", ctypes.c_int32),
    ]


class Ring(ctypes.Structure):
    _fields_ = [
        ("rows", ctypes.c_void_p),
        ("capacity_rows", ctypes.c_int64),
        ("index", ctypes.c_void_p),
        ("capacity_molecules", ctypes.c_int64),
        ("heads", ctypes.c_void_p),
        ("stride", ctypes.c_int32),
        ("lens", ctypes.c_int32),
    ]

SOFT_NPARAMS = 6
SOFT_V, SOFT_LENS_Z0, SOFT_APERTURE_R, SOFT_BORE_R, SOFT_SIGMA_VX, SOFT_SIGMA_VY = range(6)


class SoftArgs(ctypes.Structure):
    _fields_ = [
        ("n", ctypes.c_int64),
        ("precision", ctypes.c_int32),
        ("ic_mode", ctypes.c_int32),
        ("normals", ctypes.c_void_p),
        ("seed", ctypes.c_uint64),
        ("offset", ctypes.c_uint64),
        ("xdist", Distribution),
        ("vdist", Distribution),
        ("g", ctypes.c_double),
        ("width", ctypes.c_double),
        ("log_floor", ctypes.c_double),
        ("aperture", ctypes.c_int32),
        ("checkpoint", ctypes.c_int32),
        ("want_grad", ctypes.c_int32),
        ("timing", ctypes.c_int32),
    ]


class SoftResult(ctypes.Structure):
    _fields_ = [
        ("loss", ctypes.c_double),
        ("grad", ctypes.c_double * SOFT_NPARAMS),
        ("lens_molecules", ctypes.c_int64),
        ("lens_steps", ctypes.c_int64),
        ("dropped", ctypes.c_int64),
        ("bad_steps", ctypes.c_int64),
        ("kernels", ctypes.c_int32),
        ("timed", ctypes.c_int32),
        ("front_ms", ctypes.c_float),
        ("lens_ms", ctypes.c_float),
    ]

# Entry points declared in include/ctraj.h: name -> (restype, argtypes)
_P = ctypes.c_void_p
SIGNATURES = {
    "ctraj_version": (ctypes.c_int, []),
    "ctraj_last_error": (ctypes.c_char_p, []),
    "ctraj_create": (ctypes.c_int, [ctypes.c_int, ctypes.POINTER(_P)]),
    "ctraj_destroy": (ctypes.c_int, [_P]),
    "ctraj_set_stream": (ctypes.c_int, [_P, _P]),
    "ctraj_set_tuning": (ctypes.c_int, [_P, ctypes.POINTER(Tuning)]),
    "ctraj_get_tuning": (ctypes.c_int, [_P, ctypes.POINTER(Tuning)]),
    "ctraj_synchronize": (ctypes.c_int, [_P]),
    "ctraj_set_beamline": (ctypes.c_int, [_P, ctypes.POINTER(Element), ctypes.c_int32, ctypes.c_int32]),
    "ctraj_set_force_table": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(ForceTable)]),
    "ctraj_run": (ctypes.c_int, [_P, ctypes.POINTER(RunArgs), ctypes.POINTER(RunStats)]),
    "ctraj_run_batch": (ctypes.c_int, [_P, ctypes.POINTER(RunArgs), ctypes.c_int32, ctypes.POINTER(RunStats),
                                       ctypes.c_uint64]),
    "ctraj_record": (ctypes.c_int, [_P, ctypes.POINTER(RunArgs), _P, ctypes.c_int64, ctypes.c_int32,
                                    ctypes.c_int32, _P, _P]),
    "ctraj_run_sweep": (ctypes.c_int, [_P, ctypes.POINTER(Sweep), ctypes.POINTER(RunArgs), _P,
                                       ctypes.POINTER(RunStats)]),
    "ctraj_soft_transmission": (ctypes.c_int, [_P, ctypes.POINTER(SoftArgs), _P, ctypes.POINTER(SoftResult)]),
    "ctraj_run_ring": (ctypes.c_int, [_P, ctypes.POINTER(RunArgs), ctypes.POINTER(Ring), ctypes.POINTER(RunStats)]),
    "ctraj_plane": (ctypes.c_int, [_P, ctypes.POINTER(RunArgs), _P, ctypes.c_int64, ctypes.c_double, _P]),
    "ctraj_run_noalloc": (ctypes.c_int, [ctypes.POINTER(Element), ctypes.c_int32, ctypes.c_int32,
                                         ctypes.POINTER(ForceTable), ctypes.c_int32,
                                         ctypes.POINTER(RunArgs), _P, ctypes.POINTER(RunStats)]),
}

# ctraj_run_noalloc limits (include/ctraj.h)
NOALLOC_MAX_MOLECULES = 131072
NOALLOC_MAX_INTERVALS = 16384
MAX_BATCH_GROUP = 64
NOALLOC_SCRATCH_BYTES = 32 << 20


class CtrajError(RuntimeError):
    """A C-ABI call returned a non-zero status."""

    def __init__(self, status: int, message: str):
        super().__init__(f"ctraj status {status}: {message}")
        self.status = status


_lib = None


def load_library(path: os.PathLike | str | None = None) -> ctypes.CDLL:
    """Load libctraj.so (built by ``ctraj.build.build_library``).

    There is no CPU fallback: a missing library is an error.
    """
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} not found: the CUDA extension is not built. Run "
            "`python -c 'import __graft_entry__ as g; g.build()'` (needs nvcc).")
    lib = ctypes.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.ctraj_version() != ABI_VERSION:
        raise RuntimeError(f"libctraj ABI {lib.ctraj_version()} != {ABI_VERSION}")
    if path is None:
        _lib = lib
    return lib


def check(status: int, lib: ctypes.CDLL | None = None) -> None:
    """Map a C status to a Python exception, as the reference would raise."""
    if status == OK:
        return
    lib = lib or _lib
    msg = lib.ctraj_last_error().decode() if lib is not None else ""
    if status == ERANGE:
        raise ValueError(msg or "force table lookup above the interpolation range")
    if status == ESTEPS:
        raise OverflowError(msg or "lens step count is not finite")
    if status == EINVAL:
        raise ValueError(msg or "invalid argument")
    raise CtrajError(status, msg)


def f64ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
