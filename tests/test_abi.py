"""C ABI checks that need no GPU: the library loads, exports every function
declared in include/ctraj.h, and the ctypes structs match the C layout."""
import ctypes
import re
import subprocess
import tempfile
from pathlib import Path

import pytest

from ctraj import _abi

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "ctraj.h"


def declared_functions():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:int|const char\*|int64_t)\s+(ctraj_\w+)\s*\(", text, flags=re.M)))


def test_header_functions_are_bound():
    names = declared_functions()
    assert "ctraj_run" in names and "ctraj_create" in names
    assert set(names) == set(_abi.SIGNATURES), set(names) ^ set(_abi.SIGNATURES)


@pytest.fixture(scope="module")
def lib():
    from ctraj.build import build_library

    build_library()
    return ctypes.CDLL(str(_abi.LIB_PATH))


def test_library_exports_every_declared_symbol(lib):
    for name in declared_functions():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", str(_abi.LIB_PATH)], capture_output=True,
                         text=True).stdout
    exported = set(re.findall(r"\b(ctraj_\w+)\b", out))
    assert set(declared_functions()) <= exported


def test_version_and_error_without_gpu(lib):
    lib.ctraj_version.restype = ctypes.c_int
    assert lib.ctraj_version() == _abi.ABI_VERSION
    lib.ctraj_last_error.restype = ctypes.c_char_p
    assert isinstance(lib.ctraj_last_error(), bytes)


def test_struct_layout_matches_header():
    src = r"""
    #include <stdio.h>
    #include <stddef.h>
    #include "ctraj.h"
    int main(void) {
      printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\n", sizeof(ctraj_element), sizeof(ctraj_force_table),
             sizeof(ctraj_distribution), sizeof(ctraj_run_args), sizeof(ctraj_run_stats),
             sizeof(ctraj_tuning), sizeof(ctraj_sweep), sizeof(ctraj_soft_args),
             sizeof(ctraj_soft_result), sizeof(ctraj_ring_entry), sizeof(ctraj_ring));
      printf("%zu %zu %zu %zu\n", offsetof(ctraj_element, z0), offsetof(ctraj_element, p),
             offsetof(ctraj_run_args, g), offsetof(ctraj_run_args, counts));
      return 0;
    }
    """
    with tempfile.TemporaryDirectory() as d:
        c = Path(d) / "s.c"
        c.write_text(src)
        exe = Path(d) / "s"
        subprocess.run(["gcc", f"-I{ROOT / 'include'}", str(c), "-o", str(exe)], check=True)
        sizes, offs = subprocess.run([str(exe)], capture_output=True, text=True).stdout.split("\n")[:2]
    assert list(map(int, sizes.split())) == [ctypes.sizeof(_abi.Element), ctypes.sizeof(_abi.ForceTable),
                                            ctypes.sizeof(_abi.Distribution), ctypes.sizeof(_abi.RunArgs),
                                            ctypes.sizeof(_abi.RunStats), ctypes.sizeof(_abi.Tuning),
                                            ctypes.sizeof(_abi.Sweep), ctypes.sizeof(_abi.SoftArgs),
                                            ctypes.sizeof(_abi.SoftResult), ctypes.sizeof(_abi.RingEntry),
                                            ctypes.sizeof(_abi.Ring)]
    assert list(map(int, offs.split())) == [_abi.Element.z0.offset, _abi.Element.p.offset,
                                           _abi.RunArgs.g.offset, _abi.RunArgs.counts.offset]


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError, match="not built"):
        _abi.load_library(tmp_path / "nope.so")


def _noalloc_call(lib, cb, n, precision=32):
    """ctraj_run_noalloc with device draws; returns (status, message)."""
    from ctraj.distributions import device_spec
    from ctraj.workloads import source

    a = _abi.RunArgs()
    a.n, a.precision, a.g, a.ic_mode = n, precision, 9.80665, _abi.IC_DEVICE_DRAW
    a.xdist, a.vdist = (device_spec(d, r) for d, r in zip(source(), ("position", "velocity")))
    counts = (ctypes.c_int64 * (len(cb.labels) + 1))()
    a.counts = ctypes.addressof(counts)
    st = _abi.RunStats()
    tabs = cb.table_structs()
    status = lib.ctraj_run_noalloc(cb.elements, cb.n_elements, len(cb.labels), tabs, len(cb.tables),
                                   ctypes.byref(a), None, ctypes.byref(st))
    return status, lib.ctraj_last_error().decode()


def test_noalloc_rejects_what_its_scratch_cannot_hold_before_any_cuda_call():
    """Sizes beyond the allocation-free entry point's fixed scratch are refused
    with CTRAJ_EINVAL and a clear message, without touching the GPU (this runs
    on machines without one)."""
    import numpy as np
    from scipy.interpolate import interp1d

    import ctraj
    from ctraj.compiler import compile_beamline
    from ctraj.workloads import lens_beamline

    lib = _abi.load_library()
    lib.ctraj_last_error.restype = ctypes.c_char_p
    cb = compile_beamline(lens_beamline())
    st, msg = _noalloc_call(lib, cb, _abi.NOALLOC_MAX_MOLECULES + 1)
    assert st == _abi.EINVAL and "at most" in msg
    st, msg = _noalloc_call(lib, cb, 1000, precision=64)
    assert st == _abi.EINVAL and "precision 32" in msg
    # a radial table of more knot intervals than the scratch's table entries
    r = np.linspace(0.0, 0.02, _abi.NOALLOC_MAX_INTERVALS + 2)
    lens = ctraj.ElectrostaticLens(name="ES lens", z0=0.8, L=0.6, d=0.035, dz=1e-3,
                                   a_interp=interp1d(r, -1e3 * r))
    big = compile_beamline(ctraj.Beamline([lens]))
    st, msg = _noalloc_call(lib, big, 1000)
    assert st == _abi.EINVAL and "scratch holds at most" in msg, msg
