"""The FP32 soft-transmission kernels and the lens kernels' linear-table
lookups locate a molecule's table interval without the float-to-integer
conversion unit (table_interval in
csrc/molecule.cuh); the interval and the offset in it must equal, bit for
bit, what the truncating conversion and its inverse give, for every kind of
argument."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("last", [0, 15, 4094, 6143, 16379])
def test_table_interval_equals_the_conversions(last):
    from bench_kernels.build import build as build_probes

    lib = ctypes.CDLL(str(build_probes()))
    lib.ctraj_peak_interval_check.restype = ctypes.c_int
    lib.ctraj_peak_interval_check.argtypes = [ctypes.c_longlong, ctypes.c_uint,
                                              ctypes.POINTER(ctypes.c_ulonglong)]
    bad = ctypes.c_ulonglong(1)
    assert lib.ctraj_peak_interval_check(40_000_000, last, ctypes.byref(bad)) == 0
    assert bad.value == 0
