"""The FP32 on-device initial conditions draw their normals with branch-free
forms of log1p, the square root and sin / cos of pi a (philox.cuh:
log1p_atanh, sincospi_taylor, box_muller<float>), written from their series;
they must stay within a few ulp of the FP64 transform of the same Philox
words, as CUDA's own FP32 functions do (bench_kernels/box_muller_check.cu,
2^27 arguments: hashed words, every word at both ends of the two halves of
log U, even steps of the log1p and sincospi arguments)."""
import ctypes

import pytest

pytestmark = pytest.mark.gpu


def test_fp32_box_muller_is_within_a_few_ulp_of_fp64():
    from bench_kernels.build import build as build_probes

    lib = ctypes.CDLL(str(build_probes()))
    lib.ctraj_peak_bm_check.restype = ctypes.c_int
    lib.ctraj_peak_bm_check.argtypes = [ctypes.c_longlong, ctypes.POINTER(ctypes.c_float)]
    out = (ctypes.c_float * 6)()
    assert lib.ctraj_peak_bm_check(1 << 27, out) == 0
    normal, normal_libm, log1p, log1p_libm, sincospi, sincospi_libm = list(out)
    # a float ulp is 2^-23 = 1.19e-7 relative at most
    assert normal < 6e-7, normal            # |n32 - n64| / r64 (measured 3.5e-7; CUDA's functions 2.6e-7)
    assert log1p < 4e-7, log1p              # relative (measured 2.7e-7; log1pf 0.8e-7)
    assert sincospi < 2e-7, sincospi        # absolute (measured 0.8e-7; sincospif 0.5e-7)
    assert normal_libm < 6e-7 and log1p_libm < 4e-7 and sincospi_libm < 2e-7
