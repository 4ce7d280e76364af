"""ctraj_run_noalloc against ctraj_run.

ctraj_run_noalloc is for callers that cannot allocate device memory while
they run: an application that hands the library a fixed device-memory budget
at start-up and owns every allocation, or a request path that cannot afford
the device-wide synchronization of cudaMalloc/cudaFree.  It keeps all of its
scratch in one fixed-size device array instead.  It must give the same
results as the context-based ctraj_run on the same inputs, call after call:
the array keeps the previous call's contents, so anything left stale from the
first call would show up in the second.

This file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

POS_TOL = 1e-6  # m, the FP32 position tolerance of the parity tests


def _noalloc(lib, cb, n, seed=0, offset=0, xd=None, vd=None, ics=None, outputs=None,
             precision=32):
    from ctraj import _abi

    a = _abi.RunArgs()
    a.n = n
    a.precision = precision
    a.seed = seed
    a.offset = offset
    a.g = 9.80665
    if ics is None:
        a.ic_mode = _abi.IC_DEVICE_DRAW
        a.xdist, a.vdist = xd, vd
    else:
        a.ic_mode = _abi.IC_DEVICE
        a.ics = int(ics.data_ptr())
    if outputs:
        a.out_mode = _abi.OUT_DEVICE
        for k, t in outputs.items():
            setattr(a, f"out_{k}", int(t.data_ptr()))
    counts = np.zeros(len(cb.labels) + 1, np.int64)
    a.counts = counts.ctypes.data
    st = _abi.RunStats()
    tabs = cb.table_structs()
    status = lib.ctraj_run_noalloc(cb.elements, cb.n_elements, len(cb.labels), tabs, len(cb.tables),
                                   ctypes.byref(a), None, ctypes.byref(st))
    _abi.check(status, lib)
    return counts, st


def _device_outputs(n):
    import torch

    return {"label": torch.full((n,), -7, dtype=torch.int32, device="cuda"),
            "final": torch.full((10, n), float("nan"), dtype=torch.float64, device="cuda"),
            "rows": torch.full((n,), -7, dtype=torch.int32, device="cuda")}


def _compare(ref_counts, ref_out, counts, out):
    np.testing.assert_array_equal(counts, ref_counts)
    np.testing.assert_array_equal(out["label"].cpu().numpy(), ref_out["label"].cpu().numpy())
    np.testing.assert_array_equal(out["rows"].cpu().numpy(), ref_out["rows"].cpu().numpy())
    f, rf = out["final"].cpu().numpy(), ref_out["final"].cpu().numpy()
    assert np.all(np.abs(f[:2] - rf[:2]) <= POS_TOL), np.abs(f[:2] - rf[:2]).max()
    np.testing.assert_allclose(f, rf, rtol=1e-6, atol=POS_TOL)


def test_noalloc_matches_run_on_two_calls_in_a_row():
    import torch

    import fixtures
    from ctraj import _abi
    from ctraj.compiler import compile_beamline
    from ctraj.distributions import device_spec
    from ctraj.engine import Engine
    from ctraj.workloads import lens_beamline, source

    eng = Engine(0)
    try:
        lib = eng.lib
        # call 1: the hexapole lens beamline at the largest allowed size, ICs drawn on the device
        cb = compile_beamline(lens_beamline())
        xd, vd = (device_spec(d, r) for d, r in zip(source(), ("position", "velocity")))
        n = _abi.NOALLOC_MAX_MOLECULES
        ref_out = _device_outputs(n)
        ref = eng.run(cb, n, precision=32, xdist=xd, vdist=vd, seed=5, offset=77, device_outputs=ref_out)
        out = _device_outputs(n)
        counts, st = _noalloc(lib, cb, n, seed=5, offset=77, xd=xd, vd=vd, outputs=out)
        torch.cuda.synchronize()
        _compare(ref.counts, ref_out, counts, out)
        assert st.molecule_steps == ref.molecule_steps and st.lens_steps == ref.lens_steps
        assert ref.counts[-1] > 0 and ref.lens_steps > 0

        # call 2: another beamline (interp1d lens table, field plates) with ICs in device memory
        fx = fixtures.load("example_lens")
        cb2 = compile_beamline(fixtures.build_beamline(fx))
        ics = torch.from_numpy(np.ascontiguousarray(fx["ics"])).cuda()
        n2 = ics.shape[1]
        ref_out2 = _device_outputs(n2)
        ref2 = eng.run(cb2, n2, precision=32, ics=ics, device_outputs=ref_out2)
        out2 = _device_outputs(n2)
        counts2, st2 = _noalloc(lib, cb2, n2, ics=ics, outputs=out2)
        torch.cuda.synchronize()
        _compare(ref2.counts, ref_out2, counts2, out2)
        assert st2.molecule_steps == ref2.molecule_steps
    finally:
        eng.close()


def test_noalloc_rejects_what_it_cannot_hold():
    from ctraj import _abi
    from ctraj.compiler import compile_beamline
    from ctraj.distributions import device_spec
    from ctraj.workloads import lens_beamline, source

    lib = _abi.load_library()
    cb = compile_beamline(lens_beamline())
    xd, vd = (device_spec(d, r) for d, r in zip(source(), ("position", "velocity")))
    with pytest.raises(ValueError, match="at most"):
        _noalloc(lib, cb, _abi.NOALLOC_MAX_MOLECULES + 1, xd=xd, vd=vd)
    with pytest.raises(ValueError, match="precision 32"):
        _noalloc(lib, cb, 1000, xd=xd, vd=vd, precision=64)
