"""ctraj_run_noalloc against ctraj_run.

ctraj_run_noalloc is for callers that cannot allocate device memory while
they run: an application that hands the library a fixed device-memory budget
at start-up and owns every allocation, or a request path that cannot afford
the device-wide synchronization of cudaMalloc/cudaFree.  It keeps all of its
scratch in one fixed-size device array instead.  It runs the same kernels as
the context-based ctraj_run with its default tuning, so on the same inputs
its counts, stats and per-molecule outputs must equal ctraj_run's bit for
bit, call after call: the array keeps the previous call's contents, so
anything left stale from the first call would show up in the second.  Free
device memory must not move across a call.

This file is named to be collected last; the checks that need no GPU (sizes
the scratch cannot hold) are in tests/test_abi.py.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _noalloc(lib, cb, n, seed=0, offset=0, xd=None, vd=None, ics=None, outputs=None, precision=32):
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
            "rows": torch.full((n,), -7, dtype=torch.int32, device="cuda"),
            "margin": torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")}


def _compare(ref, ref_out, counts, st, out):
    """Bit equality with ctraj_run: counts, stats, every per-molecule output."""
    import torch

    np.testing.assert_array_equal(counts, ref.counts)
    assert (st.molecule_steps, st.lens_steps, st.edge_band, st.table_range) == \
           (ref.molecule_steps, ref.lens_steps, ref.edge_band, ref.table_range)
    assert st.max_lens_steps == ref.extra["max_lens_steps"] and st.linear_tables == ref.extra["linear_tables"]
    for k in ("label", "rows"):
        assert torch.equal(out[k], ref_out[k]), k
    for k in ("final", "margin"):  # NaN rows (unused final slots) compare equal as bits
        assert torch.equal(out[k].view(torch.int64), ref_out[k].view(torch.int64)), k


def _two_lens_beamline():
    """Aperture, two hexapole lenses in a row (the molecules leaving the first
    queue at the second), detection plane."""
    from ctraj import Beamline, CircularAperture, ElectrostaticLens
    from ctraj.stark import hexapole_force

    f = hexapole_force(V=30e3, R=17.5e-3, splitting_hz=6.7e9)
    return Beamline([CircularAperture(name="A1", z0=0.30, L=1e-3, d=12e-3),
                     ElectrostaticLens(name="ES lens", z0=0.80, L=0.30, d=35e-3, V=30e3, dt=1e-6, a_interp=f),
                     ElectrostaticLens(name="ES lens 2", z0=1.30, L=0.30, d=35e-3, V=30e3, dt=1e-6, a_interp=f),
                     CircularAperture(name="Detection plane", z0=3.00, L=0.0, d=float("inf"))])


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
        _compare(ref, ref_out, counts, st, out)
        assert ref.counts[-1] > 0 and ref.lens_steps > 0 and st.linear_tables == 1

        # call 2: another beamline (interp1d lens table, field plates) with ICs in device memory;
        # free device memory must not move across the call
        fx = fixtures.load("example_lens")
        cb2 = compile_beamline(fixtures.build_beamline(fx))
        ics = torch.from_numpy(np.ascontiguousarray(fx["ics"])).cuda()
        n2 = ics.shape[1]
        ref_out2 = _device_outputs(n2)
        ref2 = eng.run(cb2, n2, precision=32, ics=ics, device_outputs=ref_out2)
        out2 = _device_outputs(n2)
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        counts2, st2 = _noalloc(lib, cb2, n2, ics=ics, outputs=out2)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info()[0] == free_before
        _compare(ref2, ref_out2, counts2, st2, out2)

        # call 3: two lenses in a row (the scratch's two lens queues alternate)
        cb3 = compile_beamline(_two_lens_beamline())
        n3 = 100_000
        ref_out3 = _device_outputs(n3)
        ref3 = eng.run(cb3, n3, precision=32, xdist=xd, vdist=vd, seed=11, device_outputs=ref_out3)
        out3 = _device_outputs(n3)
        counts3, st3 = _noalloc(lib, cb3, n3, seed=11, xd=xd, vd=vd, outputs=out3)
        torch.cuda.synchronize()
        _compare(ref3, ref_out3, counts3, st3, out3)
        assert st3.linear_tables == 2
        assert ref3.counts[cb3.labels.index("Inside lens")] > 0 and ref3.counts[-1] > 0
    finally:
        eng.close()
