"""Parity at the sizes the benchmark quotes, through the C ABI.

* Lens beamline (the bench workload), 1e7 molecules: the FP32 path against
  the FP64 path on the same Philox stream.  Every molecule farther than 1 um
  from an aperture or bore edge (FP64 margin) must get the same label, and
  the same-label molecules' final x and y must agree within 1 um.  The FP64
  path itself equals the oracle bit for bit (tests/test_gpu_parity.py and the
  next test) and the reference's own outputs on the fixtures.
* Ballistic beamline (config 0), 1e5 molecules, numpy default_rng(0) initial
  conditions, FP64: labels, final rows, row counts and per-element counts
  equal to the oracle's, bit for bit.

Reference semantics: electrostatic_lens.py:79-118 (lens RK4, bore test),
apertures.py:92-115,165-189 (hit tests), trajectory_simulator.py:62-76.
"""
import os

import numpy as np
import pytest

from ctraj.compiler import compile_beamline
from ctraj.distributions import device_spec, host_draw
from ctraj.workloads import ballistic_beamline, lens_beamline, source
from oracle import oracle

pytestmark = pytest.mark.gpu

POS_TOL = 1e-6    # m: FP32 final x, y against FP64
VEL_TOL = 1e-4    # m/s
EDGE_BAND = 1e-6  # m: molecules nearer an edge than this may change label in FP32


@pytest.fixture(scope="module")
def engine():
    from ctraj.engine import Engine

    e = Engine(0)
    yield e
    e.close()


def test_lens_beamline_fp32_vs_fp64_at_1e7(engine):
    import torch

    n = 10_000_000
    cb = compile_beamline(lens_beamline())
    xs, vs = (device_spec(d, r) for d, r in zip(source(), ("position", "velocity")))
    outs, runs = {}, {}
    for prec in (32, 64):
        o = {"label": torch.empty(n, dtype=torch.int32, device="cuda"),
             "final": torch.empty((10, n), dtype=torch.float64, device="cuda"),
             "margin": torch.empty(n, dtype=torch.float64, device="cuda")}
        runs[prec] = engine.run(cb, n, precision=prec, xdist=xs, vdist=vs, seed=1019, device_outputs=o)
        outs[prec] = o
    o32, o64 = outs[32], outs[64]
    far = o64["margin"] >= EDGE_BAND
    assert int(((o32["label"] != o64["label"]) & far).sum()) == 0
    same = (o32["label"] == o64["label"]) & far
    d = (o32["final"][:, same] - o64["final"][:, same]).abs()
    assert float(d[0].max()) <= POS_TOL and float(d[1].max()) <= POS_TOL, (float(d[0].max()), float(d[1].max()))
    assert float(d[3:6].max()) <= VEL_TOL
    # the band is a tiny share of the run; the plain (timed) FP32 path gives the same counts
    assert int((~far).sum()) < n // 200  # 0.23 % at this size
    plain = engine.run(cb, n, precision=32, xdist=xs, vdist=vs, seed=1019)
    np.testing.assert_array_equal(plain.counts, runs[32].counts)
    assert plain.molecule_steps == runs[32].molecule_steps
    assert runs[64].counts[-1] > 0 and runs[64].lens_steps > 1e8


def test_ballistic_beamline_fp64_equals_oracle_at_1e5(engine):
    n = 100_000
    cb = compile_beamline(ballistic_beamline())
    xd, vd = source()
    ics = host_draw(xd, vd, n, seed=0)
    o = oracle.run(cb, ics, threads=os.cpu_count() or 1)
    r = engine.run(cb, n, precision=64, ics=ics, outputs=True)
    np.testing.assert_array_equal(r.label, o["label"])
    np.testing.assert_array_equal(r.rows, o["rows"])
    np.testing.assert_array_equal(r.counts, o["counts"])
    fin = np.isfinite(o["final"]).all(0)
    np.testing.assert_array_equal(np.isfinite(r.final).all(0), fin)
    np.testing.assert_array_equal(r.final[:, fin], o["final"][:, fin])
    assert r.molecule_steps == o["steps"]
    assert 0 < r.counts[-1] < n
