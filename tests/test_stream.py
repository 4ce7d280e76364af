"""Streamed runs (consecutive Philox ranges) and Adam tuning through the adjoint."""
import numpy as np
import pytest

from ctraj.compiler import compile_beamline
from ctraj.workloads import lens_beamline, source

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from ctraj.engine import Engine

    e = Engine(0)
    yield e
    e.close()


def _specs():
    from ctraj.distributions import device_spec

    xd, vd = source()
    return device_spec(xd, "position"), device_spec(vd, "velocity")


def test_streamed_run_equals_one_run(engine):
    from ctraj.ring import HBMRing
    from ctraj.stream import run_streamed

    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    n = 300_000
    one = engine.run(cb, n, xdist=xs, vdist=vs, seed=3, offset=1000, outputs=True)
    ring = HBMRing(capacity_rows=1_000_000, capacity_molecules=100_000, stride=50)
    st = run_streamed(cb, n, chunk=70_001, xdist=xs, vdist=vs, seed=3, offset=1000, ring=ring, engine=engine)
    assert st.chunks == 5
    np.testing.assert_array_equal(st.counts, one.counts)
    assert st.molecule_steps == one.molecule_steps and st.lens_steps == one.lens_steps
    hits = {cb.labels.index("Lens entrance"), cb.labels.index("Inside lens")}
    expected = set((1000 + np.flatnonzero(np.isin(one.label, list(hits)))).tolist())
    assert {rec.molecule for rec in ring.read()} == expected


def test_adam_raises_the_soft_transmission(engine):
    from ctraj.adjoint import SoftProblem, soft_transmission
    from ctraj.stream import adam_tune

    prob = SoftProblem.from_beamline(lens_beamline(), n=200_000, aperture="A1")
    p0 = prob.initial_params()
    out = adam_tune(prob, which=("V", "lens_z0"), steps=25, lr=0.02, engine=engine)
    assert out["trajectory"].shape == (25, 2) and np.isfinite(out["transmission"]).all()
    # same molecules before and after: the tuned lens transmits more
    prob.seed = 12345
    before = soft_transmission(prob, p0, want_grad=False, engine=engine).loss
    after = soft_transmission(prob, out["params"], want_grad=False, engine=engine).loss
    assert after > before
    assert out["params"][2:].tolist() == p0[2:].tolist()  # untouched parameters stay
    lim = prob.param_bounds()
    assert (out["params"] >= lim[:, 0]).all() and (out["params"] <= lim[:, 1]).all()
    assert (out["trajectory"][:, 0] >= 0).all()  # the voltage stays physical


def test_drained_ring_keeps_every_record_of_the_stream(engine):
    """A ring half the size of the stream's records, drained to host memory
    after every run, ends up with exactly the records one ring large enough
    for the whole stream holds; a ring too small for one run reports its
    losses."""
    from ctraj.ring import HBMRing, HostRingStore
    from ctraj.stream import run_streamed

    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    n, chunk = 300_000, 70_001
    big = HBMRing(capacity_rows=2_000_000, capacity_molecules=200_000, stride=50)
    whole = run_streamed(cb, n, chunk=chunk, xdist=xs, vdist=vs, seed=8, ring=big, engine=engine)
    assert whole.rows_lost == 0 and whole.ring_rows > 0
    ref = {r.molecule: r for r in big.read()}
    assert len(ref) == whole.ring_molecules
    small = HBMRing(capacity_rows=whole.ring_rows // 2, capacity_molecules=whole.ring_molecules // 2, stride=50)
    store = HostRingStore()
    st = run_streamed(cb, n, chunk=chunk, xdist=xs, vdist=vs, seed=8, ring=small, engine=engine, drain=store)
    assert (st.ring_rows, st.ring_molecules, st.rows_lost, st.molecules_lost) == \
           (whole.ring_rows, whole.ring_molecules, 0, 0)
    np.testing.assert_array_equal(st.counts, whole.counts)
    got = store.records()
    assert len(got) == len(ref) and store.rows_total == whole.ring_rows
    for rec in got:
        r = ref[rec.molecule]
        assert rec.label == r.label
        np.testing.assert_array_equal(rec.rows, r.rows)
    tiny = HBMRing(capacity_rows=500, capacity_molecules=50, stride=50)
    lossy = run_streamed(cb, n, chunk=chunk, xdist=xs, vdist=vs, seed=8, ring=tiny, engine=engine,
                         drain=HostRingStore(keep=False))
    assert lossy.ring_rows == whole.ring_rows and lossy.rows_lost > 0 and lossy.molecules_lost > 0
