"""Pipelined batches (ctraj_run_batch): every run of a batch must equal the
same run made alone with ctraj_run -- counts, step totals and the lens step
bound -- whichever lane ran it, under both lens modes, in FP64, with initial
conditions from the host, after the context's beamline or tuning changed,
and with the L2 flush between runs.  A run that fails validation is reported
by its index.
"""
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


def _same(batch, alone):
    assert len(batch) == len(alone)
    for b, a in zip(batch, alone):
        np.testing.assert_array_equal(b.counts, a.counts)
        assert (b.molecules, b.molecule_steps, b.lens_steps, b.table_range) == \
               (a.molecules, a.molecule_steps, a.lens_steps, a.table_range)
        assert b.extra["max_lens_steps"] == a.extra["max_lens_steps"]


@pytest.mark.parametrize("group,lanes,mpt,service", [(1, 512, 1, 64), (2, 768, 1, 5), (3, 512, 2, 64),
                                                     (16, 768, 2, 300), (4, 1024, 1, 16)])
def test_grouped_batch_equals_single_runs(engine, group, lanes, mpt, service):
    """Runs sharing lens passes (batch_group > 1) give each run's own results,
    whatever the lens pass's CTA shape; groups of 2 and 3 over 7 runs leave a
    partial last group, 16 takes them all."""
    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    n = 150_000
    seeds = [101 + 13 * k for k in range(7)]
    alone = [engine.run(cb, n + 1000 * k, xdist=xs, vdist=vs, seed=s, offset=3) for k, s in enumerate(seeds)]
    try:
        engine.set_tuning(batch_group=group, front_threads=128 if group == 3 else 256, batch_lens_threads=lanes,
                          lens_molecules=mpt, lens_service=service)
        batch = engine.run_batch(cb, [n + 1000 * k for k in range(7)], seeds, xdist=xs, vdist=vs, offset=3)
    finally:
        engine.set_tuning()
    _same(batch, alone)


def test_grouped_batch_two_lenses_and_host_ics(engine):
    """A group over a two-lens beamline (the second lens's entrants carry their
    run through the first lens pass) with initial conditions from the host."""
    import ctraj
    from ctraj.distributions import host_draw
    from ctraj.stark import hexapole_force

    f = hexapole_force(V=30e3, R=17.5e-3, splitting_hz=6.7e9)
    bl = ctraj.Beamline([ctraj.CircularAperture(name="A1", z0=0.30, L=1e-3, d=12e-3),
                         ctraj.ElectrostaticLens(name="ES lens", z0=0.8, L=0.3, d=35e-3, V=30e3, dt=1e-6, a_interp=f),
                         ctraj.ElectrostaticLens(name="ES lens 2", z0=1.3, L=0.3, d=35e-3, V=30e3, dt=1e-6,
                                                 a_interp=f),
                         ctraj.CircularAperture(name="Detection plane", z0=3.0, L=0.0, d=float("inf"))])
    cb = compile_beamline(bl)
    xd, vd = source()
    n = 120_000
    ics = [host_draw(xd, vd, n, seed=40 + k) for k in range(5)]
    alone = [engine.run(cb, n, ics=a) for a in ics]
    try:
        engine.set_tuning(batch_group=4)
        batch = engine.run_batch(cb, n, None, ics=ics)
    finally:
        engine.set_tuning()
    _same(batch, alone)
    assert alone[0].counts[cb.labels.index("Inside lens")] > 0


@pytest.mark.parametrize("n_runs", [0, 1, 2, 5])
def test_batch_equals_single_runs(engine, n_runs):
    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    n = 200_000
    seeds = [11 + 7 * k for k in range(n_runs)]
    batch = engine.run_batch(cb, n, seeds, xdist=xs, vdist=vs, offset=5)
    alone = [engine.run(cb, n, xdist=xs, vdist=vs, seed=s, offset=5) for s in seeds]
    _same(batch, alone)
    if n_runs > 1:  # distinct seeds give distinct runs
        assert not np.array_equal(batch[0].counts, batch[1].counts)


def test_batch_follows_tuning_and_beamline_changes(engine):
    xs, vs = _specs()
    n = 100_000
    cb = compile_beamline(lens_beamline())
    seeds = [3, 4, 5]
    ref = [engine.run(cb, n, xdist=xs, vdist=vs, seed=s) for s in seeds]
    try:
        engine.set_tuning(lens_mode=1, chunk_first=32)
        _same(engine.run_batch(cb, n, seeds, xdist=xs, vdist=vs, timing=True), ref)
        engine.set_tuning(lens_interval=64)
        _same(engine.run_batch(cb, n, seeds, xdist=xs, vdist=vs, l2_flush_bytes=1 << 20), ref)
    finally:
        engine.set_tuning()
    # a different beamline (the lens voltage) reaches the second lane too
    cb2 = compile_beamline(lens_beamline(V=24e3))
    ref2 = [engine.run(cb2, n, xdist=xs, vdist=vs, seed=s) for s in seeds]
    got2 = engine.run_batch(cb2, n, seeds, xdist=xs, vdist=vs)
    _same(got2, ref2)
    assert any(not np.array_equal(a.counts, b.counts) for a, b in zip(ref, ref2))


def test_batch_fp64_and_host_ics(engine):
    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    n = 4_000
    seeds = [1, 2, 3]
    _same(engine.run_batch(cb, n, seeds, precision=64, xdist=xs, vdist=vs),
          [engine.run(cb, n, precision=64, xdist=xs, vdist=vs, seed=s) for s in seeds])
    rng = np.random.default_rng(9)
    ics = []
    for _ in range(3):
        a = np.zeros((6, n))
        a[0:2] = rng.normal(0, 1e-3, (2, n))
        a[3:5] = rng.normal(0, 15.0, (2, n))
        a[5] = rng.normal(184.0, 16.0, n)
        ics.append(a)
    _same(engine.run_batch(cb, n, None, ics=ics),
          [engine.run(cb, n, ics=a) for a in ics])


def test_batch_reports_the_failing_run(engine):
    from ctraj import _abi

    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    # FP32 run 2 asks for a precision the library rejects before any launch
    engine.load(cb)
    args = (_abi.RunArgs * 4)()
    counts = [np.zeros(len(cb.labels) + 1, np.int64) for _ in range(4)]
    for k in range(4):
        a, _ = engine._args(10_000, 32, None, xs, vs, k, 0, 9.80665)
        a.counts = counts[k].ctypes.data
        args[k] = a
    args[2].precision = 16
    stats = (_abi.RunStats * 4)()
    status = engine.lib.ctraj_run_batch(engine.ctx, args, 4, stats, 0)
    assert status == _abi.EINVAL
    assert b"batch run 2" in engine.lib.ctraj_last_error()
    # the context stays usable
    r = engine.run(cb, 10_000, xdist=xs, vdist=vs, seed=0)
    assert r.counts.sum() == 10_000


def test_run_simulations_equals_the_loop():
    from ctraj import TrajectorySimulator

    xd, vd = source()
    bl = lens_beamline()
    names, seeds = ["a", "b", "c"], [1, 2, 3]
    sim = TrajectorySimulator()
    sim.run_simulations(bl, names, vdist=vd, xdist=xd, N_traj=50_000, seeds=seeds)
    loop = TrajectorySimulator()
    for name, s in zip(names, seeds):
        loop.run_simulation(bl, name, vdist=vd, xdist=xd, N_traj=50_000, seed=s)
    for name in names:
        assert sim.results[name].counter.counter_dict == loop.results[name].counter.counter_dict
    assert sim.last_run.molecule_steps == loop.last_run.molecule_steps
