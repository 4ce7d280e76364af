"""Batched lens sweep (ctraj_run_sweep).

CPU: the configuration bookkeeping (flattening, first molecule numbers, field
coefficients) and the sweep workload's shape.  GPU: per-configuration counts
of one sweep call against a loop of plain runs of each configuration (same
Philox counters), against the FP64 oracle on host initial conditions, graph
replay against direct launches, and the argument checks.
"""
import numpy as np
import pytest

from ctraj.stark import field_coefficient, hexapole_force
from ctraj.sweep import SweepConfigs, config_beamlines, sweep_beamline
from ctraj.workloads import ballistic_beamline, lens_beamline, source, sweep_configs

# A molecule whose lens trajectory passes within a few nm of the bore can be
# lost in one FP32 evaluation order and not the other (the sweep scales an
# unscaled table per molecule; the plain path folds the scale into the table).
COUNT_TOL = 2


def small_configs(n_lo=300, n_hi=3000, seed=3):
    rng = np.random.default_rng(seed)
    volts = np.array([0.0, 5e3, 12e3, 21e3, 30e3])
    forces = [hexapole_force(V=30e3, splitting_hz=a, n_knots=1024) for a in (6.7e9, 20.0e9)]
    n = rng.integers(n_lo, n_hi, (2, volts.size))
    return SweepConfigs(voltages=volts, forces=forces, n_molecules=n)


def test_config_bookkeeping():
    cfg = small_configs()
    assert cfg.shape == (2, 5) and cfg.n_configs == 10
    flat = cfg.n_molecules.reshape(-1)
    np.testing.assert_array_equal(cfg.starts(), np.concatenate([[0], np.cumsum(flat)[:-1]]))
    np.testing.assert_array_equal(cfg.table_index(), [0] * 5 + [1] * 5)
    a = cfg.alphas()
    assert a[7] == field_coefficient(cfg.voltages[2], 17.5e-3, 2)
    f = cfg.force(1, 3)
    assert f.V == cfg.voltages[3] and f.alpha == a[8]
    np.testing.assert_array_equal(f.coef, cfg.forces[1].coef)


def test_sweep_workload_shape():
    cfg = sweep_configs(n_voltages=16, n_knots=64)
    assert cfg.shape == (4, 16)
    assert cfg.n_molecules.min() >= 1e4 and cfg.n_molecules.max() <= 1e6
    assert (cfg.voltages >= 0).all() and (cfg.voltages <= 30e3).all()
    again = sweep_configs(n_voltages=16, n_knots=64)
    np.testing.assert_array_equal(cfg.n_molecules, again.n_molecules)


def test_sweep_beamline_needs_one_lens():
    with pytest.raises(ValueError, match="exactly one"):
        sweep_beamline(ballistic_beamline())
    assert sweep_beamline(lens_beamline()).n_lenses == 1


def test_config_beamlines_swap_the_lens_force():
    cfg = small_configs()
    cbs = config_beamlines(lens_beamline(), cfg)
    assert len(cbs) == cfg.n_configs
    lens = [e for e in cbs[8].elements if e.type == 4][0]
    assert lens.p[3] == cfg.voltages[3] and lens.p[6] == cfg.alphas()[8]
    np.testing.assert_array_equal(cbs[8].tables[0].coef, cfg.forces[1].coef)


# ---------------------------------------------------------------------------
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


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [True, False])
def test_sweep_matches_loop_of_plain_runs(engine, use_graph):
    from ctraj.sweep import loop_sweep, run_sweep

    cfg = small_configs(20_000, 60_000)
    bl = lens_beamline()
    xs, vs = _specs()
    r = run_sweep(bl, cfg, xdist=xs, vdist=vs, seed=11, offset=5, use_graph=use_graph, engine=engine)
    loop = loop_sweep(config_beamlines(bl, cfg), cfg, xdist=xs, vdist=vs, seed=11, offset=5,
                      engine=engine)
    np.testing.assert_array_equal(r.counts.sum(-1), cfg.n_molecules)
    np.testing.assert_array_equal(r.totals, r.counts.reshape(-1, r.counts.shape[-1]).sum(0))
    diff = np.abs(r.counts - loop).sum(-1)
    assert diff.max() <= COUNT_TOL, diff
    # the voltage matters (this Stark state is pushed to high field: defocused)
    det = r.detected_fraction()
    assert det[0, -1] < det[0, 0]
    assert r.lens_steps > 0 and r.molecule_steps > r.lens_steps
    assert r.molecules == cfg.total


@pytest.mark.gpu
def test_graph_replay_equals_direct_launches(engine):
    from ctraj.sweep import run_sweep

    cfg = small_configs(5_000, 20_000, seed=8)
    bl = lens_beamline()
    xs, vs = _specs()
    direct = run_sweep(bl, cfg, xdist=xs, vdist=vs, seed=2, use_graph=False, engine=engine)
    g1 = run_sweep(bl, cfg, xdist=xs, vdist=vs, seed=2, use_graph=True, engine=engine)
    g2 = run_sweep(bl, cfg, xdist=xs, vdist=vs, seed=2, use_graph=True, engine=engine)
    np.testing.assert_array_equal(g1.counts, direct.counts)
    np.testing.assert_array_equal(g2.counts, direct.counts)
    assert g2.molecule_steps == direct.molecule_steps and g2.lens_steps == direct.lens_steps
    # a changed input is a new graph, not a stale replay
    g3 = run_sweep(bl, cfg, xdist=xs, vdist=vs, seed=3, use_graph=True, engine=engine)
    d3 = run_sweep(bl, cfg, xdist=xs, vdist=vs, seed=3, use_graph=False, engine=engine)
    np.testing.assert_array_equal(g3.counts, d3.counts)
    assert not np.array_equal(g3.counts, g2.counts)


@pytest.mark.gpu
@pytest.mark.parametrize("use_graph", [True, False])
def test_persistent_and_chunked_sweeps_agree(engine, use_graph):
    """The one-launch persistent lens pass (default) and the chunked one give
    the same per-configuration counts and steps: the same molecules through
    the same arithmetic, in another order, at every CTA size of the
    persistent pass."""
    from ctraj.sweep import run_sweep

    cfg = small_configs(10_000, 40_000, seed=5)
    bl = lens_beamline()
    xs, vs = _specs()
    try:
        engine.set_tuning(lens_mode=1)
        chunked = run_sweep(bl, cfg, xdist=xs, vdist=vs, seed=4, use_graph=use_graph, engine=engine)
        for interval, service, threads in ((256, 64, 512), (7, 3, 512), (256, 500, 512), (128, 64, 768),
                                           (5, 9, 1024)):
            engine.set_tuning(lens_interval=interval, lens_service=service, lens_threads=threads)
            pers = run_sweep(bl, cfg, xdist=xs, vdist=vs, seed=4, use_graph=use_graph, engine=engine)
            np.testing.assert_array_equal(pers.counts, chunked.counts)
            assert pers.molecule_steps == chunked.molecule_steps and pers.lens_steps == chunked.lens_steps
    finally:
        engine.set_tuning()


@pytest.mark.gpu
def test_sweep_matches_fp64_oracle_on_host_ics(engine):
    from ctraj.distributions import host_draw
    from ctraj.sweep import run_sweep
    from oracle import oracle

    cfg = small_configs(300, 1500, seed=5)
    bl = lens_beamline()
    ics = host_draw(*source(), cfg.total, seed=9)
    r = run_sweep(bl, cfg, ics=ics, engine=engine)
    cbs = config_beamlines(bl, cfg)
    starts = cfg.starts()
    flat = r.counts.reshape(cfg.n_configs, -1)
    for c, cb in enumerate(cbs):
        n = int(cfg.n_molecules.reshape(-1)[c])
        o = oracle.run(cb, np.ascontiguousarray(ics[:, starts[c]:starts[c] + n]), outputs=False)
        assert np.abs(flat[c] - o["counts"]).sum() <= COUNT_TOL, (c, flat[c], o["counts"])


@pytest.mark.gpu
def test_sweep_argument_checks(engine):
    from ctraj.compiler import compile_beamline

    cfg = small_configs()
    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    tabs = cfg.tables()
    n = cfg.n_molecules.reshape(-1)
    with pytest.raises(ValueError, match="equal length"):
        engine.run_sweep(cb, tabs, cfg.alphas()[:-1], cfg.table_index(), n, xdist=xs, vdist=vs)
    bad_alpha = cfg.alphas()
    bad_alpha[3] = np.nan
    with pytest.raises(ValueError, match="alpha"):
        engine.run_sweep(cb, tabs, bad_alpha, cfg.table_index(), n, xdist=xs, vdist=vs)
    neg = n.copy()
    neg[0] = -1
    with pytest.raises(ValueError, match="negative"):
        engine.run_sweep(cb, tabs, cfg.alphas(), cfg.table_index(), neg, xdist=xs, vdist=vs)
    two = compile_beamline(ballistic_beamline())
    with pytest.raises(ValueError, match="exactly one lens"):
        engine.run_sweep(two, tabs, cfg.alphas(), cfg.table_index(), n, xdist=xs, vdist=vs)
    # an empty sweep runs and counts nothing
    z = engine.run_sweep(cb, tabs, cfg.alphas(), cfg.table_index(), np.zeros_like(n), xdist=xs, vdist=vs)
    assert z["counts"].sum() == 0 and z["totals"].sum() == 0
