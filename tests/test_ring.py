"""Ring recording (ctraj_run_ring) of the molecules lost on the lens.

The ring must hold exactly the molecules the run credits to "Lens entrance" and
"Inside lens", the run's counts must not change, and every recorded row must
equal (bit for bit in x, y, vx, vy; as float in z, t) the trajectory row of the
same RK4 step from the replay (ctraj_record with stride 1).  A ring smaller
than the run keeps the latest complete records.
"""
import numpy as np
import pytest

from ctraj.compiler import compile_beamline
from ctraj.workloads import lens_beamline, source

pytestmark = pytest.mark.gpu

STRIDE = 50
ENTRANCE_ROW = 3  # trajectory rows before the lens: initial, A1 z0, A1 z1, lens z0


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


def test_ring_holds_the_lens_hits_and_matches_the_replay(engine):
    from ctraj.ring import HBMRing

    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    n = 40_000
    ring = HBMRing(capacity_rows=200_000, capacity_molecules=20_000, stride=STRIDE)
    r = engine.run(cb, n, xdist=xs, vdist=vs, seed=21, ring=ring)
    plain = engine.run(cb, n, xdist=xs, vdist=vs, seed=21, outputs=True)
    np.testing.assert_array_equal(r.counts, plain.counts)
    hit_slots = {cb.labels.index("Lens entrance"), cb.labels.index("Inside lens")}
    expected = set(np.flatnonzero(np.isin(plain.label, list(hit_slots))).tolist())
    recs = ring.read()
    got = {rec.molecule for rec in recs}
    assert got == expected and len(recs) == len(expected)
    for rec in recs:
        assert rec.label == plain.label[rec.molecule]
    # rows against the replay, for a sample of both kinds of hit
    inside = [rec for rec in recs if rec.label == cb.labels.index("Inside lens")]
    entrance = [rec for rec in recs if rec.label == cb.labels.index("Lens entrance")]
    assert inside and entrance
    sample = sorted(inside, key=lambda q: -len(q.rows))[:20] + inside[:20] + entrance[:10]
    ids = [rec.molecule for rec in sample]
    rows = engine.record(cb, n, ids, stride=1, max_rows=8000, xdist=xs, vdist=vs, seed=21)
    for rec, full in zip(sample, rows):
        steps = rec.rows[:, 7].astype(np.int64)
        if rec.label == cb.labels.index("Lens entrance"):
            assert len(rec.rows) == 1 and steps[0] == 0
            ref = full[-1]  # the record ends at the entrance plane
        else:
            assert steps[0] == 0 and (np.diff(steps) > 0).all()
            assert (steps[1:-1] % STRIDE == 0).all()
            assert steps[-1] == len(full) - 1 - ENTRANCE_ROW  # the losing step is the last row
            ref = full[ENTRANCE_ROW + steps]
        ref = np.atleast_2d(ref)
        # record row: x, y, z, vx, vy, vz, ax, ay, az, t
        np.testing.assert_array_equal(rec.rows[:, [0, 1, 3, 4]], ref[:, [0, 1, 3, 4]].astype(np.float32))
        np.testing.assert_array_equal(rec.rows[:, 5], ref[:, 5].astype(np.float32))
        np.testing.assert_array_equal(rec.rows[:, 2], ref[:, 2].astype(np.float32))
        np.testing.assert_array_equal(rec.rows[:, 6], ref[:, 9].astype(np.float32))


def test_small_ring_keeps_the_latest_complete_records(engine):
    from ctraj.ring import HBMRing

    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    n = 20_000
    big = HBMRing(capacity_rows=100_000, capacity_molecules=10_000, stride=STRIDE)
    engine.run(cb, n, xdist=xs, vdist=vs, seed=5, ring=big)
    full = {rec.molecule: rec.rows for rec in big.read()}
    # rows and index entries are taken in one order (record slot order), so
    # the latest index entries hold the latest rows: the records kept are the
    # latest ones whose rows fit the 3000-row window (a record has at most
    # ~5500 / 50 + 2 rows), a suffix of the last 40 index entries
    small = HBMRing(capacity_rows=3000, capacity_molecules=40, stride=STRIDE)
    engine.run(cb, n, xdist=xs, vdist=vs, seed=5, ring=small)
    n_rows, n_mol = small.counts()
    assert n_rows > 3000 and n_mol > 40  # wrapped
    assert (n_rows, n_mol) == big.counts()
    kept = small.read()
    assert 0 < len(kept) <= 40
    idx = small.index.cpu().numpy()
    latest = [int(idx[e % 40][0]) for e in range(n_mol - 40, n_mol)]
    assert [rec.molecule for rec in kept] == latest[40 - len(kept):]
    assert sum(len(rec.rows) for rec in kept) <= 3000
    for rec in kept:
        np.testing.assert_array_equal(rec.rows, full[rec.molecule])
    # a second run appends after the first
    engine.run(cb, n, xdist=xs, vdist=vs, seed=5, ring=small)
    assert small.counts() == (2 * n_rows, 2 * n_mol)


def test_ring_is_the_same_in_both_lens_modes(engine):
    """The persistent lens pass (default) and the chunked one record the same
    molecules with the same rows."""
    from ctraj.ring import HBMRing

    cb = compile_beamline(lens_beamline())
    xs, vs = _specs()
    n = 30_000
    out = []
    try:
        for mode in (0, 1):
            engine.set_tuning(lens_mode=mode)
            ring = HBMRing(capacity_rows=150_000, capacity_molecules=15_000, stride=STRIDE)
            r = engine.run(cb, n, xdist=xs, vdist=vs, seed=8, ring=ring)
            out.append((r.counts, {rec.molecule: (rec.label, rec.rows) for rec in ring.read()}, ring.counts()))
    finally:
        engine.set_tuning()
    (c0, m0, k0), (c1, m1, k1) = out
    np.testing.assert_array_equal(c0, c1)
    assert k0 == k1 and m0.keys() == m1.keys() and m0
    for mol, (label, rows) in m0.items():
        assert m1[mol][0] == label
        np.testing.assert_array_equal(m1[mol][1], rows)


def test_ring_argument_checks(engine):
    from ctraj.ring import HBMRing

    xs, vs = _specs()
    cb = compile_beamline(lens_beamline())
    ring = HBMRing(capacity_rows=10, capacity_molecules=10)
    with pytest.raises(ValueError, match="precision 32"):
        engine.run(cb, 100, precision=64, xdist=xs, vdist=vs, ring=ring)
    with pytest.raises(ValueError):
        HBMRing(capacity_rows=0, capacity_molecules=1)
