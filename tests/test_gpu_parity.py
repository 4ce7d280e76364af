"""CUDA path against the oracle and the reference's golden outputs.

FP64 runs follow the reference's float64 operation order and must match the
reference fixtures exactly (labels, row counts, final rows).  FP32 runs must
give the same label for every molecule farther than 1 um from an edge (as
measured by the FP64 oracle) and final positions within 1 um of the FP64
result (tolerance written below).
"""
import numpy as np
import pytest

import fixtures
from ctraj.compiler import compile_beamline
from oracle import oracle

pytestmark = pytest.mark.gpu

POS_TOL = 1e-6     # m, final position FP32 vs FP64
VEL_TOL = 1e-4     # m/s, final velocity FP32 vs FP64
TIME_TOL = 1e-8    # s


@pytest.fixture(scope="module")
def engine():
    from ctraj.engine import Engine

    e = Engine(0)
    yield e
    e.close()


CASES = fixtures.available()


@pytest.mark.parametrize("case", CASES)
def test_fp64_matches_reference_exactly(engine, case):
    fx = fixtures.load(case)
    cb = compile_beamline(fixtures.build_beamline(fx))
    n = fx["ics"].shape[1]
    r = engine.run(cb, n, precision=64, ics=fx["ics"], outputs=True)
    assert r.label_names() == fixtures.expected_labels(fx)
    np.testing.assert_array_equal(r.rows, fx["rows"])
    both = np.isfinite(r.final).all(0) & np.isfinite(fx["final"]).all(0)
    np.testing.assert_array_equal(r.final[:, both], fx["final"][:, both])
    assert r.molecule_steps == int(fx["rows"].sum())
    o = oracle.run(cb, fx["ics"])
    np.testing.assert_array_equal(r.counts, o["counts"])
    np.testing.assert_array_equal(r.margin, o["margin"])
    assert r.edge_band == o["edge_band"]


@pytest.mark.parametrize("case", CASES)
def test_fp32_within_tolerance(engine, case):
    fx = fixtures.load(case)
    cb = compile_beamline(fixtures.build_beamline(fx))
    n = fx["ics"].shape[1]
    o = oracle.run(cb, fx["ics"])
    r = engine.run(cb, n, precision=32, ics=fx["ics"], outputs=True)
    far = o["margin"] >= 1e-6
    assert np.array_equal(r.label[far], o["label"][far])
    same = (r.label == o["label"]) & np.isfinite(o["final"]).all(0) & far
    # molecules of the lens beamline travel ~3 m; positions within 1 um
    dpos = np.abs(r.final[0:2, same] - o["final"][0:2, same])
    assert dpos.max(initial=0) < POS_TOL, dpos.max(initial=0)
    # z of a field-plate hit is (x_plate - x) / vx * vz: an error dx in x
    # becomes dx * |vz / vx| in z at grazing incidence, so z is checked to
    # POS_TOL there scaled by that factor
    plates = np.array([cb.label_of(s) in {e.name for e in fixtures.build_beamline(fx).elements
                                           if type(e).__name__ == "FieldPlates"} for s in o["label"]])
    ztol = np.where(plates, POS_TOL * np.maximum(1.0, np.abs(o["final"][5] / o["final"][3])), POS_TOL)
    dz = np.abs(r.final[2] - o["final"][2])
    assert np.all(dz[same] <= ztol[same]), dz[same].max()
    dvel = np.abs(r.final[3:6, same] - o["final"][3:6, same])
    assert dvel.max(initial=0) < VEL_TOL, dvel.max(initial=0)
    # time of a plate hit is (x_plate - x) / vx: an error dx in x is dx / |vx| in t
    ttol = TIME_TOL + np.where(plates, POS_TOL / np.abs(o["final"][3]), 0.0)
    dtime = np.abs(r.final[9] - o["final"][9])
    assert np.all(dtime[same] <= ttol[same]), dtime[same].max()
    # row counts agree except where rint(L/dz) sits on a rounding tie of vz
    assert np.mean(r.rows[same] == o["rows"][same]) > 0.999
    # without per-molecule outputs the persistent pass defers the molecules'
    # ends to k_lens_finish: the same counts and step totals
    plain = engine.run(cb, n, precision=32, ics=fx["ics"])
    np.testing.assert_array_equal(plain.counts, r.counts)
    assert (plain.molecule_steps, plain.lens_steps) == (r.molecule_steps, r.lens_steps)


@pytest.mark.parametrize("case", [c for c in CASES
                                  if c in ("config0", "config1", "example_lens", "kat_lens", "kat_honeycomb")])
def test_record_traces_match_reference(engine, case):
    fx = fixtures.load(case)
    cb = compile_beamline(fixtures.build_beamline(fx))
    n = fx["ics"].shape[1]
    tr = fixtures.traces(fx)
    ids = np.array(sorted(tr), dtype=np.int64)
    max_rows = max(t[2] for t in tr.values()) + 2
    rows64 = engine.record(cb, n, ids, stride=1, max_rows=max_rows, precision=64, ics=fx["ics"])
    rows32 = engine.record(cb, n, ids, stride=1, max_rows=max_rows, precision=32, ics=fx["ics"])
    for j, r64, r32 in zip(ids, rows64, rows32):
        ref, idx, full = tr[j]
        assert r64.shape[0] == full
        np.testing.assert_array_equal(r64 if idx is None else r64[idx], ref)
        if r32.shape[0] == full:
            d = np.abs((r32 if idx is None else r32[idx])[:, 0:2] - ref[:, 0:2])
            assert np.nanmax(d) < POS_TOL


def test_record_stride_keeps_last_row(engine):
    fx = fixtures.load("config1")
    cb = compile_beamline(fixtures.build_beamline(fx))
    n = fx["ics"].shape[1]
    j = int(np.argmax(fx["rows"]))  # the longest-lived molecule (a lens survivor)
    assert fx["rows"][j] > 3000
    full = engine.record(cb, n, [j], stride=1, max_rows=5000, precision=64, ics=fx["ics"])[0]
    assert full.shape[0] == fx["rows"][j] + 1
    np.testing.assert_array_equal(full[-1], fx["final"][:, j])
    sub = engine.record(cb, n, [j], stride=50, max_rows=200, precision=64, ics=fx["ics"])[0]
    expect = list(range(0, full.shape[0], 50))
    if expect[-1] != full.shape[0] - 1:
        expect.append(full.shape[0] - 1)
    np.testing.assert_array_equal(sub, full[expect])


def test_record_overflow_is_reported(engine):
    fx = fixtures.load("config1")
    cb = compile_beamline(fixtures.build_beamline(fx))
    n = fx["ics"].shape[1]
    j = int(np.argmax(fx["rows"]))
    from ctraj._abi import CtrajError

    with pytest.raises(CtrajError):
        engine.record(cb, n, [j], stride=1, max_rows=5, precision=64, ics=fx["ics"])


def test_device_draw_fp32_vs_fp64(engine):
    """Same Philox stream drawn in both precisions: the FP32 run must agree with
    the FP64 run molecule by molecule (labels off the 1 um band, positions)."""
    import ctraj
    from ctraj.distributions import device_spec

    fx = fixtures.load("config1")
    cb = compile_beamline(fixtures.build_beamline(fx))
    xd = device_spec(ctraj.GaussianPositionDistribution(1.5e-3, 1.5e-3, 0.0), "position")
    vd = device_spec(ctraj.CeNTREXVelocityDistribution(sigmax=20.0, sigmay=20.0), "velocity")
    n = 400_000
    r64 = engine.run(cb, n, precision=64, xdist=xd, vdist=vd, seed=7, offset=123, outputs=True)
    r32 = engine.run(cb, n, precision=32, xdist=xd, vdist=vd, seed=7, offset=123, outputs=True)
    far = r64.margin >= 1e-6
    assert np.array_equal(r32.label[far], r64.label[far])
    same = (r32.label == r64.label) & far
    d = np.abs(r32.final[0:2, same] - r64.final[0:2, same]).max()
    assert d < POS_TOL, d
    assert r64.molecule_steps > n


def test_device_draw_statistics(engine):
    """ICs drawn on the device follow the distributions (a zero-length plane at
    the source leaves every molecule at its initial state)."""
    import ctraj
    from ctraj.distributions import device_spec

    bl = ctraj.Beamline([ctraj.CircularAperture(name="src", z0=0.25, L=0.0, d=float("inf"))])
    cb = compile_beamline(bl)
    n = 1_000_000
    for prec in (32, 64):
        for xdist in (ctraj.GaussianPositionDistribution(1.5e-3, 2.5e-3, 0.25),
                      ctraj.CeNTREXPositionDistribution(d=0.02, z=0.25)):
            vdist = ctraj.CeNTREXVelocityDistribution(vx=1.0, sigmax=20.0, vy=-2.0, sigmay=30.0)
            r = engine.run(cb, n, precision=prec, xdist=device_spec(xdist, "position"),
                           vdist=device_spec(vdist, "velocity"), seed=3, outputs=True)
            f = r.final
            assert np.all(f[2] == 0.25)
            for row, mu, sd in ((3, 1.0, 20.0), (4, -2.0, 30.0), (5, 184.0, 16.0)):
                assert abs(f[row].mean() - mu) < 5 * sd / np.sqrt(n)
                assert abs(f[row].std() / sd - 1) < 5 / np.sqrt(2 * n)
            if isinstance(xdist, ctraj.GaussianPositionDistribution):
                assert abs(f[0].std() / 1.5e-3 - 1) < 5 / np.sqrt(2 * n)
                assert abs(f[1].std() / 2.5e-3 - 1) < 5 / np.sqrt(2 * n)
            else:
                rr = np.hypot(f[0], f[1])
                assert rr.max() <= 0.01 * (1 + 1e-6)
                # uniform disc: P(r < R/2) = 1/4
                assert abs(np.mean(rr < 0.005) - 0.25) < 5 * np.sqrt(0.25 * 0.75 / n)
            # molecules get distinct draws (FP32 rounding merges ~1 % near the mode)
            assert np.unique(f[3]).size > 0.95 * n


def test_seeded_large_run_matches_oracle(engine):
    """1e5 seeded molecules of the lens beamline: FP64 GPU == oracle exactly."""
    import ctraj
    from ctraj.distributions import host_draw

    fx = fixtures.load("config1")
    cb = compile_beamline(fixtures.build_beamline(fx))
    ics = host_draw(ctraj.GaussianPositionDistribution(1.5e-3, 1.5e-3, 0.0),
                    ctraj.CeNTREXVelocityDistribution(sigmax=20.0, sigmay=20.0), 100_000, seed=0)
    o = oracle.run(cb, ics, threads=8)
    r = engine.run(cb, ics.shape[1], precision=64, ics=ics, outputs=True)
    np.testing.assert_array_equal(r.label, o["label"])
    np.testing.assert_array_equal(r.final, o["final"])
    assert r.molecule_steps == o["steps"]
    assert r.lens_steps == o["lens_steps"]


def test_run_is_deterministic_and_offsets_partition(engine):
    """Counts of a run equal the sum over disjoint offset ranges (replica sharding)."""
    import ctraj
    from ctraj.distributions import device_spec

    fx = fixtures.load("config1")
    cb = compile_beamline(fixtures.build_beamline(fx))
    xd = device_spec(ctraj.GaussianPositionDistribution(1.5e-3, 1.5e-3, 0.0), "position")
    vd = device_spec(ctraj.CeNTREXVelocityDistribution(sigmax=20.0, sigmay=20.0), "velocity")
    full = engine.run(cb, 300_000, xdist=xd, vdist=vd, seed=11)
    again = engine.run(cb, 300_000, xdist=xd, vdist=vd, seed=11)
    np.testing.assert_array_equal(full.counts, again.counts)
    assert full.molecule_steps == again.molecule_steps
    parts = [engine.run(cb, 100_000, xdist=xd, vdist=vd, seed=11, offset=k * 100_000) for k in range(3)]
    np.testing.assert_array_equal(sum(p.counts for p in parts), full.counts)
    assert sum(p.molecule_steps for p in parts) == full.molecule_steps


def test_radial_table_range_error_raises(engine):
    import ctraj
    from scipy.interpolate import interp1d

    r = np.linspace(0, 0.0101, 50)
    lens = ctraj.ElectrostaticLens(name="L", z0=0.1, L=0.3, d=0.02, dz=5e-3, a_interp=interp1d(r, -1e5 * r))
    cb = compile_beamline(ctraj.Beamline([lens]))
    ics = np.array([[9.9e-3], [0.0], [0.1], [200.0], [0.0], [184.0]])
    for prec in (32, 64):
        with pytest.raises(ValueError):
            engine.run(cb, 1, precision=prec, ics=ics)


def test_empty_and_tiny_runs(engine):
    fx = fixtures.load("config0")
    cb = compile_beamline(fixtures.build_beamline(fx))
    r = engine.run(cb, 0, precision=32, ics=np.zeros((6, 0)))
    assert r.counts.sum() == 0 and r.molecule_steps == 0
    for n in (1, 31, 33):
        ics = np.ascontiguousarray(fx["ics"][:, :n])
        r = engine.run(cb, n, precision=64, ics=ics, outputs=True)
        assert r.label_names() == fixtures.expected_labels(fx)[:n]


def test_results_do_not_depend_on_tuning(engine):
    """The launch knobs change speed only: counts and per-molecule results are identical."""
    import ctraj
    from ctraj.distributions import device_spec
    from ctraj.workloads import lens_beamline, source

    cb = compile_beamline(lens_beamline())
    xd, vd = (device_spec(d, r) for d, r in zip(source(), ("position", "velocity")))
    ref = engine.run(cb, 200_000, xdist=xd, vdist=vd, seed=9, outputs=True)
    try:
        for t in (dict(chunk_first=16, chunk_growth=100, chunk_max=16, front_waves=1, lens_mode=1),
                  dict(chunk_first=2048, chunk_growth=150, chunk_max=8192, front_waves=8, lens_mode=1),
                  dict(lens_interval=1), dict(lens_interval=5000, front_waves=2),
                  dict(front_threads=128, front_waves=8), dict(front_threads=512, front_waves=1),
                  dict(lens_threads=768), dict(lens_threads=1024, lens_interval=64),
                  dict(lens_service=1), dict(lens_service=16), dict(lens_service=1000, lens_interval=100)):
            engine.set_tuning(**t)
            r = engine.run(cb, 200_000, xdist=xd, vdist=vd, seed=9, outputs=True)
            np.testing.assert_array_equal(r.counts, ref.counts)
            np.testing.assert_array_equal(r.label, ref.label)
            np.testing.assert_array_equal(r.final, ref.final)
            assert r.molecule_steps == ref.molecule_steps
        with pytest.raises(ValueError):
            engine.set_tuning(chunk_first=0)
        with pytest.raises(ValueError):
            engine.set_tuning(lens_mode=2)
        with pytest.raises(ValueError):
            engine.set_tuning(lens_interval=0)
        # the lens-pass CTA shapes of the throughput path (runs without
        # per-molecule outputs): counts and step totals equal
        plain = engine.run(cb, 200_000, xdist=xd, vdist=vd, seed=9)
        np.testing.assert_array_equal(plain.counts, ref.counts)
        for t in (dict(lens_threads=768), dict(lens_threads=1024, lens_interval=64),
                  dict(lens_threads=768, lens_molecules=2), dict(lens_threads=512, lens_molecules=2, lens_interval=32),
                  dict(lens_threads=1024, lens_molecules=2, lens_interval=1000),
                  dict(lens_threads=1024, lens_service=256), dict(lens_threads=768, lens_molecules=2, lens_service=7)):
            engine.set_tuning(**t)
            r = engine.run(cb, 200_000, xdist=xd, vdist=vd, seed=9)
            np.testing.assert_array_equal(r.counts, ref.counts)
            assert (r.molecule_steps, r.lens_steps) == (plain.molecule_steps, plain.lens_steps), t
        with pytest.raises(ValueError):
            engine.set_tuning(lens_molecules=3)
        with pytest.raises(ValueError):
            engine.set_tuning(front_threads=300)
        with pytest.raises(ValueError):
            engine.set_tuning(batch_group=65)
        with pytest.raises(ValueError):
            engine.set_tuning(lens_service=0)
    finally:
        engine.set_tuning()


@pytest.mark.parametrize("case, linear", [("config1", 1), ("kat_lens", 0)])
def test_stark_table_form(engine, case, linear):
    """The 4096-knot hexapole table goes to the FP32 lens kernels as quarter-
    interval linear pieces (accurate to 4e-7 of its largest force); the coarse
    known-answer table (6.5e-6) keeps the exact quadratic.  Both are held to
    the FP32 tolerance by test_fp32_within_tolerance; FP64 never uses pieces."""
    fx = fixtures.load(case)
    cb = compile_beamline(fixtures.build_beamline(fx))
    n = fx["ics"].shape[1]
    assert engine.run(cb, n, precision=32, ics=fx["ics"]).extra["linear_tables"] == linear
    assert engine.run(cb, n, precision=64, ics=fx["ics"]).extra["linear_tables"] == 0


def test_front_staging_overflow(engine):
    """A beam that mostly reaches the lens: a front CTA of 128 threads meets
    more lens entrants than its staging area holds (192), and its warps append
    the rest to the queue themselves.  Per-molecule results, counts and step
    totals equal those of a launch shape that stages every entrant (512
    threads, one iteration per CTA), in a plain run, a grouped batch and a run
    with ring recording."""
    import ctraj
    from ctraj.distributions import device_spec
    from ctraj.ring import HBMRing
    from ctraj.workloads import lens_beamline

    cb = compile_beamline(lens_beamline(aperture_d=0.1))
    xd = device_spec(ctraj.GaussianPositionDistribution(1.5e-3, 1.5e-3, 0.0), "position")
    vd = device_spec(ctraj.CeNTREXVelocityDistribution(sigmax=1.0, sigmay=1.0), "velocity")
    n = 400_000
    try:
        engine.set_tuning(front_threads=512, front_waves=8)  # ceil(n / 512) CTAs of one iteration
        ref = engine.run(cb, n, xdist=xd, vdist=vd, seed=5, outputs=True)
        reached = 1.0 - ref.counts[cb.labels.index("A1")] / n
        assert reached > 0.9  # > 0.58 of 329 molecules per CTA overflow 192 entries
        ring_ref = HBMRing(capacity_rows=28_000_000, capacity_molecules=n, stride=50)  # holds every record
        rr = engine.run(cb, n, xdist=xd, vdist=vd, seed=5, ring=ring_ref)
        assert ring_ref.counts()[0] <= ring_ref.capacity_rows
        batch_ref = engine.run_batch(cb, n, [5, 6], xdist=xd, vdist=vd)
        engine.set_tuning(front_threads=128, front_waves=1, batch_group=2)  # 1216 CTAs: ~329 molecules each
        r = engine.run(cb, n, xdist=xd, vdist=vd, seed=5, outputs=True)
        np.testing.assert_array_equal(r.counts, ref.counts)
        np.testing.assert_array_equal(r.label, ref.label)
        np.testing.assert_array_equal(r.final, ref.final)
        assert (r.molecule_steps, r.lens_steps) == (ref.molecule_steps, ref.lens_steps)
        ring = HBMRing(capacity_rows=28_000_000, capacity_molecules=n, stride=50)
        rg = engine.run(cb, n, xdist=xd, vdist=vd, seed=5, ring=ring)
        np.testing.assert_array_equal(rg.counts, rr.counts)
        want = {q.molecule: q for q in ring_ref.read()}
        got = ring.read()
        assert len(got) == len(want) > 0
        for q in got:
            np.testing.assert_array_equal(q.rows, want[q.molecule].rows)
        batch = engine.run_batch(cb, n, [5, 6], xdist=xd, vdist=vd)
        for a, b in zip(batch, batch_ref):
            np.testing.assert_array_equal(a.counts, b.counts)
            assert (a.molecule_steps, a.lens_steps) == (b.molecule_steps, b.lens_steps)
        np.testing.assert_array_equal(batch[0].counts, ref.counts)
    finally:
        engine.set_tuning()


def test_unusable_lens_step_count_raises(engine):
    """A molecule entering a fixed-time-step lens with vz = 1e-9 m/s: rint(L /
    dz) = 3e14 exceeds CTRAJ_MAX_LENS_STEPS, where the reference's step count
    is unusable (electrostatic_lens.py:87-88).  The run finishes, credits the
    molecule to the lens and raises OverflowError -- with and without
    per-molecule outputs (molecule ends inside the pass or in k_lens_finish),
    in both precisions, alone and beside a normal molecule."""
    import ctraj
    from ctraj.stark import hexapole_force

    lens = ctraj.ElectrostaticLens(name="L", z0=0.0, L=0.3, d=0.02, V=30e3, dt=1e-6,
                                   a_interp=hexapole_force(V=30e3, R=10e-3))
    det = ctraj.CircularAperture(name="Det", z0=1.0, L=0.0, d=float("inf"))
    cb = compile_beamline(ctraj.Beamline([lens, det]))
    ics = np.array([[1e-3, 0.0], [0.0, 0.0], [0.0, 0.0], [0.0, 0.0], [0.0, 0.0], [1e-9, 184.0]])
    for prec in (32, 64):
        for outputs in (False, True):
            for n in (1, 2):
                with pytest.raises(OverflowError):
                    engine.run(cb, n, precision=prec, ics=np.ascontiguousarray(ics[:, :n]), outputs=outputs)
    ok = engine.run(cb, 1, precision=32, ics=np.ascontiguousarray(ics[:, 1:]))  # the normal one alone
    assert ok.counter_dict().get("Detected", 0) == 1


@pytest.mark.parametrize("first", ["circle", "rectangle", "lens"])
def test_front_screening_matches_the_full_walk(engine, first):
    """Runs without per-molecule outputs screen molecules at element 0 (a
    circular or rectangular aperture) on their x alone, from the first Philox
    call; runs with outputs walk every molecule.  Both must give the same
    counts and step totals for every seed and offset, including a first
    aperture a beam mostly misses, one it mostly passes, and no aperture at
    all (no screening)."""
    import ctraj
    from ctraj.distributions import device_spec
    from ctraj.workloads import lens_beamline, source

    if first == "circle":
        bl = lens_beamline()
    elif first == "rectangle":
        rect = ctraj.RectangularAperture(name="R0", z0=0.30, L=1e-3, w=10e-3, h=8e-3)
        base = lens_beamline().elements
        bl = ctraj.Beamline([rect] + [e for e in base if e.name != "A1"])
    else:
        bl = ctraj.Beamline([e for e in lens_beamline().elements if e.name != "A1"])
    cb = compile_beamline(bl)
    xd, vd = (device_spec(d, r) for d, r in zip(source(), ("position", "velocity")))
    for seed, offset, n in ((3, 0, 300_000), (4, 12_345, 100_001), (5, 7, 33)):
        full = engine.run(cb, n, xdist=xd, vdist=vd, seed=seed, offset=offset, outputs=True)
        fast = engine.run(cb, n, xdist=xd, vdist=vd, seed=seed, offset=offset)
        np.testing.assert_array_equal(fast.counts, full.counts)
        assert (fast.molecule_steps, fast.lens_steps) == (full.molecule_steps, full.lens_steps)
    narrow = device_spec(ctraj.CeNTREXVelocityDistribution(sigmax=1.0, sigmay=1.0), "velocity")
    full = engine.run(cb, 200_000, xdist=xd, vdist=narrow, seed=9, outputs=True)
    fast = engine.run(cb, 200_000, xdist=xd, vdist=narrow, seed=9)
    np.testing.assert_array_equal(fast.counts, full.counts)
    assert fast.molecule_steps == full.molecule_steps
