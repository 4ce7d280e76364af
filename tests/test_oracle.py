"""The FP64 oracle against the reference's own outputs (tests/golden/*.npz).

The fixtures were produced by running the reference package on injected
initial conditions (tests/golden/make_golden.py).  The oracle must reproduce
every label and every row count exactly and every finite final trajectory row
bit for bit (it restates the reference's float64 operation order).
"""
import numpy as np
import pytest

import fixtures
from ctraj.compiler import compile_beamline
from oracle import oracle

CASES = fixtures.available()


def test_fixtures_present():
    assert set(CASES) == set(fixtures.CASES)


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_reference(case):
    fx = fixtures.load(case)
    cb = compile_beamline(fixtures.build_beamline(fx))
    r = oracle.run(cb, fx["ics"], threads=2)
    assert r["status"] == 0
    got = [cb.label_of(s) for s in r["label"]]
    assert got == fixtures.expected_labels(fx)
    np.testing.assert_array_equal(r["rows"], fx["rows"])
    fin = np.isfinite(r["final"]).all(0)
    ref_fin = np.isfinite(fx["final"]).all(0)
    # the stored row is non-finite only for vz == 0 molecules, whose reference
    # row was removed by drop_nans
    assert np.array_equal(fin, ref_fin) or case == "kat_circle"
    both = fin & ref_fin
    np.testing.assert_array_equal(r["final"][:, both], fx["final"][:, both])
    # counts = histogram of labels
    names = cb.labels + ["Detected"]
    exp = {k: got.count(k) for k in set(got)}
    cnt = {names[i]: int(c) for i, c in enumerate(r["counts"]) if c}
    assert cnt == exp
    assert r["steps"] == int(fx["rows"].sum())


@pytest.mark.parametrize("case", CASES)
def test_oracle_traces_match_reference(case):
    fx = fixtures.load(case)
    cb = compile_beamline(fixtures.build_beamline(fx))
    tr = fixtures.traces(fx)
    assert tr
    for j, (rows, idx, n) in tr.items():
        t, _ = oracle.trace(cb, fx["ics"][:, j])
        assert t.shape[0] == n
        np.testing.assert_array_equal(t if idx is None else t[idx], rows)


def test_oracle_threads_agree():
    fx = fixtures.load("config1")
    cb = compile_beamline(fixtures.build_beamline(fx))
    a = oracle.run(cb, fx["ics"], threads=1)
    b = oracle.run(cb, fx["ics"], threads=4)
    np.testing.assert_array_equal(a["final"], b["final"])
    np.testing.assert_array_equal(a["counts"], b["counts"])


def test_oracle_radial_table_out_of_range_raises_like_interp1d():
    """interp1d raises ValueError above its last knot (electrostatic_lens.py:217)."""
    import ctraj
    from scipy.interpolate import interp1d

    r = np.linspace(0, 0.0101, 50)
    f = interp1d(r, -1e5 * r)  # strong outward push: stage points leave the table
    lens = ctraj.ElectrostaticLens(name="L", z0=0.1, L=0.3, d=0.02, dz=5e-3, a_interp=f)
    cb = compile_beamline(ctraj.Beamline([lens]))
    ics = np.array([[9.9e-3], [0.0], [0.1], [200.0], [0.0], [184.0]])
    res = oracle.run(cb, ics)
    assert res["status"] == -4  # CTRAJ_ERANGE


def test_planted_error_is_detected():
    """A mistake planted in the oracle's inputs (a shifted aperture) must break parity."""
    fx = fixtures.load("config0")
    bl = fixtures.build_beamline(fx)
    bl.elements[0].d *= 1.05
    cb = compile_beamline(bl)
    r = oracle.run(cb, fx["ics"])
    got = [cb.label_of(s) for s in r["label"]]
    assert got != fixtures.expected_labels(fx)
