"""Honeycomb mesh element (meshes.py:26-178).

The reference's Honeycomb needs hexalattice and matplotlib, neither of which
is installed; its propagation is pinned through the kat_honeycomb fixture,
made by running the reference's own Honeycomb with stand-ins for those two
packages (tests/golden/make_golden.py) -- the control flow (flights, argmin,
the ``if not idx`` re-lookup, labels) is the reference's, the lattice and the
hexagon test are restatements.  This file checks:

* the package's lattice and hexagon against the fixture script's independent
  restatements (crossing-number polygon test on cos/sin vertices);
* that the device's search window (5 x 5 cells, 4 rows at the grid's ends)
  always holds the nearest and
  second-nearest centre of the reference's argmin over all centres (a numpy
  copy of the window logic against brute force, on CPU);
* the oracle's known answers, among them the ``if not idx`` quirk;
* on the GPU: FP64 bit-exact against the oracle over a wide beam (far
  outside the grid too), FP32 labels off the 1 um edge band, the
  allocation-free entry point, and a honeycomb behind the lens.
"""
from math import ceil

import numpy as np
import pytest

import fixtures
from ctraj.beamline_elements.meshes import Hexagon, Honeycomb, hexalattice_grid
from ctraj.compiler import compile_beamline
from oracle import oracle


def _window_search(xc, yc, nx, inv_row, inv_col, px, py):
    """numpy copy of mesh_nearest64 (csrc/molecule.cuh)."""
    ny = xc.size // nx

    def wi(u, hi):
        r = np.floor(u + 0.5)
        if not r >= 0.0:
            return 0
        return hi if r >= hi else int(r)

    j0 = wi((py - yc[0]) * inv_row, ny - 1)
    lo = max(ny - 4, 0) if j0 == ny - 1 else max(j0 - 2, 0)
    hi = min(3, ny - 1) if j0 == 0 else min(j0 + 2, ny - 1)
    idx, best, second = -1, np.inf, np.inf
    for j in range(lo, hi + 1):
        row = j * nx
        i0 = wi((px - xc[row]) * inv_col, nx - 1)
        for k in range(row + max(i0 - 2, 0), row + min(i0 + 2, nx - 1) + 1):
            dx, dy = px - xc[k], py - yc[k]
            d = np.sqrt(dx * dx + dy * dy)  # numpy's array ** 2 is x * x
            if d < best:
                idx, best, second = k, d, best
            elif d < second:
                second = d
    return max(idx, 0), best, second


@pytest.mark.parametrize("nx,ny", [(19, 22), (1, 1), (1, 5), (6, 1), (2, 2), (7, 4), (10, 9)])
def test_lattice_matches_the_fixture_stand_in(nx, ny):
    import make_golden

    for min_diam in (25.4e-3 / 16 * np.sqrt(3), 1.0, 3.7e-3):
        x, y = hexalattice_grid(nx, ny, min_diam)
        sx, sy = make_golden.stand_in_make_grid(nx, ny, 0, min_diam)
        assert x.shape == (nx * ny, 1) and y.shape == (nx * ny, 1)
        np.testing.assert_array_equal(x, sx)
        np.testing.assert_array_equal(y, sy)


def test_lattice_known_answers():
    h = Honeycomb("H", 0.5, 0.0254)
    lc = 25.4e-3 / 16
    assert (h.nx, h.ny) == (19, 22)
    assert h.xcoords.shape == (19 * 22, 1)
    x, y = h.xcoords.ravel(), h.ycoords.ravel()
    # the centre cell (row ceil(ny/2)-1, column ceil(nx/2)-1) is the origin
    mid = (ceil(22 / 2) - 1) * 19 + ceil(19 / 2) - 1
    assert x[mid] == 0.0 and y[mid] == 0.0
    # cells row by row; odd rows shifted half a pitch; rows sqrt(3)/2 pitch apart
    pitch = lc * np.sqrt(3)
    np.testing.assert_allclose(np.diff(x[:19]), pitch, rtol=1e-12)
    np.testing.assert_allclose(x[19] - x[0], pitch / 2, rtol=1e-12)
    np.testing.assert_allclose(y[19] - y[0], pitch * np.sqrt(3) / 2, rtol=1e-12)
    assert np.all(y[:19] == y[0])
    # the patches: one hexagon per centre with the reference's radius expression
    assert len(h.patches) == 19 * 22
    assert h.patches[0].radius == (lc * np.sqrt(3) - 1e-4 / 2) / 2
    # the grid ignores x0 / y0, as in the reference
    h2 = Honeycomb("H", 0.5, 0.0254, x0=0.01, y0=-0.02)
    np.testing.assert_array_equal(h2.xcoords, h.xcoords)
    assert h2.x1 == 0.01 - 25.4e-3


def test_hexagon_matches_the_crossing_number_stand_in():
    import make_golden

    rng = np.random.default_rng(1)
    for _ in range(20):
        xc, yc, R = rng.normal(size=2).tolist() + [abs(rng.normal()) + 0.1]
        hexagon = Hexagon((np.array([xc]), np.array([yc])), R)
        poly = make_golden.StandInRegularPolygon((np.array([xc]), np.array([yc])), 6, radius=R)
        pts = rng.uniform(-1.3 * R, 1.3 * R, size=(2000, 2)) + [xc, yc]
        for px, py in pts:
            dx, dy = abs(px - xc), abs(py - yc)
            edge = min(abs(R * np.sqrt(3) / 2 - dx), abs(R - dx / np.sqrt(3) - dy) * np.sqrt(3) / 2)
            if edge < 1e-9 * R:
                continue
            assert hexagon.contains_point((px, py)) == poly.contains_point((px, py))
    assert not Hexagon((0.0, 0.0), 1.0).contains_point((np.nan, 0.0))
    assert not Hexagon((0.0, 0.0), 1.0).contains_point((np.inf, 0.0))


@pytest.mark.parametrize("nx,ny", [(19, 22), (1, 1), (1, 6), (5, 1), (2, 3), (8, 8)])
def test_search_window_holds_nearest_and_second(nx, ny):
    pitch = 2.75e-3
    x, y = (a.ravel() for a in hexalattice_grid(nx, ny, pitch))
    inv_row, inv_col = 1.0 / (pitch * np.sqrt(3) / 2), 1.0 / pitch
    rng = np.random.default_rng(nx * 100 + ny)
    span = max(nx, ny) * pitch
    pts = np.concatenate([
        rng.uniform(-0.7 * span, 0.7 * span, size=(3000, 2)),    # on and around the grid
        rng.normal(scale=30 * span, size=(1000, 2)),             # far outside
        np.column_stack([np.cos(a := rng.uniform(0, 2 * np.pi, 3000)), np.sin(a)])
        * np.exp(rng.uniform(np.log(0.5 * span), np.log(1e4 * span), 3000))[:, None],  # all angles
        np.column_stack([np.full(200, 50 * span), rng.uniform(-span, span, 200)]),
        np.column_stack([rng.uniform(-span, span, 200), np.full(200, -50 * span)]),
        np.column_stack([x[:50], y[:50]]),                      # exactly on centres
        np.array([[np.nan, 0.0], [0.0, np.nan], [np.inf, 0.0], [-np.inf, np.inf]]),
    ])
    for px, py in pts:
        d = np.sqrt((px - x) ** 2 + (py - y) ** 2)
        idx, best, second = _window_search(x, y, nx, inv_row, inv_col, px, py)
        assert idx == int(np.argmin(d)), (px, py)
        if np.isfinite(d).any():
            s = np.sort(d)
            assert best == s[0]
            assert second == (s[1] if d.size > 1 else np.inf), (px, py)


def _fixture_beamline():
    fx = fixtures.load("kat_honeycomb")
    return fx, compile_beamline(fixtures.build_beamline(fx))


def test_compiled_element():
    fx, cb = _fixture_beamline()
    from ctraj import _abi

    h = [e for e in fixtures.build_beamline(fx).elements if type(e).__name__ == "Honeycomb"]
    els = [cb.elements[i] for i in range(cb.n_elements) if cb.elements[i].type == _abi.HONEYCOMB]
    assert len(els) == len(h) == 2
    for e, s in zip(h, els):
        assert s.p[0] == e.cell_radius and s.p[1] == e.nx
        t = cb.tables[s.table]
        assert t.kind == _abi.TABLE_MESH
        np.testing.assert_array_equal(t.knots, e.xcoords.ravel())
        np.testing.assert_array_equal(t.values, e.ycoords.ravel())
        assert cb.label_of(s.label) == e.name


def test_oracle_known_answers():
    fx, cb = _fixture_beamline()
    r = oracle.run(cb, fx["ics"][:, :8])
    got = [cb.label_of(s) for s in r["label"]]
    # cell 0 at z0 is looked up again at z1 (`if not idx`): it survives the
    # honeycomb in cell 1 and is lost later at the lens bore; cell 1 -> 2 is lost
    assert got[0] == "Lens entrance" and got[1] == "Honeycomb"
    assert got[2] == "Detected" and got[3] == "Honeycomb"
    assert got[4] == "Lens entrance"
    assert got[5:] == ["Honeycomb"] * 3


def test_oracle_without_the_quirk_would_differ():
    """Planted on the CPU: with the cell of z0 kept (no re-lookup), the first
    known-answer molecule is lost in the honeycomb -- the fixture tells the two
    behaviours apart."""
    fx, cb = _fixture_beamline()
    ic = fx["ics"][:, 0]
    lab = fixtures.expected_labels(fx)[0]
    h = [e for e in fixtures.build_beamline(fx).elements if type(e).__name__ == "Honeycomb"][0]
    x, y = h.xcoords.ravel(), h.ycoords.ravel()
    t = (h.z1 - ic[2]) / ic[5]
    p1 = (ic[0] + ic[3] * t, ic[1] + ic[4] * t - 9.80665 * t * t / 2)
    assert lab == "Lens entrance"
    assert not h.patches[0].contains_point(p1)
    assert h.patches[int(np.argmin(np.hypot(p1[0] - x, p1[1] - y)))].contains_point(p1)


def test_save_to_hdf_skips_the_patches(monkeypatch):
    import sys

    import fake_h5py

    monkeypatch.setitem(sys.modules, "h5py", fake_h5py)
    fake_h5py.STORES.clear()
    h = Honeycomb("Honeycomb", 0.5, 0.0254)
    h.save_to_hdf("mesh.h5", "run/beamline")
    attrs = fake_h5py.snapshot("mesh.h5")["run/beamline/Honeycomb"]["attrs"]
    assert attrs["class"] == "Honeycomb" and "patches" not in attrs
    assert set(attrs) == {"class"} | (set(vars(h)) - {"patches"})
    np.testing.assert_array_equal(attrs["xcoords"], h.xcoords)
    assert attrs["nx"] == 19 and attrs["ny"] == 22


# ---- GPU -----------------------------------------------------------------------


@pytest.fixture(scope="module")
def engine():
    from ctraj.engine import Engine

    e = Engine(0)
    yield e
    e.close()


def _wide_beam(n, seed):
    """A beam wider than the grid, some molecules far outside it."""
    rng = np.random.default_rng(seed)
    ics = np.vstack([rng.normal(0, 12e-3, n), rng.normal(0, 12e-3, n), np.zeros(n),
                     rng.normal(0, 3.0, n), rng.normal(0, 3.0, n), rng.normal(184.0, 16.0, n)])
    far = rng.random(n) < 0.05
    ics[0, far] *= 40.0
    return ics


def _honeycomb_beamline():
    import ctraj

    return ctraj.Beamline([
        Honeycomb("Honeycomb", 0.5, 0.0254),
        Honeycomb("Fine mesh", 0.9, 0.005, width=0.02, height=0.012, cell_wall_length=0.4e-3,
                  cell_wall_thickness=2e-5),
        ctraj.CircularAperture("Detection plane", 1.5, 0.0, d=np.inf),
    ])


@pytest.mark.gpu
def test_fp64_wide_beam_matches_oracle_exactly(engine):
    cb = compile_beamline(_honeycomb_beamline())
    ics = _wide_beam(200_000, 3)
    o = oracle.run(cb, ics, threads=8)
    r = engine.run(cb, ics.shape[1], precision=64, ics=ics, outputs=True)
    np.testing.assert_array_equal(r.label, o["label"])
    np.testing.assert_array_equal(r.rows, o["rows"])
    np.testing.assert_array_equal(r.final, o["final"])
    np.testing.assert_array_equal(r.margin, o["margin"])
    np.testing.assert_array_equal(r.counts, o["counts"])
    names = r.counter_dict()
    assert names.get("Detected", 0) > 0 and names.get("Fine mesh", 0) > 0


@pytest.mark.gpu
@pytest.mark.parametrize("which", ["wide", "fixture"])
def test_fp32_labels_off_the_edge_band(engine, which):
    if which == "wide":
        cb = compile_beamline(_honeycomb_beamline())
        ics = _wide_beam(200_000, 4)
    else:
        fx, cb = _fixture_beamline()
        ics = fx["ics"]
    o = oracle.run(cb, ics, threads=8)
    r = engine.run(cb, ics.shape[1], precision=32, ics=ics, outputs=True)
    far = o["margin"] >= 1e-6
    # far outside the grid two rows' nearest cells are near ties: the band
    # holds a few per cent of the wide beam
    assert far.mean() > 0.95
    np.testing.assert_array_equal(r.label[far], o["label"][far])


@pytest.mark.gpu
def test_noalloc_honeycomb_matches_run(engine):
    import torch
    from test_zz_no_alloc import _compare, _device_outputs, _noalloc

    fx, cb = _fixture_beamline()
    ics = torch.from_numpy(np.ascontiguousarray(fx["ics"])).cuda()
    n = ics.shape[1]
    ref_out = _device_outputs(n)
    ref = engine.run(cb, n, precision=32, ics=ics, device_outputs=ref_out)
    out = _device_outputs(n)
    counts, st = _noalloc(engine.lib, cb, n, ics=ics, outputs=out)
    torch.cuda.synchronize()
    _compare(ref, ref_out, counts, st, out)
