"""Generate golden fixtures by running the reference itself.

Run where the reference is checked out (its src directory given by
--reference-src or CTRAJ_REFERENCE_SRC); the GPU machines never run this, they only read the .npz
files it writes next to itself.

    python tests/golden/make_golden.py --reference-src <reference>/src

For every case it builds the case's beamline from the reference's own classes,
injects seeded initial conditions straight into ``Molecule.init_trajectory``
(the reference's ``Distribution.draw`` has no seed, distributions.py:41) and
calls ``Beamline.propagate_through`` exactly as trajectory_simulator.py:62-72
does.  Stored per molecule: the label (``aperture_hit``), the last trajectory
row after ``drop_nans`` (x, v, a, t), ``len(trajectory.t) - 1``; plus full
row traces for a few molecules.

The lens force is injected through the public ``a_interp`` field
(electrostatic_lens.py:32, used only as ``self.a_interp(r)`` at :217):

* "stark_spline" lenses get a_r(r) = -(W'(E) * dE/dr) / m with |E| = alpha r^n
  and W' from a scipy CubicSpline of the two-level Stark curve;
* "radial_linear" lenses get the reference's own interp1d construction
  (:194-209) with the two-level curve standing in for ``stark_potential``
  (centrex_TlF is not installed).

A lens with ``dt`` in its spec realises a fixed time step the only way the
reference allows: ``lens.dz = vz * dt`` set per molecule before
``init_trajectory`` (dt = dz / vz at :88).
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parent))
import refstubs  # noqa: E402

HERE = Path(__file__).resolve().parent
M_PER_IN = 0.0254
INF = float("inf")

# ---- Stark tables ----------------------------------------------------------


def two_level(splitting_hz, dipole_debye, sign=-1.0):
    from scipy.constants import c, h

    a = h * splitting_hz
    d = dipole_debye * 1e-21 / c

    def W(E):
        return sign * (np.sqrt(a * a + (d * E) ** 2) - a)

    return W


def make_tables():
    from scipy.interpolate import CubicSpline, interp1d

    tables = {}
    # hexapole workload: 4096 knots over 0..1e7 V/m, W = -(sqrt(a^2+(dE)^2) - a)
    E = np.linspace(0.0, 1e7, 4096)
    sp = CubicSpline(E, two_level(6.7e9, 4.2)(E))
    tables["hex"] = dict(kind="stark_spline", knots=sp.x.copy(), coef=np.ascontiguousarray(sp.c.T),
                         spline=sp)
    # reference-style radial table (electrostatic_lens.py:194-209), low-field seeker
    d, V, mass, dr = 1.75 * M_PER_IN, 27.6e3, (204.38 + 19.00) * 1.67e-27, 1e-4
    r_values = np.linspace(0, d / 2 * 1.01, int(np.round(d / 2 / dr)))
    E_values = 2 * V / ((d / 2) ** 2) * r_values
    a_values = -np.gradient(two_level(6.7e9, 4.2, sign=+1.0)(E_values), dr) / mass
    tables["radial"] = dict(kind="radial_linear", knots=r_values, values=a_values,
                            interp=interp1d(r_values, a_values))
    # small hexapole table for the known-answer lens
    E2 = np.linspace(0.0, 2e7, 1024)
    sp2 = CubicSpline(E2, two_level(13.3e9, 4.2, sign=+1.0)(E2))
    tables["hex_kat"] = dict(kind="stark_spline", knots=sp2.x.copy(), coef=np.ascontiguousarray(sp2.c.T),
                             spline=sp2)
    return tables


def spline_a_interp(spline, V, R, mass, order):
    """a_r(r) for |E| = alpha r^n; the expression order is what the device FP64 path follows."""
    if order == 2:
        alpha = 3.0 * V / R ** 3

        def a_interp(r):
            E = alpha * (r * r)
            return -(spline(E, 1) * (2.0 * alpha * r)) / mass
    else:
        alpha = 2.0 * V / R ** 2

        def a_interp(r):
            E = alpha * r
            return -(spline(E, 1) * alpha) / mass
    return a_interp


# ---- cases ------------------------------------------------------------------

TLF_MASS = (204.38 + 19.00) * 1.67e-27


def config0_elements():
    return [
        dict(cls="CircularAperture", name="A1", z0=0.30, L=1e-3, d=12e-3),
        dict(cls="RectangularAperture", name="R1", z0=1.00, L=1e-3, w=10e-3, h=8e-3),
        dict(cls="CircularAperture", name="A2", z0=2.00, L=1e-3, d=20e-3),
        dict(cls="CircularAperture", name="Detection plane", z0=3.00, L=0.0, d=INF),
    ]


def config1_elements():
    return [
        dict(cls="CircularAperture", name="A1", z0=0.30, L=1e-3, d=12e-3),
        dict(cls="ElectrostaticLens", name="ES lens", z0=0.80, L=0.60, d=35e-3, V=30e3, dt=1e-6,
             force=dict(table="hex", V=30e3, R=17.5e-3, mass=TLF_MASS, order=2)),
        dict(cls="CircularAperture", name="Detection plane", z0=3.00, L=0.0, d=INF),
    ]


def example_elements():
    """The lens beamline of examples/lens_simulation_beamline.py:21-59 (reference default lens)."""
    fourK = dict(cls="CircularAperture", z0=1.7 * M_PER_IN, L=0.25 * M_PER_IN, d=1 * M_PER_IN,
                 name="4K shield")
    z = fourK["z0"] + fourK["L"]
    fortyK = dict(cls="CircularAperture", z0=z + 1.25 * M_PER_IN, L=0.25 * M_PER_IN, d=1 * M_PER_IN,
                  name="40K shield")
    z = fortyK["z0"] + fortyK["L"]
    bb = dict(cls="CircularAperture", z0=z + 2.5 * M_PER_IN, L=0.75 * M_PER_IN, d=4 * M_PER_IN,
              name="BB exit")
    z_bb1 = bb["z0"] + bb["L"]
    lens = dict(cls="ElectrostaticLens", z0=z_bb1 + 33 * M_PER_IN, L=0.6, name="ES lens",
                force=dict(table="radial"))
    fp = dict(cls="FieldPlates", z0=2.43, L=3.0, w=0.02, name="Field plates")
    dr = dict(cls="RectangularAperture", z0=2.43 + 3.0 + 39.9 * M_PER_IN, L=0.25 * M_PER_IN,
              name="DR aperture", w=0.018, h=0.03)
    return [fourK, fortyK, bb, lens, fp, dr]


def kat_cases():
    """Hand-built known-answer cases, each on its own short beamline."""
    cases = {}
    cases["kat_circle"] = dict(
        elements=[dict(cls="CircularAperture", name="C1", z0=0.5, L=0.01, d=10e-3)],
        ics=np.array([
            # exactly on the edge at z0 (dt = 0 keeps the state; rho == d/2 survives), lost at z1
            [5e-3, 0.0, 0.5, 0.0, 0.0, 184.0],
            [0.0, -5e-3, 0.5, 0.0, 0.0, 184.0],
            [3e-3, 4e-3, 0.5, 0.0, 0.0, 184.0],
            # just inside / outside
            [4.999999e-3, 0.0, 0.0, 0.0, 0.0, 184.0],
            [5.000001e-3, 0.0, 0.5, 0.0, 0.0, 184.0],
            # backward flight (vz < 0) and a molecule that never moves in z (vz == 0)
            [1e-3, 1e-3, 0.0, 1.0, 1.0, -184.0],
            [1e-3, 1e-3, 0.0, 1.0, 1.0, 0.0],
            [1e-3, 1e-3, 0.5, 1.0, 1.0, 0.0],
        ]).T)
    cases["kat_rect"] = dict(
        elements=[dict(cls="RectangularAperture", name="R1", z0=1.0, L=0.01, w=8e-3, h=6e-3)],
        ics=np.array([
            [-4e-3, 0.0, 1.0, 0.0, 0.0, 184.0],   # x == x1: lost (strict)
            [4e-3, 0.0, 1.0, 0.0, 0.0, 184.0],    # x == x2: lost
            [0.0, 3e-3, 1.0, 0.0, 0.0, 184.0],    # y == y2: lost
            [0.0, -3e-3, 1.0, 0.0, 0.0, 184.0],   # y == y1: lost
            [0.0, 2.9999e-3, 1.0, 0.0, 0.0, 184.0],  # inside at z0, gravity keeps it inside
            [3.9e-3, 0.0, 1.0, 30.0, 0.0, 184.0],  # leaves through x2 between z0 and z1
            [0.0, 0.0, 0.0, 0.0, 0.0, 184.0],
        ]).T)
    cases["kat_plates"] = dict(
        elements=[dict(cls="FieldPlates", name="FP", z0=1.5, L=0.5, w=6e-3)],
        ics=np.array([
            [0.0, 0.0, 1.5, 2.0, 0.0, 184.0],    # hits x2 inside the plates
            [0.0, 0.0, 1.5, -2.0, 0.0, 184.0],   # hits x1
            [0.0, 0.0, 1.5, 0.5, 0.0, 184.0],    # passes
            [3e-3, 0.0, 1.5, 0.0, 0.0, 184.0],   # x == x2 at z0: lost at z0
            [0.0, 0.0, 0.0, 0.0, 1.0, 184.0],    # y is not checked by the plates
        ]).T)
    lens = dict(cls="ElectrostaticLens", name="ES lens", z0=2.2, L=0.3, d=0.02, dz=1e-3, V=20e3,
                force=dict(table="hex_kat", V=20e3, R=0.01, mass=TLF_MASS, order=2))
    cases["kat_lens"] = dict(
        elements=[lens, dict(cls="CircularAperture", name="Detection plane", z0=3.0, L=0.0, d=INF)],
        ics=np.array([
            [0.0101, 0.0, 2.2, 0.0, 0.0, 184.0],    # lens entrance
            [9e-3, 0.0, 2.2, 20.0, 0.0, 184.0],     # inside lens
            [1e-4, 0.0, 2.2, 0.0, 0.0, 184.0],      # survives (focusing)
            [2e-3, 1e-3, 2.2, -1.0, 0.5, 150.0],
            [0.0, 0.0, 2.2, 0.0, 0.0, 184.0],       # on axis: r == 0 branch
            [1e-3, 1e-3, 0.0, 0.0, 0.0, -184.0],    # negative vz: N = rint(L/dz) with dz fixed
        ]).T)
    cases["kat_honeycomb"] = honeycomb_case()
    # the classic-RK4 scheme and field order 1 are extensions: no reference output exists
    return cases


# ---- honeycomb (meshes.py) ---------------------------------------------------
#
# The reference's Honeycomb takes its cell centres from hexalattice.make_grid
# and its hexagons from matplotlib.patches.RegularPolygon; neither package is
# installed.  Stand-ins restating both are installed into the reference's
# meshes module, so its own __post_init__ (nx, ny, patch radius) and
# propagate_through (flights, argmin, the `if not idx` re-lookup, labels) run.
# The fixture therefore pins that control flow and arithmetic, and checks the
# product's lattice and hexagon test against these independent restatements
# (a polygon crossing-number test on cos/sin vertices, like matplotlib's
# point_in_path); it does not pin hexalattice or matplotlib themselves.

HALF_SQRT3 = np.sqrt(3) / 2


def stand_in_make_grid(nx, ny, n=0, min_diam=1.0, align_to_origin=True, crop_circ=0.0, rotate_deg=0.0):
    """hexalattice make_grid for the arguments meshes.py:54-62 passes: rows of nx
    cells (odd rows shifted half a pitch), the centre cell moved to the origin."""
    import math

    assert n == 0 and align_to_origin and crop_circ == 0 and rotate_deg == 0
    mid_row, mid_col = math.ceil(ny / 2) - 1, math.ceil(nx / 2) - 1
    mid_x = (mid_col + (0.5 if mid_row % 2 else 0.0)) * min_diam
    mid_y = (mid_row * HALF_SQRT3) * min_diam
    xs, ys = [], []
    for j in range(ny):
        for i in range(nx):
            xs.append((i + (0.5 if j % 2 else 0.0)) * min_diam - mid_x)
            ys.append((j * HALF_SQRT3) * min_diam - mid_y)
    return np.array(xs).reshape(-1, 1), np.array(ys).reshape(-1, 1)


class StandInRegularPolygon:
    """matplotlib RegularPolygon(xy, numVertices, radius) with orientation 0:
    vertices at angles pi/2 + 2 pi k / n; contains_point by crossing number."""

    def __init__(self, xy, numVertices, radius=5.0, orientation=0.0, **kwargs):
        x0, y0 = (float(np.ravel(v)[0]) for v in xy)
        th = np.pi / 2 + 2 * np.pi / numVertices * np.arange(numVertices) + orientation
        self.vx = radius * np.cos(th) + x0
        self.vy = radius * np.sin(th) + y0

    def contains_point(self, point):
        px, py = float(point[0]), float(point[1])
        if not (np.isfinite(px) and np.isfinite(py)):
            return False
        inside = False
        j = len(self.vx) - 1
        for i in range(len(self.vx)):
            if (self.vy[i] > py) != (self.vy[j] > py):
                xc = (self.vx[j] - self.vx[i]) * (py - self.vy[i]) / (self.vy[j] - self.vy[i]) + self.vx[i]
                if px < xc:
                    inside = not inside
            j = i
        return inside


def install_mesh_stand_ins():
    import trajectories.beamline_elements.meshes as meshes

    meshes.hexalattice.make_grid = stand_in_make_grid
    meshes.RegularPolygon = StandInRegularPolygon


def honeycomb_case():
    """Aperture, honeycomb, lens, a coarser honeycomb behind the lens, plane."""
    lc = 25.4e-3 / 16
    hc0, hc_len, vz = 0.5, 0.0254, 184.0
    nx = int(np.ceil(2 * 25.4e-3 / (lc * np.sqrt(3))))
    ny = int(np.ceil(2 * 25.4e-3 / (lc * 3 / 2)))
    xc, yc = (a.ravel() for a in stand_in_make_grid(nx, ny, 0, lc * np.sqrt(3)))
    t_fly = hc_len / vz
    mid = (int(np.ceil(ny / 2)) - 1) * nx + int(np.ceil(nx / 2)) - 1

    def hop(a, b, dx=2e-4, dy=1e-4):
        """starts near cell a's centre at z0, reaches cell b's centre at z1"""
        x0, y0 = xc[a] + dx, yc[a] + dy
        return [x0, y0, hc0, (xc[b] - x0) / t_fly, (yc[b] - y0) / t_fly, vz]

    known = np.array([
        hop(0, 1),               # cell 0 at z0: looked up again at z1, survives in cell 1
        hop(1, 2),               # cell 1 keeps its index: outside it at z1, lost
        hop(mid, mid),           # centre cell, straight through
        hop(mid, mid + 1),       # drifts into the neighbour: lost
        hop(0, 0, 0.0, 0.0),     # centre of cell 0
        [0.028, 0.0, hc0, 0.0, 0.0, vz],    # outside the grid, inside the aperture: lost
        [-0.027, 0.026, hc0, 0.0, 0.0, vz],  # beyond a corner: lost
        [xc[mid] + 1.25e-3, yc[mid], hc0, 0.0, 0.0, vz],  # in the wall band between cells: lost
    ]).T
    rng = np.random.default_rng(7)
    beam = draw_ics(rng, 1500, 6e-3, 6e-3, 0.0, 4.0, 4.0, 184.0, 12.0)
    lens = dict(cls="ElectrostaticLens", name="ES lens", z0=1.0, L=0.3, d=0.03, dz=1e-3, V=20e3,
                force=dict(table="hex_kat", V=20e3, R=0.015, mass=TLF_MASS, order=2))
    return dict(
        elements=[
            dict(cls="CircularAperture", name="Aperture", z0=0.2, L=0.005, d=0.15),
            dict(cls="Honeycomb", name="Honeycomb", z0=hc0, L=hc_len),
            lens,
            dict(cls="Honeycomb", name="Honeycomb 2", z0=1.6, L=0.01, width=0.03, height=0.03,
                 cell_wall_length=25.4e-3 / 8, cell_wall_thickness=2e-4),
            dict(cls="CircularAperture", name="Detection plane", z0=2.0, L=0.0, d=INF),
        ],
        ics=np.hstack([known, beam]))


def draw_ics(rng, n, sx, sy, z, svx, svy, vz, svz):
    """Velocity first, then position (trajectory_simulator.py:57-58)."""
    vx = rng.normal(0.0, svx, n)
    vy = rng.normal(0.0, svy, n)
    vzs = rng.normal(vz, svz, n)
    x = rng.normal(0.0, sx, n)
    y = rng.normal(0.0, sy, n)
    return np.vstack((x, y, np.full(n, z), vx, vy, vzs))


def draw_disc_ics(rng, n, d, z, svx, svy, vz, svz):
    vx = rng.normal(0.0, svx, n)
    vy = rng.normal(0.0, svy, n)
    vzs = rng.normal(vz, svz, n)
    theta = rng.uniform(size=n) * 2 * np.pi
    r = np.sqrt(rng.uniform(size=n)) * d / 2
    return np.vstack((r * np.cos(theta), r * np.sin(theta), np.full(n, z), vx, vy, vzs))


def build_cases(quick=False):
    rng = np.random.default_rng(0)
    k = 10 if quick else 1
    cases = {}
    # config 0: plain ballistic beamline, FP64
    ics = np.hstack([draw_ics(rng, 3000 // k, 1.5e-3, 1.5e-3, 0.0, 20.0, 20.0, 184.0, 16.0),
                     draw_ics(rng, 1500 // k, 1.5e-3, 1.5e-3, 0.0, 3.0, 3.0, 184.0, 16.0)])
    cases["config0"] = dict(elements=config0_elements(), ics=ics, trace=12)
    # config 1: aperture + hexapole lens with dt = 1 us
    ics = np.hstack([draw_ics(rng, 2000 // k, 1.5e-3, 1.5e-3, 0.0, 20.0, 20.0, 184.0, 16.0),
                     draw_ics(rng, 300 // k, 1.0e-3, 1.0e-3, 0.0, 2.0, 2.0, 184.0, 16.0)])
    cases["config1"] = dict(elements=config1_elements(), ics=ics, trace=4)
    # the reference's example beamline with its default lens (dz = 1 mm, interp1d table)
    ics = np.hstack([draw_disc_ics(rng, 2000 // k, 0.02, 0.25 * M_PER_IN, 39.5, 39.5, 184.0, 16.0),
                     draw_disc_ics(rng, 300 // k, 0.02, 0.25 * M_PER_IN, 2.0, 2.0, 184.0, 16.0)])
    cases["example_lens"] = dict(elements=example_elements(), ics=ics, trace=4)
    for name, c in kat_cases().items():
        c["trace"] = c["ics"].shape[1]
        cases[name] = c
    return cases


# ---- reference runner -------------------------------------------------------


def build_reference_beamline(specs, tables):
    from trajectories.beamline import Beamline
    from trajectories.beamline_elements.apertures import (CircularAperture, FieldPlates,
                                                          RectangularAperture)
    from trajectories.beamline_elements.electrostatic_lens import ElectrostaticLens
    from trajectories.beamline_elements.meshes import Honeycomb

    classes = dict(CircularAperture=CircularAperture, RectangularAperture=RectangularAperture,
                   FieldPlates=FieldPlates, ElectrostaticLens=ElectrostaticLens, Honeycomb=Honeycomb)
    elems = []
    for s in specs:
        kw = {k: v for k, v in s.items() if k not in ("cls", "force", "dt")}
        if s["cls"] == "ElectrostaticLens":
            f = s["force"]
            tab = tables[f["table"]]
            if tab["kind"] == "stark_spline":
                kw["a_interp"] = spline_a_interp(tab["spline"], f["V"], f["R"], f["mass"], f["order"])
            else:
                kw["a_interp"] = tab["interp"]
        elems.append(classes[s["cls"]](**kw))
    return Beamline(elems)


def run_reference(specs, tables, ics, n_trace):
    from trajectories.molecule import Molecule

    beamline = build_reference_beamline(specs, tables)
    lenses = [(e, s) for e, s in zip(beamline.elements, sorted(specs, key=lambda s: s["z0"]))
              if s["cls"] == "ElectrostaticLens"]
    n = ics.shape[1]
    labels, final, rows, traces = [], np.full((10, n), np.nan), np.zeros(n, np.int32), []
    for i in range(n):
        for e, s in lenses:
            if s.get("dt") is not None:
                e.dz = ics[5, i] * s["dt"]
        m = Molecule()
        m.init_trajectory(beamline, ics[:3, i], ics[3:, i])
        try:
            beamline.propagate_through(m)
            labels.append(m.aperture_hit)
        except ValueError:
            labels.append("__error__")
            m.trajectory.drop_nans()
        tr = m.trajectory
        rows[i] = len(tr.t) - 1
        if len(tr.t):
            final[:, i] = np.concatenate([tr.x[-1], tr.v[-1], tr.a[-1], [tr.t[-1]]])
        if i < n_trace:
            same = len(tr.x) == len(tr.v) == len(tr.a) == len(tr.t)
            t = np.column_stack([tr.x, tr.v, tr.a, tr.t]) if same else None
            traces.append(t)
    return labels, final, rows, traces


def main():
    ap = argparse.ArgumentParser()
    refstubs.add_argument(ap)
    ap.add_argument("--only", nargs="*")
    ap.add_argument("--quick", action="store_true", help="10x fewer molecules (smoke)")
    args = ap.parse_args()
    refstubs.install(refstubs.require(args.reference_src))
    install_mesh_stand_ins()
    import numpy
    import scipy

    tables = make_tables()
    cases = build_cases(args.quick)
    for name, c in cases.items():
        if args.only and name not in args.only:
            continue
        t0 = time.time()
        labels, final, rows, traces = run_reference(c["elements"], tables, c["ics"], c["trace"])
        names = sorted(set(labels))
        out = dict(ics=c["ics"], label_names=np.array(names), label=np.array([names.index(s) for s in labels],
                   np.int32), final=final, rows=rows,
                   spec=np.array(json.dumps(dict(elements=c["elements"]))),
                   versions=np.array(json.dumps(dict(numpy=numpy.__version__, scipy=scipy.__version__,
                                                     python=sys.version.split()[0]))))
        used = {e["force"]["table"] for e in c["elements"] if "force" in e}
        for tname in used:
            tab = tables[tname]
            out[f"table_{tname}_knots"] = tab["knots"]
            if tab["kind"] == "stark_spline":
                out[f"table_{tname}_coef"] = tab["coef"]
            else:
                out[f"table_{tname}_values"] = tab["values"]
        for j, t in enumerate(traces):
            if t is None:
                continue
            if t.shape[0] > 400:  # long lens traces: every 50th row plus the last three
                idx = np.unique(np.concatenate([np.arange(0, t.shape[0], 50), np.arange(t.shape[0] - 3, t.shape[0])]))
                out[f"trace_{j}_idx"] = idx.astype(np.int32)
                out[f"trace_{j}"] = t[idx]
                out[f"trace_{j}_len"] = np.int64(t.shape[0])
            else:
                out[f"trace_{j}"] = t
        np.savez_compressed(HERE / f"{name}.npz", **out)
        print(f"{name}: {c['ics'].shape[1]} molecules in {time.time() - t0:.1f}s, labels "
              + ", ".join(f"{s}={labels.count(s)}" for s in names), flush=True)


if __name__ == "__main__":
    main()
