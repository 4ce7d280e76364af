"""Beamline compiler: reference-style element objects -> C ABI element table.

Walks ``beamline.elements`` in their stored order (the reference sorts them
by z0 once, in ``Beamline.__post_init__``, beamline.py:17-18,40-45) and emits
one ``ctraj_element`` each, duck-typed on the class name so the reference's own
objects and this package's mirrors both compile.  It also builds the counter
label table, reproducing the strings the reference credits:

* apertures, field plates and honeycombs: ``element.name`` (apertures.py:113,188,242,264,
  meshes.py:114)
* electrostatic lens: "Lens entrance" and "Inside lens" (electrostatic_lens.py:63,117)
* survivors: "Detected" (beamline.py:34-35), the last count slot

An element type without a device implementation raises TypeError: there is no
CPU fallback.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Any, List

import numpy as np

from . import _abi
from .stark import StarkForce

LENS_ENTRANCE = "Lens entrance"
INSIDE_LENS = "Inside lens"
DETECTED = "Detected"


@dataclass
class Table:
    kind: int
    knots: np.ndarray
    coef: np.ndarray | None = None
    values: np.ndarray | None = None

    def as_struct(self) -> _abi.ForceTable:
        t = _abi.ForceTable()
        t.kind = self.kind
        t.n_knots = int(self.knots.size)
        t.knots = _abi.f64ptr(self.knots)
        t.coef = _abi.f64ptr(self.coef) if self.coef is not None else None
        t.values = _abi.f64ptr(self.values) if self.values is not None else None
        return t


@dataclass
class CompiledBeamline:
    elements: Any                      # ctypes array of _abi.Element
    labels: List[str]                  # counter slot -> label string
    tables: List[Table] = field(default_factory=list)
    n_lenses: int = 0
    max_rows: int = 10                 # reference Trajectory rows (molecule.py:118-122)

    @property
    def n_elements(self) -> int:
        return len(self.elements)

    def table_structs(self):
        arr = (_abi.ForceTable * max(1, len(self.tables)))()
        for i, t in enumerate(self.tables):
            arr[i] = t.as_struct()
        return arr

    def label_of(self, slot: int) -> str:
        return DETECTED if slot < 0 or slot >= len(self.labels) else self.labels[slot]


def _table_from_interp1d(f) -> Table:
    kind = getattr(f, "_kind", getattr(f, "kind", "linear"))
    if kind != "linear":
        raise TypeError(f"interp1d kind {kind!r} has no device implementation (only 'linear')")
    if not getattr(f, "bounds_error", True):
        raise TypeError("interp1d with bounds_error=False has no device implementation")
    x = np.ascontiguousarray(np.asarray(f.x, dtype=np.float64))
    y = np.ascontiguousarray(np.asarray(f.y, dtype=np.float64).reshape(-1))
    if x.ndim != 1 or y.size != x.size or x.size < 2:
        raise TypeError("interp1d table must be 1-D with at least two knots")
    dx = np.diff(x)
    if not np.allclose(dx, dx[0], rtol=1e-9, atol=0.0) or dx[0] <= 0:
        raise TypeError("interp1d knots must be ascending and uniformly spaced")
    return Table(_abi.TABLE_RADIAL_LINEAR, x, values=y)


def _lens_table(lens) -> tuple[Table, StarkForce | None]:
    f = lens.a_interp
    if f is None:
        raise ValueError(
            f"ElectrostaticLens {lens.name!r}: a_interp is None. Building a Stark table from the "
            "TlF Hamiltonian needs centrex_TlF; pass a ctraj.stark.StarkForce or an interp1d.")
    if isinstance(f, StarkForce) or type(f).__name__ == "StarkForce":
        return Table(_abi.TABLE_STARK_SPLINE, np.ascontiguousarray(f.knots, np.float64),
                     coef=np.ascontiguousarray(f.coef, np.float64)), f
    if type(f).__name__ == "interp1d":
        return _table_from_interp1d(f), None
    raise TypeError(f"ElectrostaticLens.a_interp of type {type(f).__name__} has no device "
                    "implementation (use StarkForce or scipy interp1d)")


def compile_beamline(beamline) -> CompiledBeamline:
    elems = list(beamline.elements)
    if len(elems) > _abi.MAX_ELEMENTS:
        raise ValueError(f"at most {_abi.MAX_ELEMENTS} elements are supported")
    labels: List[str] = []

    def slot(name: str) -> int:
        if name == DETECTED:
            return -1  # merges with the survivors' key, as the reference's dict would
        if name not in labels:
            labels.append(name)
        return labels.index(name)

    arr = (_abi.Element * max(1, len(elems)))()
    tables: List[Table] = []
    table_ids: dict[int, int] = {}
    n_lenses = 0
    max_rows = 10
    for i, e in enumerate(elems):
        kind = type(e).__name__
        s = _abi.Element()
        s.z0 = float(e.z0)
        s.z1 = float(e.z1)
        s.x0 = float(e.x0)
        s.y0 = float(e.y0)
        s.label = -1
        s.label_inside = -1
        s.table = -1
        if kind == "CircularAperture":
            s.type = _abi.CIRCULAR_APERTURE
            s.label = slot(e.name)
            s.p[0] = float(e.d)
            max_rows += 2
        elif kind == "RectangularAperture":
            s.type = _abi.RECTANGULAR_APERTURE
            s.label = slot(e.name)
            s.p[0], s.p[1], s.p[2], s.p[3] = float(e.x1), float(e.x2), float(e.y1), float(e.y2)
            max_rows += 2
        elif kind == "FieldPlates":
            s.type = _abi.FIELD_PLATES
            s.label = slot(e.name)
            s.p[0], s.p[1] = float(e.x1), float(e.x2)
            max_rows += 2
        elif kind == "ElectrostaticLens":
            s.type = _abi.ELECTROSTATIC_LENS
            s.label = slot(LENS_ENTRANCE)
            s.label_inside = slot(INSIDE_LENS)
            table, force = _lens_table(e)
            key = id(e.a_interp)
            if key not in table_ids:
                if len(tables) >= _abi.MAX_TABLES:
                    raise ValueError(f"at most {_abi.MAX_TABLES} distinct force tables")
                table_ids[key] = len(tables)
                tables.append(table)
            s.table = table_ids[key]
            dt = getattr(e, "dt", None)
            s.step_mode = _abi.STEP_DT if dt is not None else _abi.STEP_DZ
            scheme = getattr(e, "scheme", "reference")
            if scheme not in ("reference", "classic"):
                raise ValueError(f"unknown RK4 scheme {scheme!r}")
            s.scheme = _abi.RK4_CLASSIC if scheme == "classic" else _abi.RK4_REFERENCE
            s.p[0] = float(e.d)
            s.p[1] = float(e.dz)
            s.p[2] = float(dt) if dt is not None else 0.0
            s.p[7] = float(e.L)
            if force is not None:
                s.field_order = int(force.field_order)
                s.p[3] = float(force.V)
                s.p[4] = float(force.R)
                s.p[5] = float(force.mass)
                s.p[6] = float(force.alpha)
            else:
                s.field_order = 0
                s.p[3] = float(e.V)
                s.p[4] = float(e.d) / 2
                s.p[5] = float(e.mass)
            n_lenses += 1
            if dt is None:
                max_rows += 1 + int(np.rint(e.L / e.dz))
            else:
                max_rows += 1  # per-molecule step count; recording sizes it from vz
        elif kind == "Honeycomb":
            s.type = _abi.HONEYCOMB
            s.label = slot(e.name)
            xc = np.ascontiguousarray(np.asarray(e.xcoords, np.float64).reshape(-1))
            yc = np.ascontiguousarray(np.asarray(e.ycoords, np.float64).reshape(-1))
            nx, ny = int(e.nx), int(e.ny)
            if xc.size != nx * ny or yc.size != xc.size:
                raise ValueError(f"Honeycomb {e.name!r}: {xc.size} centres for a {nx} x {ny} grid")
            if len(tables) >= _abi.MAX_TABLES:
                raise ValueError(f"at most {_abi.MAX_TABLES} distinct force and mesh tables")
            s.table = len(tables)
            tables.append(Table(_abi.TABLE_MESH, xc, values=yc))
            pitch = float(e.cell_wall_length * np.sqrt(3))  # hexalattice min_diam
            s.p[0] = float((e.cell_wall_length * np.sqrt(3) - e.cell_wall_thickness / 2) / 2)
            s.p[1] = float(nx)
            s.p[2] = 1.0 / (pitch * np.sqrt(3) / 2)
            s.p[3] = 1.0 / pitch
            max_rows += 2
        else:
            raise TypeError(f"beamline element type {kind} has no device implementation")
        arr[i] = s
    if len(labels) > _abi.MAX_LABELS:
        raise ValueError(f"at most {_abi.MAX_LABELS} distinct labels")
    return CompiledBeamline(elements=arr, labels=labels, tables=tables, n_lenses=n_lenses,
                            max_rows=max_rows)
