"""Honeycomb mesh element with the reference's dataclass fields and geometry.

Mirrors ``src/trajectories/beamline_elements/meshes.py:26-178``: a grid of
hexagonal cells; a molecule survives when, at z0 and at z1, it lies inside the
hexagon of the cell whose centre was nearest at z0 (looked up again at z1 when
that cell has index 0: the reference tests ``if not idx``, meshes.py:104).

The cell centres come from ``hexalattice.make_grid`` in the reference
(meshes.py:54-62; the reference pins no hexalattice version) and the hexagons
are matplotlib ``RegularPolygon`` patches (meshes.py:71-78).  Neither package
is needed here: ``hexalattice_grid`` restates the published make_grid
algorithm for the arguments the reference passes (n=0, align_to_origin=True,
crop_circ=0, rotate_deg=0) and ``Hexagon`` is the exact pointy-top hexagon a
six-vertex RegularPolygon with orientation 0 describes.  Propagation runs on
the device (element type CTRAJ_HONEYCOMB); ``plot`` and ``plot_mesh`` are out
of scope.
"""
from __future__ import annotations

from dataclasses import dataclass
from math import ceil

import numpy as np

from .apertures import BeamlineElement

__all__ = ["Honeycomb", "Hexagon", "hexalattice_grid"]

SQRT3 = np.sqrt(3)


def hexalattice_grid(nx: int, ny: int, min_diam: float) -> tuple[np.ndarray, np.ndarray]:
    """Centres of an nx x ny hexagonal grid, as (nx*ny, 1) columns x and y.

    hexalattice's make_grid with n=0, crop_circ=0, rotate_deg=0 and
    align_to_origin=True: cell (row j, column i) sits at (i + j%2 / 2,
    j sqrt(3)/2) pitches of min_diam; the grid is then shifted so that the
    centre of cell (ceil(ny/2) - 1, ceil(nx/2) - 1) is the origin (half a
    pitch further right when that row is an odd, shifted one).  Cells are
    numbered row by row (index j * nx + i).  Each product is formed in the
    order the library forms it, so the doubles match.
    """
    nx, ny = int(nx), int(ny)
    row = np.repeat(np.arange(ny), nx)
    col = np.tile(np.arange(nx), ny)
    half = np.sqrt(3) / 2
    x = (col.astype(float) + 0.5 * (row % 2)) * min_diam
    y = (row * half) * min_diam
    mid_row, mid_col = ceil(ny / 2) - 1, ceil(nx / 2) - 1
    mid_x = (float(mid_col) + (0.5 if mid_row % 2 == 1 else 0.0)) * min_diam
    mid_y = (mid_row * half) * min_diam
    return (x - mid_x).reshape(-1, 1), (y - mid_y).reshape(-1, 1)


@dataclass
class Hexagon:
    """A regular hexagon with circumradius ``radius`` centred on ``xy`` and a
    vertex on +y: matplotlib's ``RegularPolygon(xy, 6, radius=radius)``."""

    xy: tuple
    radius: float
    numvertices: int = 6
    orientation: float = 0.0

    def contains_point(self, point) -> bool:
        """Strict interior: |dx| < R sqrt(3)/2 and |dy| < R - |dx|/sqrt(3)
        (the same double operations as the device test)."""
        R = float(self.radius)
        dx = abs(float(point[0]) - float(np.ravel(self.xy[0])[0]))
        dy = abs(float(point[1]) - float(np.ravel(self.xy[1])[0]))
        return bool(dx < R * SQRT3 / 2.0 and dy < R - dx / SQRT3)


@dataclass
class Honeycomb(BeamlineElement):
    """meshes.py:26-65: width x height of hexagonal cells with wall length
    ``cell_wall_length`` (the hexagon side) and wall thickness
    ``cell_wall_thickness``.  Like the reference, the grid is centred on the
    beam axis whatever x0 and y0 are."""

    width: float = 2 * 25.4e-3
    height: float = 2 * 25.4e-3
    cell_wall_thickness: float = 1e-4
    cell_wall_length: float = 25.4e-3 / 16

    def __post_init__(self):
        super().__post_init__()
        self.x1 = self.x0 - self.width / 2
        self.x2 = self.x0 + self.width / 2
        self.y1 = self.y0 - self.height / 2
        self.y2 = self.y0 + self.height / 2
        self.nx = ceil(self.width / (self.cell_wall_length * np.sqrt(3)))
        self.ny = ceil(self.height / (self.cell_wall_length * 3 / 2))
        self.xcoords, self.ycoords = hexalattice_grid(self.nx, self.ny, self.cell_wall_length * np.sqrt(3))
        self.patches = self.make_patches()

    @property
    def cell_radius(self) -> float:
        """Circumradius of each cell's hexagon (meshes.py:76-79)."""
        return (self.cell_wall_length * np.sqrt(3) - self.cell_wall_thickness / 2) / 2

    def make_patches(self) -> list:
        """One hexagon per cell centre (meshes.py:67-83)."""
        R = self.cell_radius
        return [Hexagon((x, y), R) for x, y in zip(self.xcoords, self.ycoords)]

    def N_steps(self) -> int:
        return 2

    def save_to_hdf(self, filepath, parent_group_path: str) -> None:
        """meshes.py:156-178: the element's fields without the patches."""
        from ..hdf import save_element

        save_element(self, filepath, parent_group_path, skip=("patches",))
