"""Beamline elements with the reference's dataclass fields and geometry.

Mirrors ``src/trajectories/beamline_elements/apertures.py``: the same class
names, fields, defaults and ``__post_init__`` geometry, so a beamline written
for the reference builds unchanged.  Propagation itself is not done here: the
compiler (``ctraj.compiler``) turns elements into the C ABI's element table and
the CUDA kernels propagate.  ``plot``/``save_to_hdf`` of the reference are out
of scope.
"""
from __future__ import annotations

from dataclasses import dataclass

__all__ = ["BeamlineElement", "CircularAperture", "RectangularAperture", "FieldPlates"]


@dataclass
class BeamlineElement:
    """Base element, apertures.py:22-36: name, z0, L, x0, y0 and z1 = z0 + L."""

    name: str
    z0: float
    L: float
    x0: float = 0.0
    y0: float = 0.0

    def __post_init__(self):
        self.z1 = self.z0 + self.L

    def N_steps(self) -> int:  # pragma: no cover - overridden
        raise NotImplementedError

    def save_to_hdf(self, filepath, parent_group_path: str) -> None:
        """apertures.py:56-78: group parent/name with attrs class and the fields."""
        from ..hdf import save_element

        save_element(self, filepath, parent_group_path)


@dataclass
class CircularAperture(BeamlineElement):
    """apertures.py:83-122: a molecule is lost iff sqrt(x^2 + y^2) > d/2 at z0 or z1."""

    d: float = 0.0254

    def N_steps(self) -> int:
        return 2


@dataclass
class RectangularAperture(BeamlineElement):
    """apertures.py:147-196: alive iff x1 < x < x2 and y1 < y < y2 at z0 and z1.

    As in the reference, ``w`` spans X and ``h`` spans Y (apertures.py:160-163).
    """

    w: float = 0.02
    h: float = 0.02

    def __post_init__(self):
        super().__post_init__()
        self.x1 = self.x0 - self.w / 2
        self.x2 = self.x0 + self.w / 2
        self.y1 = self.y0 - self.h / 2
        self.y2 = self.y0 + self.h / 2

    def N_steps(self) -> int:
        return 2


@dataclass
class FieldPlates(BeamlineElement):
    """apertures.py:213-277: X-only slab between x1 and x2 from z0 to z1."""

    w: float = 0.02

    def __post_init__(self):
        super().__post_init__()
        self.x1 = self.x0 - self.w / 2
        self.x2 = self.x0 + self.w / 2

    def N_steps(self) -> int:
        return 2
