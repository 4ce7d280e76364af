"""ElectrostaticLens with the reference's fields (electrostatic_lens.py:23-46).

The reference integrates the lens interior with RK4 and a radial
acceleration ``a_interp(r)`` (:79-118, :168-227).  Here the same dataclass
describes the lens and the CUDA kernel integrates it.  ``a_interp`` may be

* a ``scipy.interpolate.interp1d`` over r (what the reference builds and
  pickles, :194-213): it becomes a linear radial table on the device;
* a :class:`ctraj.stark.StarkForce` (a cubic-spline Stark table W(E) plus the
  lens field model): it becomes a piecewise-cubic table in |E|.

Two fields extend the reference and default to its behaviour:

* ``dt`` -- when set, each molecule uses dz = vz * dt (a fixed time step);
  ``None`` keeps the reference's fixed ``dz`` (N = rint(L/dz), dt = dz/vz).
* ``scheme`` -- "reference" keeps the reference's stage-2 point x + dt*k1
  (:97); "classic" uses textbook RK4 (x + dt*k1/2).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Any, Optional

from .apertures import BeamlineElement

__all__ = ["ElectrostaticLens"]


@dataclass
class ElectrostaticLens(BeamlineElement):
    d: float = 1.75 * 0.0254
    dz: float = 1e-3
    V: float = 27.6e3
    a_interp: Any = None
    state: Any = None
    mass: float = (204.38 + 19.00) * 1.67e-27
    dt: Optional[float] = None
    scheme: str = "reference"

    def save_to_hdf(self, filepath, parent_group_path: str) -> None:
        """electrostatic_lens.py:145-166 (the force table is not saved)."""
        from ..hdf import save_lens

        save_lens(self, filepath, parent_group_path)

    def N_steps(self) -> int:
        """1 + rint(L/dz), electrostatic_lens.py:120-125."""
        import numpy as np

        return 1 + int(np.rint(self.L / self.dz))
