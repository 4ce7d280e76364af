"""Molecule / Trajectory result objects (molecule.py:8-187 of the reference).

Molecules that end on an "aperture of interest" are returned to the caller as
these objects, filled from the device's trajectory recording, so code written
against the reference's ``SimulationResult.molecules`` (plotting,
``post_processing``) reads the same attributes: ``trajectory.x/v/a`` (n, 3),
``trajectory.t`` (n,), ``trajectory.n``, ``aperture_hit`` and ``alive``.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

__all__ = ["Molecule", "Trajectory"]


class Trajectory:
    """Row store of positions, velocities, accelerations and times."""

    def __init__(self, x: np.ndarray, v: np.ndarray, a: np.ndarray, t: np.ndarray):
        self.x = np.asarray(x, dtype=np.float64)
        self.v = np.asarray(v, dtype=np.float64)
        self.a = np.asarray(a, dtype=np.float64)
        self.t = np.asarray(t, dtype=np.float64)
        self.n = int(self.t.shape[0])

    @classmethod
    def from_rows(cls, rows: np.ndarray) -> "Trajectory":
        """rows: (n, 10) x, y, z, vx, vy, vz, ax, ay, az, t."""
        rows = np.asarray(rows, dtype=np.float64)
        return cls(rows[:, 0:3].copy(), rows[:, 3:6].copy(), rows[:, 6:9].copy(), rows[:, 9].copy())

    def save_to_hdf(self, file, run_name: str, group_name: str) -> None:
        """molecule.py:169-185 (datasets x, v, a, t of the group run_name/group_name)."""
        from .hdf import save_trajectory

        save_trajectory(self, file, run_name, group_name)

    def drop_nans(self):
        """molecule.py:160-167."""
        self.x = self.x[np.all(np.isfinite(self.x), axis=1), :]
        self.v = self.v[np.all(np.isfinite(self.v), axis=1), :]
        self.a = self.a[np.all(np.isfinite(self.a), axis=1), :]
        self.t = self.t[np.isfinite(self.t)]


@dataclass
class Molecule:
    alive: bool = True

    def x(self, delta_t: float = None):
        """Current position, or the constant-acceleration extrapolation (molecule.py:26-34)."""
        if not delta_t:
            return self.trajectory.x[self.trajectory.n - 1, :]
        return self.x() + self.v() * delta_t + self.a() * delta_t ** 2 / 2

    def v(self, delta_t: float = None):
        if not delta_t:
            return self.trajectory.v[self.trajectory.n - 1, :]
        return self.v() + self.a() * delta_t

    def a(self):
        return self.trajectory.a[self.trajectory.n - 1, :]

    def t(self):
        return self.trajectory.t[self.trajectory.n - 1]

    def set_aperture_hit(self, aperture_name):
        self.aperture_hit = aperture_name

    def set_dead(self):
        self.alive = False

    def save_to_hdf(self, file, run_name: str, group_name: str):
        """molecule.py:97-106: the trajectory plus attrs aperture_hit and alive."""
        from .hdf import save_molecule

        save_molecule(self, file, run_name, group_name)
