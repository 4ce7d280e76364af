"""z-plane post-processing (the reference's post_processing.py), on the device.

``find_radial_pos_dist`` and ``find_vel_dist`` take a ``SimulationResult`` from
``ctraj.TrajectorySimulator.run_simulation`` and a plane z, and return the x, y
positions (shape (k, 2)) or the velocities ((k, 3)) of the result's molecules
at that plane, in the order of ``result.molecules``, skipping the molecules
whose trajectory ends before the plane and, with ``elements``, those whose
label is not in it (post_processing.py:20-140).  Each state comes from the
trajectory row on the plane, or from the row before the first one past the
plane advanced by ``take_timestep`` (:9-17).  The molecules are re-propagated
on the GPU (``ctraj_plane``); no trajectory rows are read from the host.
"""
from __future__ import annotations

from typing import List

import numpy as np

from .engine import default_engine

__all__ = ["take_timestep", "find_radial_pos_dist", "find_vel_dist", "plane_states"]


def take_timestep(x0: np.ndarray, v0: np.ndarray, a0: np.ndarray, dt: float):
    """Position and velocity after dt from x0, v0, a0 (post_processing.py:9-17)."""
    x = x0 + v0 * dt + a0 * (dt * dt) / 2
    v = v0 + a0 * dt
    return x, v


def plane_states(result, z: float, elements: List[str] | None = None) -> np.ndarray:
    """(k, 8) x, y, z, vx, vy, vz, status, 0 at the plane for the molecules the
    reference keeps (status > 0), in result order."""
    rp = getattr(result, "replay", None)
    if not rp:
        raise ValueError("post-processing needs a SimulationResult from ctraj.TrajectorySimulator")
    ids = np.asarray(rp["ids"], dtype=np.int64)
    if ids.size != len(result.molecules):
        raise ValueError("result.molecules does not match its replay information")
    keep = np.ones(ids.size, bool)
    if elements is not None:
        keep = np.array([m.aperture_hit in elements for m in result.molecules], dtype=bool)
    sel = ids[keep]
    if sel.size == 0:
        return np.zeros((0, 8))
    eng = default_engine(rp["device"])
    out = eng.plane(rp["cb"], rp["n"], sel, float(z), precision=rp["precision"], ics=rp["ics"],
                    xdist=rp["xdist"], vdist=rp["vdist"], seed=rp["seed"], g=rp["g"])
    return out[out[:, 6] > 0]


def find_radial_pos_dist(result, z: float, elements: List[str] | None = None) -> np.ndarray:
    """x, y of the result's molecules at the plane z: (k, 2) (post_processing.py:20-76)."""
    print("Determining radial positions...")
    st = plane_states(result, z, elements)
    return np.array(st[:, 0:2]) if len(st) else np.array([])  # the reference returns np.array([]) when empty


def find_vel_dist(result, z: float, elements: List[str] | None = None) -> np.ndarray:
    """vx, vy, vz of the result's molecules at the plane z: (k, 3) (post_processing.py:79-140)."""
    print("Determining radial velocities...")
    st = plane_states(result, z, elements)
    return np.array(st[:, 3:6]) if len(st) else np.array([])
