"""Initial-condition distributions with the reference's classes and fields.

Mirrors ``src/trajectories/distributions.py``.  ``draw(n)`` returns the
reference's (3, n) float64 array on the host (scipy.stats, global numpy RNG,
:40-41,69-76,112-119,155-162) so that unknown code paths keep working; the
simulator does not call it for these classes.  It recognises them and draws
on the device instead (Philox-4x32-10 + Box-Muller, see
``csrc/philox.cuh``), from the parameters returned by :func:`device_spec`.
A Distribution subclass the device does not know is drawn here, on the host,
and uploaded.
"""
from __future__ import annotations

from abc import ABC, abstractmethod
from dataclasses import dataclass

import numpy as np
from scipy.stats import norm, uniform

from . import _abi

__all__ = ["Distribution", "GaussianDistribution", "CeNTREXVelocityDistribution",
           "CeNTREXPositionDistribution", "GaussianPositionDistribution", "device_spec",
           "host_draw"]


class Distribution(ABC):
    @abstractmethod
    def draw(self, n: int) -> np.ndarray:
        ...


@dataclass
class GaussianDistribution(Distribution):
    mean: float
    sigma: float

    def draw(self, n: int) -> np.ndarray:
        return norm.rvs(loc=self.mean, scale=self.sigma, size=n)

    def save_to_hdf(self, filepath, run_name: str, group_name: str = ""):
        """distributions.py:48-52."""
        raise NotImplementedError("Saving GaussianDistribution to hdf is not implemented. Save child class instead.")


@dataclass
class CeNTREXVelocityDistribution(Distribution):
    vx: float = 0.0
    sigmax: float = 39.5
    vy: float = 0.0
    sigmay: float = 39.5
    vz: float = 184.0
    sigmaz: float = 16.0

    def draw(self, n: int) -> np.ndarray:
        return np.array((GaussianDistribution(self.vx, self.sigmax).draw(n),
                         GaussianDistribution(self.vy, self.sigmay).draw(n),
                         GaussianDistribution(self.vz, self.sigmaz).draw(n)))

    def save_to_hdf(self, filepath, run_name: str):
        """distributions.py:78-98: group run_name/velocity_distribution."""
        from .hdf import save_distribution

        save_distribution(self, filepath, run_name, "velocity_distribution", "velocity")


@dataclass
class CeNTREXPositionDistribution(Distribution):
    d: float = 0.02
    z: float = 0.25 * 0.0254

    def draw(self, n: int) -> np.ndarray:
        theta = uniform.rvs(size=n) * 2 * np.pi
        r = np.sqrt(uniform.rvs(size=n)) * self.d / 2
        return np.array((r * np.cos(theta), r * np.sin(theta), np.full(n, self.z)))

    def save_to_hdf(self, filepath, run_name: str):
        """distributions.py:122-142: group run_name/position_distribution."""
        from .hdf import save_distribution

        save_distribution(self, filepath, run_name, "position_distribution", "position")


@dataclass
class GaussianPositionDistribution(Distribution):
    sigmax: float = 0.25 * 25.4 / 5 * 3.8e-3
    sigmay: float = 0.25 * 25.4 / 5 * 3.8e-3
    z: float = 0.25 * 0.0254

    def draw(self, n: int) -> np.ndarray:
        x = GaussianDistribution(0, self.sigmax).draw(n)
        y = GaussianDistribution(0, self.sigmay).draw(n)
        return np.vstack((x, y, np.full(n, self.z)))

    def save_to_hdf(self, filepath, run_name: str):
        """distributions.py:166-186: group run_name/position_distribution."""
        from .hdf import save_distribution

        save_distribution(self, filepath, run_name, "position_distribution", "position")


def device_spec(dist, role: str) -> _abi.Distribution | None:
    """C ABI descriptor for a distribution the device can draw, else None.

    Matching is by class name and fields, so the reference's own objects are
    recognised too.  ``role`` is "position" or "velocity".
    """
    s = _abi.Distribution()
    name = type(dist).__name__
    if role == "position" and name == "GaussianPositionDistribution":
        s.kind = _abi.DIST_GAUSSIAN_POSITION
        s.p[0], s.p[1], s.p[2] = float(dist.sigmax), float(dist.sigmay), float(dist.z)
        return s
    if role == "position" and name == "CeNTREXPositionDistribution":
        s.kind = _abi.DIST_DISC_POSITION
        s.p[0], s.p[1] = float(dist.d), float(dist.z)
        return s
    if role == "velocity" and name == "CeNTREXVelocityDistribution":
        s.kind = _abi.DIST_GAUSSIAN_VELOCITY
        for i, f in enumerate(("vx", "sigmax", "vy", "sigmay", "vz", "sigmaz")):
            s.p[i] = float(getattr(dist, f))
        return s
    return None


def host_draw(xdist, vdist, n: int, seed: int | None = None) -> np.ndarray:
    """(6, n) float64 initial conditions drawn on the host.

    With ``seed`` the known classes are drawn from ``numpy.random.default_rng``
    (velocity first, then position, as trajectory_simulator.py:57-58), which is
    how seeded parity inputs are made; without it ``draw`` is called, which
    uses the global RNG like the reference.
    """
    if seed is None:
        vs = np.asarray(vdist.draw(n), dtype=np.float64)
        xs = np.asarray(xdist.draw(n), dtype=np.float64)
        return np.ascontiguousarray(np.vstack((xs, vs)))
    rng = np.random.default_rng(seed)
    out = np.empty((6, n))
    vk, xk = type(vdist).__name__, type(xdist).__name__
    if vk != "CeNTREXVelocityDistribution":
        raise TypeError(f"seeded host draw does not know {vk}")
    out[3] = rng.normal(vdist.vx, vdist.sigmax, n)
    out[4] = rng.normal(vdist.vy, vdist.sigmay, n)
    out[5] = rng.normal(vdist.vz, vdist.sigmaz, n)
    if xk == "GaussianPositionDistribution":
        out[0] = rng.normal(0.0, xdist.sigmax, n)
        out[1] = rng.normal(0.0, xdist.sigmay, n)
        out[2] = xdist.z
    elif xk == "CeNTREXPositionDistribution":
        theta = rng.uniform(size=n) * 2 * np.pi
        r = np.sqrt(rng.uniform(size=n)) * xdist.d / 2
        out[0] = r * np.cos(theta)
        out[1] = r * np.sin(theta)
        out[2] = xdist.z
    else:
        raise TypeError(f"seeded host draw does not know {xk}")
    return out
