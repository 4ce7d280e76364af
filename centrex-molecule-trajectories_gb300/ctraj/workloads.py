"""The benchmark beamlines and the lens sweep, built from this package's reference-mirror classes.

* ballistic_beamline(): plain ballistic beamline -- circular aperture
  r = 6 mm at 0.30 m (L = 1 mm), rectangular 10 x 8 mm at 1.00 m (L = 1 mm),
  circular r = 10 mm at 2.00 m (L = 1 mm), detection plane at 3.00 m.
* lens_beamline(): aperture r = 6 mm at 0.30 m, hexapole lens z0 = 0.80 m,
  L = 0.60 m, bore radius 17.5 mm, V = 30 kV, |E| = 3 V r^2 / R^3, two-level
  Stark table on 4096 knots over 0-100 kV/cm (a = h 6.7 GHz, d = 4.2 D), RK4
  with dt = 1 us, detection plane at 3.0 m.
* source(): x, y ~ N(0, 1.5 mm) at z = 0; vx, vy ~ N(0, 20 m/s); vz ~ N(184, 16).

The detection plane is a CircularAperture of infinite diameter and zero
length, which never loses a molecule but stores the molecule's state at 3 m.
Gravity is the reference's scipy.constants.g = 9.80665 m/s^2.
"""
from __future__ import annotations

from .beamline import Beamline
from .beamline_elements import CircularAperture, ElectrostaticLens, RectangularAperture
from .distributions import CeNTREXVelocityDistribution, GaussianPositionDistribution
from .stark import hexapole_force

INF = float("inf")


def source():
    return (GaussianPositionDistribution(sigmax=1.5e-3, sigmay=1.5e-3, z=0.0),
            CeNTREXVelocityDistribution(sigmax=20.0, sigmay=20.0))


def ballistic_beamline() -> Beamline:
    return Beamline([
        CircularAperture(name="A1", z0=0.30, L=1e-3, d=12e-3),
        RectangularAperture(name="R1", z0=1.00, L=1e-3, w=10e-3, h=8e-3),
        CircularAperture(name="A2", z0=2.00, L=1e-3, d=20e-3),
        CircularAperture(name="Detection plane", z0=3.00, L=0.0, d=INF),
    ])


def lens_beamline(V: float = 30e3, splitting_hz: float = 6.7e9, z0: float = 0.80,
                  aperture_d: float = 12e-3, force=None, detector_d: float = INF,
                  low_field_seeker: bool = False) -> Beamline:
    """``detector_d``: the diameter of the detection plane at 3.0 m (infinite:
    every molecule reaching it counts; finite: a detector aperture, e.g.
    10 mm, whose misses are credited to "Detection plane").
    ``low_field_seeker``: the Stark curve's other sign, a state the hexapole
    focuses (the workloads' curve is a high-field seeker, which it defocuses)."""
    if force is None:
        force = hexapole_force(V=V, R=17.5e-3, splitting_hz=splitting_hz, low_field_seeker=low_field_seeker)
    return Beamline([
        CircularAperture(name="A1", z0=0.30, L=1e-3, d=aperture_d),
        ElectrostaticLens(name="ES lens", z0=z0, L=0.60, d=35e-3, V=V, dt=1e-6, a_interp=force),
        CircularAperture(name="Detection plane", z0=3.00, L=0.0, d=detector_d),
    ])


SWEEP_SPLITTINGS_HZ = (6.7e9, 13.3e9, 20.0e9, 26.6e9)


def sweep_configs(n_voltages: int = 256, splittings_hz=SWEEP_SPLITTINGS_HZ, n_min: float = 1e4,
                  n_max: float = 1e6, v_max: float = 30e3, seed: int = 0, n_knots: int = 4096):
    """The batched lens sweep: n_voltages lens voltages drawn uniformly in
    [0, v_max] x one two-level Stark table per splitting (4096 knots over
    0-100 kV/cm, d = 4.2 D), molecules per configuration log-uniform in
    [n_min, n_max].  One numpy default_rng(seed) draws the voltages, then the
    counts (table-major: configuration (t, j) is splitting t at voltage j)."""
    import numpy as np

    from .stark import hexapole_force
    from .sweep import SweepConfigs

    rng = np.random.default_rng(seed)
    voltages = rng.uniform(0.0, v_max, n_voltages)
    n = np.exp(rng.uniform(np.log(n_min), np.log(n_max), (len(splittings_hz), n_voltages)))
    forces = [hexapole_force(V=v_max, R=17.5e-3, splitting_hz=a, n_knots=n_knots) for a in splittings_hz]
    return SweepConfigs(voltages=voltages, forces=forces, n_molecules=np.rint(n).astype(np.int64))
