"""TEST INFRASTRUCTURE, NOT PRODUCT CODE: time the reference's own Python
``TrajectorySimulator.run_simulation(..., n_jobs=os.cpu_count())`` on the
lens-beamline workload and write the rate to reference_python_rate.json.

    python oracle/measure_reference_python.py --reference-src <reference>/src

The reference cannot run on the GPU machines (it is not installed there and
its third-party imports are absent), so its rate is measured here, in the
container that holds it, and reported by bench.py beside the timed CPU
baseline as a labelled figure (machine, cores, molecules) -- never in the
GPU/CPU ratio, whose CPU side is timed on the GPU machine's own cores.

The workload is the benchmark's: circular aperture r = 6 mm at 0.30 m,
hexapole lens 0.80-1.40 m (4096-knot cubic spline of W(E) = -(sqrt(a^2 +
(dE)^2) - a), a = h 6.7 GHz, d = 4.2 D, V = 30 kV, R = 17.5 mm), RK4 at
dt = 1 us, detection plane at 3.0 m; x, y ~ N(0, 1.5 mm), vx, vy ~
N(0, 20 m/s), vz ~ N(184, 16).  The reference is driven through its public
API only:

* its imports of h5py, matplotlib, centrex_TlF and hexalattice are stubbed
  (tests/golden/refstubs.py), in the workers too, through a sitecustomize
  module on PYTHONPATH;
* the lens force is the public ``a_interp`` field: a callable built from the
  FP64 scipy CubicSpline of W(E) (electrostatic_lens.py:174,217 call it as
  ``self.a_interp(r)``);
* dt = 1 us is realised as the reference allows, ``dz = vz * dt`` set on the
  lens per molecule before its ``propagate_through`` (``dt = dz / vz``,
  electrostatic_lens.py:87-88), by a subclass that also sizes ``N_steps()``
  (the Trajectory preallocation, molecule.py:115-128) for molecules as slow
  as vz = 88 m/s (six standard deviations below the mean);
* distributions are the reference's GaussianPositionDistribution and
  CeNTREXVelocityDistribution, drawn by the reference in its workers.

Rate = molecules per second of the timed run_simulation (best of --reps,
apertures_of_interest empty, the reference's default) x trajectory rows after
the initial one per molecule (len(trajectory.t) - 1, the benchmark's unit),
counted from --reps further runs that keep every molecule
(apertures_of_interest = every label).
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import sys
import tempfile
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
GOLDEN = ROOT / "tests" / "golden"
sys.path.insert(0, str(GOLDEN))
import refstubs  # noqa: E402

LABELS = ["A1", "Lens entrance", "Inside lens", "Detected"]
VZ_SLOWEST = 184.0 - 6 * 16.0  # m/s: trajectory rows are preallocated for molecules this slow


def cpu_model() -> str:
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.startswith("model name"):
                return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return platform.processor() or platform.machine()


def worker_site(reference_src: str) -> str:
    """A directory holding a sitecustomize that installs the stubs in every worker."""
    d = tempfile.mkdtemp(prefix="refsite")
    Path(d, "sitecustomize.py").write_text(
        f"import sys\nsys.path.insert(0, {str(GOLDEN)!r})\nimport refstubs\nrefstubs.install({reference_src!r})\n")
    return d


def build(dt: float = 1e-6):
    import numpy as np
    from scipy.constants import c, h
    from scipy.interpolate import CubicSpline
    from trajectories.beamline import Beamline
    from trajectories.beamline_elements import CircularAperture, ElectrostaticLens
    from trajectories.distributions import CeNTREXVelocityDistribution, GaussianPositionDistribution

    a, d = h * 6.7e9, 4.2 * 1e-21 / c
    E = np.linspace(0.0, 1e7, 4096)
    spline = CubicSpline(E, -(np.sqrt(a * a + (d * E) ** 2) - a))
    V, R, mass = 30e3, 17.5e-3, (204.38 + 19.00) * 1.67e-27
    alpha = 3.0 * V / R ** 3

    def a_interp(r):
        return -(spline(alpha * (r * r), 1) * (2.0 * alpha * r)) / mass

    class FixedDtLens(ElectrostaticLens):
        """The reference's lens with dz = vz * dt set per molecule (dt = dz / vz).
        Trajectory rows are preallocated from N_steps() before a molecule's dz
        is known (molecule.py:115-128), so N_steps() counts the steps of the
        slowest molecule expected: vz = 184 - 6 x 16 m/s."""

        def propagate_through(self, molecule):
            self.dz = molecule.v()[2] * dt
            return super().propagate_through(molecule)

        def N_steps(self):
            return 1 + int(np.rint(self.L / (VZ_SLOWEST * dt)))

    inf = float("inf")
    bl = Beamline([CircularAperture(name="A1", z0=0.30, L=1e-3, d=12e-3),
                   FixedDtLens(name="ES lens", z0=0.80, L=0.60, d=35e-3, V=V, mass=mass, a_interp=a_interp),
                   CircularAperture(name="Detection plane", z0=3.00, L=0.0, d=inf)])
    return bl, GaussianPositionDistribution(sigmax=1.5e-3, sigmay=1.5e-3, z=0.0), \
        CeNTREXVelocityDistribution(sigmax=20.0, sigmay=20.0)


def main():
    ap = argparse.ArgumentParser()
    refstubs.add_argument(ap)
    ap.add_argument("--per-chunk", type=int, default=20, help="molecules per joblib task (N_traj / (100 n_jobs))")
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", default=str(HERE / "reference_python_rate.json"))
    args = ap.parse_args()
    src = refstubs.require(args.reference_src)
    os.environ["PYTHONPATH"] = os.pathsep.join([worker_site(src), os.environ.get("PYTHONPATH", "")])
    refstubs.install(src)
    import numpy as np
    from trajectories.trajectory_simulator import TrajectorySimulator

    n_jobs = os.cpu_count() or 1
    n_traj = 100 * n_jobs * args.per_chunk
    bl, xd, vd = build()
    sim = TrajectorySimulator()
    sim.run_simulation(bl, "warm", vdist=vd, xdist=xd, N_traj=100 * n_jobs, n_jobs=n_jobs)  # workers up
    times = []
    for k in range(args.reps):
        t0 = time.perf_counter()
        sim.run_simulation(bl, f"t{k}", vdist=vd, xdist=xd, N_traj=n_traj, n_jobs=n_jobs)
        times.append(time.perf_counter() - t0)
    rows = []
    for k in range(args.reps):
        sim.run_simulation(bl, f"s{k}", vdist=vd, xdist=xd, N_traj=n_traj, apertures_of_interest=LABELS,
                           n_jobs=n_jobs)
        rows += [len(m.trajectory.t) - 1 for m in sim.result.molecules]
    steps_per_molecule = float(np.mean(rows))
    best = min(times)
    out = {"metric": "molecule-steps/s", "value": n_traj / best * steps_per_molecule,
           "molecules_per_s": n_traj / best, "steps_per_molecule": steps_per_molecule,
           "steps_sample_molecules": len(rows), "molecules": n_traj, "n_jobs": n_jobs, "cores": n_jobs,
           "seconds": times, "machine": f"{cpu_model()}, {platform.machine()}, {n_jobs} cores",
           "python": platform.python_version(),
           "api": "trajectories.trajectory_simulator.TrajectorySimulator.run_simulation(beamline, name, vdist, "
                  f"xdist, N_traj={n_traj}, n_jobs={n_jobs}) (best of {args.reps})",
           "recipe": "oracle/measure_reference_python.py",
           "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    Path(args.out).write_text(json.dumps(out, indent=1) + "\n")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
