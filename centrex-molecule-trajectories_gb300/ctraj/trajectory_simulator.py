"""Drop-in for trajectories.trajectory_simulator (TrajectorySimulator, Counter,
SimulationResult), with the propagation on the GPU.

``TrajectorySimulator.run_simulation`` keeps the reference's signature and
side effects (trajectory_simulator.py:34-103):

* the number of molecules is ``100 * n_jobs * int(N_traj / (100 * n_jobs))``
  (the reference's chunking, :48-49); ``n_jobs`` changes nothing else, since
  every molecule is propagated by the same CUDA launch;
* ``self.counter`` is a fresh :class:`Counter` of label -> count, and
  ``self.result`` / ``self.results[run_name]`` are :class:`SimulationResult`
  objects holding the molecules whose label is in ``apertures_of_interest``,
  with their full trajectories (molecule.py:111-167);
* known distribution classes are drawn on the device (Philox-4x32-10 +
  Box-Muller); any other ``Distribution`` is drawn on the host with its own
  ``draw`` (velocity first, then position, per chunk, as :57-58) and uploaded.

Extensions (keyword-only): ``seed`` (the reference has none), ``ics`` to inject
a (6, n) initial-condition array, ``precision`` (32 or 64) and ``device``.
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field
from typing import List

import numpy as np

from . import _abi
from .compiler import DETECTED, compile_beamline
from .distributions import (CeNTREXPositionDistribution, CeNTREXVelocityDistribution,
                            Distribution, device_spec)
from .engine import G, default_engine
from .molecule import Molecule, Trajectory

__all__ = ["TrajectorySimulator", "Counter", "SimulationResult", "simulated_count"]


def simulated_count(N_traj: int, n_jobs: int) -> int:
    """Molecules the reference actually simulates (trajectory_simulator.py:48-49, 81-83)."""
    n_loops = 100 * n_jobs
    if n_loops <= 0:
        return 0
    n = int(N_traj / n_loops)
    if n < 0:
        raise ValueError("negative dimensions are not allowed")
    return n_loops * n


class Counter:
    """trajectory_simulator.py:106-158."""

    def __init__(self) -> None:
        self.counter_dict = {}

    def increment_counter(self, aperture_hit: str) -> None:
        self.counter_dict[aperture_hit] = self.counter_dict.get(aperture_hit, 0) + 1

    def print(self) -> None:
        print("Number of molecules that hit each element:")
        for key, value in self.counter_dict.items():
            print(f"{key} : {value}")

    def calculate_efficiency(self) -> float:
        total = sum(self.counter_dict.values())
        if "Detected" in self.counter_dict:
            return self.counter_dict["Detected"] / total
        return 0

    def merge_counters(self, others: List) -> None:
        for other in others:
            for key, value in other.counter_dict.items():
                self.counter_dict[key] = self.counter_dict.get(key, 0) + value

    def save_to_hdf(self, filepath, run_name: str) -> None:
        """trajectory_simulator.py:160-176: attrs label -> count of run_name/counter."""
        from .hdf import save_counter

        save_counter(self, filepath, run_name)


@dataclass
class SimulationResult:
    """trajectory_simulator.py:180-191.  ``replay`` (extension) holds what
    ctraj.post_processing needs to re-propagate ``molecules`` on the device:
    the compiled beamline, the run's initial-condition source and the
    molecules' indices in the run."""

    counter: Counter
    beamline: object
    xdist: Distribution
    vdist: Distribution
    molecules: List[Molecule]
    replay: dict | None = field(default=None, repr=False, compare=False)

    def save_to_hdf(self, filepath, run_name: str) -> None:
        """trajectory_simulator.py:218-244 (layout in ctraj.hdf)."""
        from .hdf import save_result

        save_result(self, filepath, run_name)

    def save_molecules_to_hdf(self, filepath, run_name: str) -> None:
        """trajectory_simulator.py:246-254: run_name/trajectories/molecule_<i>."""
        from .hdf import save_molecules

        save_molecules(self, filepath, run_name)


class TrajectorySimulator:
    def __init__(self, device: int = 0, precision: int = 32) -> None:
        self.counter = Counter()
        self.results = {}
        self.device = device
        self.precision = precision
        self.last_run = None

    def run_simulation(self, beamline, run_name: str, vdist=CeNTREXVelocityDistribution(),
                       xdist=CeNTREXPositionDistribution(), N_traj: int = 1000,
                       apertures_of_interest=[], n_jobs=1, *, seed: int | None = None, ics=None,
                       precision: int | None = None, g: float = G):
        n = simulated_count(N_traj, n_jobs)
        prec = precision or self.precision
        cb = compile_beamline(beamline)
        eng = default_engine(self.device)
        if seed is None:
            seed = int.from_bytes(os.urandom(8), "little")
        xs, vs = device_spec(xdist, "position"), device_spec(vdist, "velocity")
        if ics is None and (xs is None or vs is None) and n > 0:
            n_loops = 100 * n_jobs
            per = n // n_loops
            chunks = []
            for _ in range(n_loops):
                v = np.asarray(vdist.draw(per), dtype=np.float64).reshape(3, per)
                x = np.asarray(xdist.draw(per), dtype=np.float64).reshape(3, per)
                chunks.append(np.vstack((x, v)))
            ics = np.ascontiguousarray(np.hstack(chunks))
        aoi = set(apertures_of_interest)
        want_out = bool(aoi) and n > 0
        res = eng.run(cb, n, precision=prec, ics=ics, xdist=xs, vdist=vs, seed=seed, g=g,
                      outputs=want_out)
        self.last_run = res
        molecules = []
        ids = np.zeros(0, np.int64)
        if want_out:
            names = res.label_names()
            ids = np.array([i for i, s in enumerate(names) if s in aoi], dtype=np.int64)
            if ids.size:
                max_rows = self._max_rows(cb, beamline, res.final[5, ids])
                traces = eng.record(cb, n, ids, stride=1, max_rows=max_rows, precision=prec,
                                    ics=ics, xdist=xs, vdist=vs, seed=seed, g=g)
                for i, rows in zip(ids, traces):
                    m = Molecule(alive=names[i] == DETECTED)
                    m.trajectory = Trajectory.from_rows(rows)
                    m.trajectory.drop_nans()
                    m.trajectory.n = len(m.trajectory.t)
                    m.set_aperture_hit(names[i])
                    molecules.append(m)
        self.counter = Counter()
        self.counter.counter_dict = res.counter_dict()
        replay = dict(device=self.device, cb=cb, n=n, precision=prec, ics=ics, xdist=xs, vdist=vs, seed=seed,
                      g=g, ids=ids)
        self.result = SimulationResult(self.counter, beamline, xdist, vdist, molecules, replay)
        self.results[run_name] = SimulationResult(self.counter, beamline, xdist, vdist, molecules, replay)

    def run_simulations(self, beamline, run_names, vdist=CeNTREXVelocityDistribution(),
                        xdist=CeNTREXPositionDistribution(), N_traj: int = 1000, n_jobs=1, *,
                        seeds=None, precision: int | None = None, g: float = G, l2_flush_bytes: int = 0):
        """The caller's loop ``for name in run_names: run_simulation(beamline,
        name, ...)`` as one call: every batch of N_traj molecules is its own run
        (own seed, own Counter under results[name]), and the runs are pipelined
        on the device (ctraj_run_batch), so one batch's ballistic front overlaps
        the previous batch's lens pass.  Trajectories are not kept
        (apertures_of_interest empty); last_runs holds the per-batch RunResults
        and last_run the last one.  l2_flush_bytes > 0: that many bytes of
        device scratch are written before each batch (cold caches between
        batches, for timing)."""
        names = list(run_names)
        n = simulated_count(N_traj, n_jobs)
        prec = precision or self.precision
        if seeds is None:
            seeds = [int.from_bytes(os.urandom(8), "little") for _ in names]
        seeds = list(seeds)
        if len(seeds) != len(names):
            raise ValueError("one seed per run name")
        cb = compile_beamline(beamline)
        eng = default_engine(self.device)
        xs, vs = device_spec(xdist, "position"), device_spec(vdist, "velocity")
        ics = None
        if (xs is None or vs is None) and n > 0:
            n_loops = 100 * n_jobs
            per = n // n_loops
            ics = []
            for _ in names:
                chunks = []
                for _ in range(n_loops):
                    v = np.asarray(vdist.draw(per), dtype=np.float64).reshape(3, per)
                    x = np.asarray(xdist.draw(per), dtype=np.float64).reshape(3, per)
                    chunks.append(np.vstack((x, v)))
                ics.append(np.ascontiguousarray(np.hstack(chunks)))
        runs = eng.run_batch(cb, n, seeds, precision=prec, ics=ics, xdist=xs, vdist=vs, g=g,
                             l2_flush_bytes=int(l2_flush_bytes))
        self.last_runs = runs
        for k, (name, res) in enumerate(zip(names, runs)):
            self.last_run = res
            self.counter = Counter()
            self.counter.counter_dict = res.counter_dict()
            replay = dict(device=self.device, cb=cb, n=n, precision=prec, ics=None if ics is None else ics[k],
                          xdist=xs, vdist=vs, seed=seeds[k], g=g, ids=np.zeros(0, np.int64))
            self.result = SimulationResult(self.counter, beamline, xdist, vdist, [], replay)
            self.results[name] = self.result

    @staticmethod
    def _max_rows(cb, beamline, vz) -> int:
        """Trajectory rows a molecule can need (Trajectory.__init__, molecule.py:115-128)."""
        rows = 10
        vmin = float(np.min(np.abs(vz))) if np.size(vz) else 1.0
        for e in beamline.elements:
            if type(e).__name__ == "ElectrostaticLens":
                dt = getattr(e, "dt", None)
                dz = e.dz if dt is None else max(vmin * dt, 1e-300)
                rows += 2 + int(np.rint(e.L / dz))
            else:
                rows += 2
        if rows > _abi.MAX_LENS_STEPS:
            raise MemoryError("trajectory too long to record")
        return rows
