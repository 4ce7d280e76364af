"""Batched lens sweeps: many lens configurations in one launch sequence.

The reference sweeps a beamline by looping over configurations and calling
``run_simulation`` once per configuration (the per-state loop of
examples/lens_simulation_different_states.py:136-156 changes the lens's
Stark state and rebuilds its force table each time).  Here a configuration is
(lens voltage, Stark table) on an otherwise fixed beamline with one
electrostatic lens, and ``run_sweep`` propagates every configuration's
molecules with one ``ctraj_run_sweep`` call: one front launch over all of
them, then one chunked lens sequence per Stark table, optionally replayed from
a captured CUDA graph.  ``loop_sweep`` is the same sweep as a loop of plain
runs (one compiled beamline per configuration), for comparison.

Configuration (t, j) = forces[t] at voltages[j], flattened as c = t * n_V + j;
its molecules are numbers start_c .. start_c + N_c - 1 of the sweep, so a
device draw gives configuration c the Philox counters of a plain run with
offset = offset + start_c.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .compiler import CompiledBeamline, Table, compile_beamline
from .engine import G, default_engine
from .distributions import device_spec
from .stark import StarkForce, field_coefficient

__all__ = ["SweepConfigs", "SweepResult", "run_sweep", "loop_sweep", "sweep_beamline"]


@dataclass
class SweepConfigs:
    voltages: np.ndarray           # (n_V,) lens voltages
    forces: list                   # n_T StarkForce tables (the voltage of each is ignored)
    n_molecules: np.ndarray        # (n_T, n_V) molecules per configuration

    def __post_init__(self):
        self.voltages = np.asarray(self.voltages, dtype=np.float64).reshape(-1)
        self.n_molecules = np.asarray(self.n_molecules, dtype=np.int64).reshape(len(self.forces),
                                                                               self.voltages.size)
        if (self.n_molecules < 0).any():
            raise ValueError("n_molecules must be >= 0")
        f0 = self.forces[0]
        for f in self.forces:
            if (f.R, f.mass, f.field_order) != (f0.R, f0.mass, f0.field_order):
                raise ValueError("all sweep tables need the same lens radius, mass and field order")

    @property
    def shape(self):
        return self.n_molecules.shape

    @property
    def n_configs(self) -> int:
        return int(self.n_molecules.size)

    @property
    def total(self) -> int:
        return int(self.n_molecules.sum())

    def alphas(self) -> np.ndarray:
        """Field coefficient per configuration (flattened), as the lens force law computes it."""
        f0 = self.forces[0]
        a = np.array([field_coefficient(float(V), f0.R, f0.field_order) for V in self.voltages])
        return np.tile(a, len(self.forces))

    def table_index(self) -> np.ndarray:
        return np.repeat(np.arange(len(self.forces), dtype=np.int32), self.voltages.size)

    def starts(self) -> np.ndarray:
        """First sweep molecule number of each configuration (flattened)."""
        n = self.n_molecules.reshape(-1)
        return np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)

    def tables(self) -> list:
        return [Table(_abi.TABLE_STARK_SPLINE, np.ascontiguousarray(f.knots, np.float64),
                      coef=np.ascontiguousarray(f.coef, np.float64)) for f in self.forces]

    def force(self, t: int, j: int) -> StarkForce:
        return self.forces[t].with_voltage(float(self.voltages[j]))


@dataclass
class SweepResult:
    counts: np.ndarray             # (n_T, n_V, n_labels + 1), last slot "Detected"
    totals: np.ndarray             # (n_labels + 1,)
    labels: list
    molecules: int
    molecule_steps: int
    lens_steps: int
    kernels: int
    extra: dict = field(default_factory=dict)

    def detected_fraction(self) -> np.ndarray:
        n = self.counts.sum(axis=-1)
        return np.where(n > 0, self.counts[..., -1] / np.maximum(n, 1), 0.0)


def _spec(d, role):
    if d is None or isinstance(d, _abi.Distribution):
        return d
    s = device_spec(d, role)
    if s is None:
        raise TypeError(f"{type(d).__name__} cannot be drawn on the device; pass ics instead")
    return s


def sweep_beamline(beamline) -> CompiledBeamline:
    cb = beamline if isinstance(beamline, CompiledBeamline) else compile_beamline(beamline)
    if cb.n_lenses != 1:
        raise ValueError(f"a sweep beamline needs exactly one electrostatic lens (it has {cb.n_lenses})")
    return cb


def run_sweep(beamline, configs: SweepConfigs, xdist=None, vdist=None, ics=None, seed: int = 0,
              offset: int = 0, g: float = G, use_graph: bool = True, timing: bool = False,
              engine=None) -> SweepResult:
    """All configurations in one ctraj_run_sweep call (the beamline's own lens
    voltage and table are replaced by each configuration's)."""
    cb = sweep_beamline(beamline)
    eng = engine or default_engine()
    if not hasattr(configs, "_tables"):
        configs._tables = configs.tables()  # kept: the engine skips re-uploading the same objects
    r = eng.run_sweep(cb, configs._tables, configs.alphas(), configs.table_index(),
                      configs.n_molecules.reshape(-1), ics=ics, xdist=_spec(xdist, "position"),
                      vdist=_spec(vdist, "velocity"), seed=seed,
                      offset=offset, g=g, use_graph=use_graph, timing=timing)
    st = r["stats"]
    return SweepResult(counts=r["counts"].reshape(configs.shape + (len(cb.labels) + 1,)),
                       totals=r["totals"], labels=list(cb.labels), molecules=st["molecules"],
                       molecule_steps=st["molecule_steps"], lens_steps=st["lens_steps"],
                       kernels=st["kernels"], extra=r["extra"])


def config_beamlines(beamline, configs: SweepConfigs) -> list:
    """One compiled beamline per configuration (flattened order): the beamline
    with its lens's force replaced by the configuration's."""
    import copy

    out = []
    for t in range(len(configs.forces)):
        for j in range(configs.voltages.size):
            bl = copy.copy(beamline)
            bl.elements = [copy.copy(e) for e in beamline.elements]
            for e in bl.elements:
                if type(e).__name__ == "ElectrostaticLens":
                    f = configs.force(t, j)
                    e.a_interp = f
                    e.V = f.V
            out.append(compile_beamline(bl))
    return out


def loop_sweep(compiled: list, configs: SweepConfigs, xdist=None, vdist=None, seed: int = 0,
               offset: int = 0, g: float = G, engine=None) -> np.ndarray:
    """The sweep as a loop of plain runs (ctraj_run per configuration, device
    draws with the sweep's Philox counters); returns counts (n_T, n_V, n_labels + 1)."""
    eng = engine or default_engine()
    xdist, vdist = _spec(xdist, "position"), _spec(vdist, "velocity")
    n = configs.n_molecules.reshape(-1)
    starts = configs.starts()
    out = np.zeros((n.size, len(compiled[0].labels) + 1), np.int64)
    for c, cb in enumerate(compiled):
        if n[c] == 0:
            continue
        out[c] = eng.run(cb, int(n[c]), xdist=xdist, vdist=vdist, seed=seed,
                         offset=offset + int(starts[c]), g=g).counts
    return out.reshape(configs.shape + (out.shape[1],))
