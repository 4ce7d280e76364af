"""Streamed runs and gradient-based beamline tuning.

``run_streamed`` propagates more molecules than one run should hold (e.g.
1e9) as consecutive runs of ``chunk`` molecules on consecutive Philox
counter ranges, summing the counts (the reference splits N_traj into chunks
the same way, trajectory_simulator.py:48-49, and merges their Counters,
:94-97), optionally appending the molecules lost on the lens to an HBM ring
(ctraj.ring.HBMRing).

``adam_tune`` maximises the soft transmission over a subset of its
parameters (e.g. lens voltage and lens position) with torch.optim.Adam, one
discrete-adjoint gradient (ctraj.adjoint) per step on fresh molecules.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .engine import G, default_engine

__all__ = ["StreamResult", "run_streamed", "adam_tune"]


@dataclass
class StreamResult:
    counts: np.ndarray
    labels: list
    molecules: int
    molecule_steps: int
    lens_steps: int
    chunks: int
    kernels: int
    seconds: float
    chunk_ms: list = field(default_factory=list)
    ring_rows: int = 0          # rows appended to the ring (with drain: over all runs)
    ring_molecules: int = 0
    rows_lost: int = 0          # with drain: rows overwritten before they could be drained
    molecules_lost: int = 0

    def counter_dict(self) -> dict:
        names = list(self.labels) + ["Detected"]
        return {names[k]: int(c) for k, c in enumerate(self.counts) if c}


def run_streamed(cb, n_total: int, chunk: int = 134_000_000, xdist=None, vdist=None, seed: int = 0,
                 offset: int = 0, g: float = G, ring=None, engine=None, timing: bool = True,
                 drain=None) -> StreamResult:
    """n_total molecules in runs of at most `chunk`; molecule k of the stream
    has Philox counter offset + k (so the result equals one run of n_total).
    With a ring and ``drain`` (a consumer such as ctraj.ring.HostRingStore)
    the ring is drained after every run, so it keeps every record as long as
    one run's records fit it; the result counts what was appended and lost."""
    eng = engine or default_engine()
    counts = np.zeros(len(cb.labels) + 1, np.int64)
    steps = lsteps = kernels = 0
    chunk_ms = []
    ring_tot = [0, 0, 0, 0]  # rows, molecules, rows lost, molecules lost
    t0 = time.perf_counter()
    k = 0
    for first in range(0, int(n_total), int(chunk)):
        n = min(int(chunk), int(n_total) - first)
        r = eng.run(cb, n, xdist=xdist, vdist=vdist, seed=seed, offset=offset + first, g=g, ring=ring,
                    timing=timing)
        counts += r.counts
        steps += r.molecule_steps
        lsteps += r.lens_steps
        kernels += r.kernels
        if timing:
            chunk_ms.append(r.extra["front_ms"] + r.extra["lens_ms"])
        if ring is not None and drain is not None:
            d = ring.drain(drain)
            ring_tot = [a + d[key] for a, key in zip(ring_tot, ("rows", "molecules", "rows_lost", "molecules_lost"))]
        k += 1
    if ring is not None and drain is None:
        ring_tot[0], ring_tot[1] = ring.counts()
        ring_tot[2] = max(0, ring_tot[0] - ring.capacity_rows)
        ring_tot[3] = max(0, ring_tot[1] - ring.capacity_molecules)
    return StreamResult(counts=counts, labels=list(cb.labels), molecules=int(n_total), molecule_steps=steps,
                        lens_steps=lsteps, chunks=k, kernels=kernels, seconds=time.perf_counter() - t0,
                        chunk_ms=chunk_ms, ring_rows=ring_tot[0], ring_molecules=ring_tot[1],
                        rows_lost=ring_tot[2], molecules_lost=ring_tot[3])


def adam_tune(prob, which=("V", "lens_z0"), steps: int = 200, lr: float = 1e-2, params0=None,
              engine=None, seed0: int = 0, bounds=None) -> dict:
    """Projected Adam on the named parameters (relative units: p = p0 * u, u
    starts at 1) maximising the soft transmission of `prob` (a
    ctraj.adjoint.SoftProblem); after each step the parameters are clipped to
    `bounds` ((6, 2), default prob.param_bounds(): e.g. the lens may not move
    past its neighbours).  Each step draws new molecules (seed seed0 + step).
    Returns the parameter and loss history."""
    import torch

    from .adjoint import PARAM_NAMES, soft_loss

    p0 = np.asarray(prob.initial_params() if params0 is None else params0, dtype=np.float64)
    sel = [PARAM_NAMES.index(w) for w in which]
    if np.any(p0[sel] == 0.0):
        raise ValueError("relative units need nonzero starting values")
    lim = np.asarray(prob.param_bounds() if bounds is None else bounds, dtype=np.float64)[sel]
    lo_u = torch.tensor(np.minimum(lim[:, 0] / p0[sel], lim[:, 1] / p0[sel]), dtype=torch.float64)
    hi_u = torch.tensor(np.maximum(lim[:, 0] / p0[sel], lim[:, 1] / p0[sel]), dtype=torch.float64)
    base = torch.tensor(p0, dtype=torch.float64)
    u = torch.ones(len(sel), dtype=torch.float64, requires_grad=True)
    scale = torch.tensor(p0[sel], dtype=torch.float64)
    opt = torch.optim.Adam([u], lr=lr)
    hist_p, hist_loss = [], []
    t0 = time.perf_counter()
    for k in range(steps):
        prob.seed = seed0 + k
        p = base.clone()
        p[sel] = scale * u
        loss = -soft_loss(p, prob, engine)
        opt.zero_grad()
        loss.backward()
        opt.step()
        with torch.no_grad():
            u.copy_(torch.minimum(torch.maximum(u, lo_u), hi_u))
        hist_loss.append(-float(loss.detach()))
        hist_p.append(p.detach().numpy()[sel].copy())
    final = p0.copy()
    final[sel] = (scale * u).detach().numpy()
    return {"params": final, "which": list(which), "transmission": np.array(hist_loss),
            "trajectory": np.array(hist_p), "seconds": time.perf_counter() - t0, "steps": steps}
