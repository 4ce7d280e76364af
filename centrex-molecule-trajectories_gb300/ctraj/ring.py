"""HBM ring of recorded trajectories (ctraj_run_ring).

The reference keeps full ``Trajectory`` objects of the molecules whose label
is in ``apertures_of_interest`` (trajectory_simulator.py:75-76); for runs of
1e9 molecules that is replaced by a ring of float32 rows in device memory,
filled during the run for the molecules lost on one lens ("Lens entrance" or
"Inside lens"): the lens entrance state, the state after every ``stride``-th
RK4 step, and the state where the molecule was lost.  Each row is
(x, y, z, vx, vy, vz, t, step).  The ring keeps the latest
``capacity_rows`` rows and ``capacity_molecules`` index entries; older ones
are overwritten.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi

__all__ = ["HBMRing", "RingRecord"]


@dataclass
class RingRecord:
    molecule: int        # index of the molecule in its run (Philox counter - offset)
    label: int           # counter slot it was lost on
    rows: np.ndarray     # (k, 8) float32: x, y, z, vx, vy, vz, t, RK4 step


class HBMRing:
    def __init__(self, capacity_rows: int, capacity_molecules: int, stride: int = 50, device: int = 0):
        import torch

        if capacity_rows < 1 or capacity_molecules < 1 or stride < 1:
            raise ValueError("capacities and stride must be >= 1")
        dev = torch.device("cuda", device)
        self.rows = torch.zeros((int(capacity_rows), 8), dtype=torch.float32, device=dev)
        # ctraj_ring_entry: int64 molecule, uint64 first_row, int32 rows, int32 label
        self.index = torch.zeros((int(capacity_molecules), 3), dtype=torch.int64, device=dev)
        self.heads = torch.zeros(2, dtype=torch.int64, device=dev)
        self.stride = int(stride)

    @property
    def capacity_rows(self) -> int:
        return self.rows.shape[0]

    @property
    def capacity_molecules(self) -> int:
        return self.index.shape[0]

    def reset(self):
        self.heads.zero_()

    def struct(self, lens: int) -> _abi.Ring:
        return _abi.Ring(self.rows.data_ptr(), self.capacity_rows, self.index.data_ptr(),
                         self.capacity_molecules, self.heads.data_ptr(), self.stride, int(lens))

    def counts(self) -> tuple[int, int]:
        """(rows, molecules) appended since the last reset."""
        h = self.heads.cpu().numpy()
        return int(h[0]), int(h[1])

    def read(self) -> list:
        """The records still complete in the ring, oldest first."""
        n_rows, n_mol = self.counts()
        idx = self.index.cpu().numpy()
        rows = self.rows.cpu().numpy()
        cap_r, cap_m = self.capacity_rows, self.capacity_molecules
        out = []
        for e in range(max(0, n_mol - cap_m), n_mol):
            mol, first, packed = idx[e % cap_m]
            k = int(packed & 0xFFFFFFFF)
            label = int(np.int32(np.uint32((int(packed) >> 32) & 0xFFFFFFFF)))
            first = int(np.uint64(np.int64(first)))
            if first + k > n_rows or first < n_rows - cap_r:
                continue  # rows overwritten (or not yet written)
            sel = (np.arange(first, first + k) % cap_r)
            out.append(RingRecord(int(mol), label, rows[sel].copy()))
        return out
