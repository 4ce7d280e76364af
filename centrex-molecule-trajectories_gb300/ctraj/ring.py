"""HBM ring of recorded trajectories (ctraj_run_ring).

The reference keeps full ``Trajectory`` objects of the molecules whose label
is in ``apertures_of_interest`` (trajectory_simulator.py:75-76); for runs of
1e9 molecules that is replaced by a ring of float32 rows in device memory,
filled during the run for the molecules lost on one lens ("Lens entrance" or
"Inside lens"): the lens entrance state, the state after every ``stride``-th
RK4 step, and the state where the molecule was lost.  Each row is
(x, y, z, vx, vy, vz, t, step).  The ring keeps the latest
``capacity_rows`` rows and ``capacity_molecules`` index entries; older ones
are overwritten.  A stream of runs keeps every record by draining the ring
between runs (``HBMRing.drain``): the records of the runs since the last
drain go to a consumer -- ``HostRingStore`` copies them to pinned host memory
-- and the ring starts empty again, so it only has to hold one run's records.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi

__all__ = ["HBMRing", "HostRingStore", "RingRecord"]


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

    def drain(self, consumer=None) -> dict:
        """Hand the records appended since the last reset to ``consumer`` and
        empty the ring.  consumer(rows, index) gets the rows (k, 8) float32 and
        the index entries (m, 3) int64 (molecule, first row, rows | label << 32)
        with first_row counted from the start of ``rows``: views of the ring in
        device memory when nothing was overwritten, else host arrays of the
        records still complete.  Returns the rows and molecules appended, and
        those lost because the ring was too small for them."""
        n_rows, n_mol = self.counts()
        out = {"rows": n_rows, "molecules": n_mol, "rows_lost": 0, "molecules_lost": 0}
        if n_rows <= self.capacity_rows and n_mol <= self.capacity_molecules:
            if consumer is not None and (n_rows or n_mol):
                consumer(self.rows[:n_rows], self.index[:n_mol])
        else:  # overwritten: the complete records only
            recs = self.read()
            kept = sum(len(r.rows) for r in recs)
            out.update(rows_lost=n_rows - kept, molecules_lost=n_mol - len(recs))
            if consumer is not None and recs:
                rows = np.concatenate([r.rows for r in recs]).astype(np.float32, copy=False)
                first = np.concatenate([[0], np.cumsum([len(r.rows) for r in recs])[:-1]]).astype(np.int64)
                packed = np.array([len(r.rows) | (int(np.uint32(np.int32(r.label))) << 32) for r in recs],
                                  dtype=np.uint64).view(np.int64)
                index = np.stack([np.array([r.molecule for r in recs], np.int64), first, packed], axis=1)
                consumer(rows, index)
        self.reset()
        return out

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


class HostRingStore:
    """A ring-drain consumer that copies the records to host memory.

    Rows and index entries are copied from the device through a pinned
    staging buffer (grown as needed).  With ``keep`` every record is kept
    (``records()``, first rows counted over all drains); without it the
    records are only copied and counted, for a caller that processes them
    from the staging buffer (``last_rows`` / ``last_index``) before the
    next drain."""

    def __init__(self, keep: bool = True):
        self.keep = keep
        self.rows_total = 0
        self.molecules_total = 0
        self._rows, self._index = [], []
        self._stage_r = self._stage_i = None
        self.last_rows = self.last_index = None

    def _stage(self, buf, shape, dtype):
        import torch

        if buf is None or buf.shape[0] < shape[0]:
            buf = torch.empty((max(shape[0] + shape[0] // 4, 1),) + tuple(shape[1:]), dtype=dtype, pin_memory=True)
        return buf

    def __call__(self, rows, index):
        import torch

        if isinstance(rows, np.ndarray):
            rows, index = torch.from_numpy(rows), torch.from_numpy(index)
        self._stage_r = self._stage(self._stage_r, tuple(rows.shape), rows.dtype)
        self._stage_i = self._stage(self._stage_i, tuple(index.shape), index.dtype)
        r, i = self._stage_r[:rows.shape[0]], self._stage_i[:index.shape[0]]
        r.copy_(rows, non_blocking=True)
        i.copy_(index, non_blocking=True)
        if rows.is_cuda:
            torch.cuda.current_stream(rows.device).synchronize()
        self.last_rows, self.last_index = r, i
        if self.keep:
            self._rows.append(r.numpy().copy())
            ix = i.numpy().copy()
            ix[:, 1] += self.rows_total
            self._index.append(ix)
        self.rows_total += int(rows.shape[0])
        self.molecules_total += int(index.shape[0])

    def records(self) -> list:
        """Every kept record, in the order they were appended."""
        if not self._rows:
            return []
        rows = np.concatenate(self._rows)
        out = []
        for mol, first, packed in np.concatenate(self._index):
            k = int(packed & 0xFFFFFFFF)
            label = int(np.int32(np.uint32((int(packed) >> 32) & 0xFFFFFFFF)))
            out.append(RingRecord(int(mol), label, rows[int(first):int(first) + k].copy()))
        return out
