"""Thin ctypes layer over libctraj.so: one Engine = one ctraj_context.

Every call maps a C status to the exception the reference would raise
(``_abi.check``); ctypes releases the GIL for the duration of each call.
There is no CPU fallback: a missing library raises on construction.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _abi
from .compiler import CompiledBeamline

G = 9.80665  # scipy.constants.g, the reference's gravity (molecule.py:15-16,58)


@dataclass
class RunResult:
    counts: np.ndarray                # n_labels + 1 (last = "Detected")
    labels: list                      # slot -> label string
    molecules: int
    molecule_steps: int
    lens_steps: int
    edge_band: int
    table_range: int
    kernels: int
    label: np.ndarray | None = None   # per molecule counter slot (-1 = Detected)
    final: np.ndarray | None = None   # (10, n) last row x, y, z, vx, vy, vz, ax, ay, az, t
    rows: np.ndarray | None = None    # per molecule len(trajectory.t) - 1
    margin: np.ndarray | None = None  # per molecule smallest edge distance (m)
    extra: dict = field(default_factory=dict)

    def counter_dict(self) -> dict:
        names = list(self.labels) + ["Detected"]
        out: dict = {}
        for slot, c in enumerate(self.counts):
            if c:
                out[names[slot]] = out.get(names[slot], 0) + int(c)
        return out

    def label_names(self) -> list:
        names = list(self.labels)
        return [names[s] if s >= 0 else "Detected" for s in self.label]


def _dev_ptr(t):
    """Device pointer of a torch CUDA tensor (or an object exposing data_ptr)."""
    return ctypes.c_void_p(int(t.data_ptr()))


class Engine:
    def __init__(self, device: int = 0):
        self.lib = _abi.load_library()
        self.ctx = ctypes.c_void_p()
        _abi.check(self.lib.ctraj_create(int(device), ctypes.byref(self.ctx)), self.lib)
        self.device = device
        self._loaded = None
        self._keep = None

    def close(self):
        if self.ctx:
            self.lib.ctraj_destroy(self.ctx)
            self.ctx = ctypes.c_void_p()

    def __del__(self):  # pragma: no cover - interpreter shutdown order
        try:
            self.close()
        except Exception:
            pass

    def set_stream(self, stream_handle: int | None):
        _abi.check(self.lib.ctraj_set_stream(self.ctx, ctypes.c_void_p(stream_handle or 0)), self.lib)

    def synchronize(self):
        _abi.check(self.lib.ctraj_synchronize(self.ctx), self.lib)

    def set_tuning(self, chunk_first: int = 64, chunk_growth: int = 200, chunk_max: int = 1024,
                   front_waves: int = 4, lens_mode: int = _abi.LENS_PERSISTENT, lens_interval: int = 256,
                   front_threads: int = 256, batch_group: int = 4, lens_threads: int = 512,
                   lens_molecules: int = 1, batch_lens_threads: int = 1024, lens_service: int = 64):
        """ctraj_set_tuning: chunked-lens knobs, front grid and block size, the
        FP32 lens pass (persistent or chunked) with its compaction and service
        intervals, and the runs of a batch that share one lens pass."""
        t = _abi.Tuning(int(chunk_first), int(chunk_growth), int(chunk_max), int(front_waves), int(lens_mode),
                        int(lens_interval), int(front_threads), int(batch_group), int(lens_threads),
                        int(lens_molecules), int(batch_lens_threads), int(lens_service))
        _abi.check(self.lib.ctraj_set_tuning(self.ctx, ctypes.byref(t)), self.lib)

    def get_tuning(self) -> dict:
        t = _abi.Tuning()
        _abi.check(self.lib.ctraj_get_tuning(self.ctx, ctypes.byref(t)), self.lib)
        return {k: int(getattr(t, k)) for k, _ in _abi.Tuning._fields_}

    def load(self, cb: CompiledBeamline):
        """Upload a compiled beamline and its force tables (skipped when already loaded)."""
        if self._loaded is cb:
            return
        for tid, t in enumerate(cb.tables):
            st = t.as_struct()
            _abi.check(self.lib.ctraj_set_force_table(self.ctx, tid, ctypes.byref(st)), self.lib)
        _abi.check(self.lib.ctraj_set_beamline(self.ctx, cb.elements, cb.n_elements, len(cb.labels)),
                   self.lib)
        self._loaded = cb
        self._sweep_tables = None

    def load_sweep_tables(self, cb: CompiledBeamline, tables) -> list:
        """Upload a sweep's Stark tables after the beamline's own; returns their table ids
        (skipped when the same tables are already loaded for this beamline)."""
        self.load(cb)
        tables = list(tables)
        base = len(cb.tables)
        if base + len(tables) > _abi.MAX_TABLES:
            raise ValueError(f"at most {_abi.MAX_TABLES} force tables (beamline {base} + sweep {len(tables)})")
        key = tuple(id(t) for t in tables)
        if getattr(self, "_sweep_tables", None) != key:
            for k, t in enumerate(tables):
                st = t.as_struct()
                _abi.check(self.lib.ctraj_set_force_table(self.ctx, base + k, ctypes.byref(st)), self.lib)
            self._sweep_tables = key
            self._sweep_keep = tables
        return [base + k for k in range(len(tables))]

    def run_sweep(self, cb: CompiledBeamline, tables, alpha, table_index, n_molecules, ics=None,
                  xdist=None, vdist=None, seed: int = 0, offset: int = 0, g: float = G,
                  use_graph: bool = True, timing: bool = False) -> dict:
        """ctraj_run_sweep: configuration c uses Stark table tables[table_index[c]] with
        field coefficient alpha[c] and n_molecules[c] molecules.  Returns
        {"counts": (n_configs, n_labels + 1), "totals", "stats", "extra"}."""
        ids = self.load_sweep_tables(cb, tables)
        alpha = np.ascontiguousarray(alpha, dtype=np.float64)
        n_mol = np.ascontiguousarray(n_molecules, dtype=np.int64)
        tid = np.ascontiguousarray(np.asarray(ids, np.int32)[np.asarray(table_index, np.int64)],
                                   dtype=np.int32)
        if not (alpha.shape == n_mol.shape == tid.shape) or alpha.ndim != 1:
            raise ValueError("alpha, table_index and n_molecules must be 1-D of equal length")
        n = int(n_mol.sum())
        a, keep = self._args(n, 32, ics, xdist, vdist, seed, offset, g)
        a.timing = 1 if timing else 0
        nl = len(cb.labels)
        totals = np.zeros(nl + 1, np.int64)
        a.counts = totals.ctypes.data
        counts = np.zeros((alpha.size, nl + 1), np.int64)
        sw = _abi.Sweep(int(alpha.size), 1 if use_graph else 0, n_mol.ctypes.data, alpha.ctypes.data,
                        tid.ctypes.data)
        st = _abi.RunStats()
        status = self.lib.ctraj_run_sweep(self.ctx, ctypes.byref(sw), ctypes.byref(a),
                                          counts.ctypes.data, ctypes.byref(st))
        del keep
        _abi.check(status, self.lib)
        extra = {}
        if st.timed:
            extra.update(front_ms=float(st.front_ms), lens_ms=float(st.lens_ms))
        stats = dict(molecules=int(st.molecules), molecule_steps=int(st.molecule_steps),
                     lens_steps=int(st.lens_steps), table_range=int(st.table_range),
                     kernels=int(st.kernels))
        return {"counts": counts, "totals": totals, "stats": stats, "extra": extra}

    def _args(self, n, precision, ics, xdist, vdist, seed, offset, g):
        a = _abi.RunArgs()
        a.n = int(n)
        a.precision = int(precision)
        a.seed = int(seed) & 0xFFFFFFFFFFFFFFFF
        a.offset = int(offset) & 0xFFFFFFFFFFFFFFFF
        a.g = float(g)
        keep = []
        if ics is None:
            if xdist is None or vdist is None:
                raise ValueError("either ics or both device distributions are required")
            a.ic_mode = _abi.IC_DEVICE_DRAW
            a.xdist = xdist
            a.vdist = vdist
        elif isinstance(ics, np.ndarray):
            arr = np.ascontiguousarray(ics, dtype=np.float64)
            if arr.shape != (6, n):
                raise ValueError(f"ics must have shape (6, {n}), got {arr.shape}")
            keep.append(arr)
            a.ic_mode = _abi.IC_HOST
            a.ics = arr.ctypes.data
        else:  # torch CUDA tensor (6, n) float64, contiguous
            if tuple(ics.shape) != (6, n) or not ics.is_contiguous() or str(ics.dtype) != "torch.float64":
                raise ValueError("device ics must be a contiguous (6, n) float64 tensor")
            keep.append(ics)
            a.ic_mode = _abi.IC_DEVICE
            a.ics = int(ics.data_ptr())
        return a, keep

    def run(self, cb: CompiledBeamline, n: int, precision: int = 32, ics=None, xdist=None,
            vdist=None, seed: int = 0, offset: int = 0, g: float = G, outputs: bool = False,
            device_outputs: dict | None = None, timing: bool = False, ring=None) -> RunResult:
        """ctraj_run; with ``ring`` (a ctraj.ring.HBMRing) ctraj_run_ring, which
        also appends the molecules lost on the first lens to the ring."""
        self.load(cb)
        a, keep = self._args(n, precision, ics, xdist, vdist, seed, offset, g)
        a.timing = 1 if timing else 0
        nl = len(cb.labels)
        counts = np.zeros(nl + 1, np.int64)
        a.counts = counts.ctypes.data
        res_extra = {}
        label = final = rows = margin = None
        if device_outputs is not None:
            a.out_mode = _abi.OUT_DEVICE
            for k in ("label", "final", "rows", "margin"):
                if k in device_outputs:
                    setattr(a, f"out_{k}", int(device_outputs[k].data_ptr()))
        elif outputs:
            a.out_mode = _abi.OUT_HOST
            label = np.empty(n, np.int32)
            final = np.empty((10, n), np.float64)
            rows = np.empty(n, np.int32)
            margin = np.empty(n, np.float64)
            a.out_label, a.out_final = label.ctypes.data, final.ctypes.data
            a.out_rows, a.out_margin = rows.ctypes.data, margin.ctypes.data
        st = _abi.RunStats()
        if ring is None:
            status = self.lib.ctraj_run(self.ctx, ctypes.byref(a), ctypes.byref(st))
        else:
            lenses = [i for i, e in enumerate(cb.elements) if e.type == _abi.ELECTROSTATIC_LENS]
            rs = ring.struct(lenses[0] if lenses else -1)
            status = self.lib.ctraj_run_ring(self.ctx, ctypes.byref(a), ctypes.byref(rs), ctypes.byref(st))
        del keep
        _abi.check(status, self.lib)
        res_extra["max_lens_steps"] = int(st.max_lens_steps)
        res_extra["linear_tables"] = int(st.linear_tables)
        if st.timed:
            res_extra.update(front_ms=float(st.front_ms), lens_ms=float(st.lens_ms))
        return RunResult(counts=counts, labels=list(cb.labels), molecules=st.molecules,
                         molecule_steps=st.molecule_steps, lens_steps=st.lens_steps,
                         edge_band=st.edge_band, table_range=st.table_range, kernels=st.kernels,
                         label=label, final=final, rows=rows, margin=margin, extra=res_extra)

    def run_batch(self, cb: CompiledBeamline, n: int, seeds, precision: int = 32, ics=None, xdist=None,
                  vdist=None, offset: int = 0, g: float = G, timing: bool = False,
                  l2_flush_bytes: int = 0) -> list:
        """ctraj_run_batch: one run per entry of ``seeds`` (with device draws) or
        of ``ics`` (a list of (6, n) arrays or tensors), pipelined over two
        lanes, groups of ``batch_group`` runs sharing each lens pass; result k
        equals ``run(cb, n, seed=seeds[k], ...)``.  ``n`` is one molecule count
        for every run or a list of them."""
        self.load(cb)
        if ics is not None:
            ics_list = list(ics)
            seeds = list(seeds) if seeds is not None else [0] * len(ics_list)
            if len(seeds) != len(ics_list):
                raise ValueError("seeds and ics must have the same length")
        else:
            seeds = list(seeds)
            ics_list = [None] * len(seeds)
        n_runs = len(seeds)
        ns = [int(x) for x in n] if np.ndim(n) else [int(n)] * n_runs
        if len(ns) != n_runs:
            raise ValueError("one molecule count per run")
        nl = len(cb.labels)
        args = (_abi.RunArgs * max(n_runs, 1))()
        stats = (_abi.RunStats * max(n_runs, 1))()
        counts = [np.zeros(nl + 1, np.int64) for _ in range(n_runs)]
        keep = []
        for k in range(n_runs):
            a, kk = self._args(ns[k], precision, ics_list[k], xdist, vdist, seeds[k], offset, g)
            a.timing = 1 if timing else 0
            a.counts = counts[k].ctypes.data
            args[k] = a
            keep.append(kk)
        status = self.lib.ctraj_run_batch(self.ctx, args, n_runs, stats, int(l2_flush_bytes))
        del keep
        _abi.check(status, self.lib)
        out = []
        for k in range(n_runs):
            st = stats[k]
            extra = {"max_lens_steps": int(st.max_lens_steps), "linear_tables": int(st.linear_tables)}
            if st.timed:
                extra.update(front_ms=float(st.front_ms), lens_ms=float(st.lens_ms))
            out.append(RunResult(counts=counts[k], labels=list(cb.labels), molecules=st.molecules,
                                 molecule_steps=st.molecule_steps, lens_steps=st.lens_steps,
                                 edge_band=st.edge_band, table_range=st.table_range, kernels=st.kernels,
                                 extra=extra))
        return out

    def plane(self, cb: CompiledBeamline, n: int, ids, z: float, precision: int = 32, ics=None, xdist=None,
              vdist=None, seed: int = 0, offset: int = 0, g: float = G) -> np.ndarray:
        """ctraj_plane: (len(ids), 8) x, y, z, vx, vy, vz, status, 0 of molecules `ids` of a run
        at the plane z (status 0: ends before the plane)."""
        self.load(cb)
        a, keep = self._args(n, precision, ics, xdist, vdist, seed, offset, g)
        counts = np.zeros(len(cb.labels) + 1, np.int64)
        a.counts = counts.ctypes.data
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        out = np.empty((ids.size, 8), np.float64)
        status = self.lib.ctraj_plane(self.ctx, ctypes.byref(a), ids.ctypes.data, ids.size, float(z),
                                      out.ctypes.data)
        del keep
        _abi.check(status, self.lib)
        return out

    def record(self, cb: CompiledBeamline, n: int, ids, stride: int = 1, max_rows: int = 64,
               precision: int = 32, ics=None, xdist=None, vdist=None, seed: int = 0,
               offset: int = 0, g: float = G):
        """Replay molecules `ids` of a run and return their rows: list of (k_i, 10) arrays."""
        self.load(cb)
        a, keep = self._args(n, precision, ics, xdist, vdist, seed, offset, g)
        counts = np.zeros(len(cb.labels) + 1, np.int64)
        a.counts = counts.ctypes.data
        ids = np.ascontiguousarray(ids, dtype=np.int64)
        out = np.empty((ids.size, max_rows, 10), np.float64)
        cnt = np.zeros(ids.size, np.int32)
        status = self.lib.ctraj_record(self.ctx, ctypes.byref(a), ids.ctypes.data, ids.size,
                                       int(stride), int(max_rows), out.ctypes.data, cnt.ctypes.data)
        del keep
        _abi.check(status, self.lib)
        return [out[k, :cnt[k]].copy() for k in range(ids.size)]


_default: dict[int, Engine] = {}


def default_engine(device: int = 0) -> Engine:
    if device not in _default:
        _default[device] = Engine(device)
    return _default[device]
