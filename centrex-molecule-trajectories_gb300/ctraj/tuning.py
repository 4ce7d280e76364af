"""Autotuner for the engine's launch knobs.

The knobs (``ctraj_set_tuning``): which FP32 lens pass runs (one persistent
launch that refills lanes and compacts the last molecules every
``lens_interval`` steps, or chunked launches), the length of the first lens
chunk, the growth of later chunks and their maximum (how often molecules still
inside a lens are compacted into full warps in chunked mode, which FP64 runs
always use), the persistent pass's molecules per CTA (``lens_threads``) and
per thread (``lens_molecules``) and the steps between a warp's refills of
its finished lanes (``lens_service``), the front kernel's grid (``front_waves``)
and block size
(``front_threads``), and how many consecutive runs of a batch share one lens
pass (``batch_group``).  None of them changes a result.
The best setting depends on the beamline: how fast molecules are lost inside
the lens and how long the survivors stay.  ``autotune`` searches one knob at a
time (coordinate descent from the defaults: each axis's values are timed with
the other knobs at their best so far) on the actual workload with CUDA events
-- kernel time of a run for the per-run knobs, the CUDA-event time of a
pipelined batch for ``batch_group`` -- keeps the fastest, applies it to the
engine and caches it per (beamline, molecule count, GPU) in a JSON file.
"""
from __future__ import annotations

import hashlib
import itertools
import json
import os
from pathlib import Path

DEFAULT = dict(chunk_first=64, chunk_growth=200, chunk_max=1024, front_waves=4, lens_mode=0, lens_interval=256,
               front_threads=256, batch_group=4, lens_threads=512, lens_molecules=1, batch_lens_threads=1024,
               lens_service=64)


def axes():
    """The search axes, in order: each is a list of partial settings tried on
    top of the best setting found so far.  First the lens pass (persistent, or
    chunked with each chunk schedule), then the persistent pass's CTA size,
    service and compaction intervals, then the front kernel's grid and block
    size."""
    lens = [dict(lens_mode=0)]
    for cf, g, cm in itertools.product((32, 64, 128), (150, 200, 300), (256, 512, 1024, 2048)):
        if cm >= cf:
            lens.append(dict(lens_mode=1, chunk_first=cf, chunk_growth=g, chunk_max=cm))
    return [lens,
            [dict(lens_threads=lt, lens_molecules=m) for lt in (512, 768, 1024) for m in (1, 2)],
            [dict(lens_service=sv) for sv in (16, 32, 64, 128, 256)],
            [dict(lens_interval=iv) for iv in (64, 128, 256, 512, 1024)],
            [dict(front_waves=fw) for fw in (1, 2, 4, 8)],
            [dict(front_threads=ft) for ft in (128, 256, 512)]]


BATCH_GROUPS = (1, 2, 4, 8, 10, 16, 20, 32)
BATCH_LENS_THREADS = (512, 768, 1024)
BATCH_SERVICE = (32, 64, 128, 256)


def candidates():
    """Every setting the search may time (the axes' values on top of the defaults)."""
    out = [dict(DEFAULT, **v) for axis in axes() for v in axis]
    out += [dict(DEFAULT, batch_group=g, batch_lens_threads=t) for g in BATCH_GROUPS for t in BATCH_LENS_THREADS]
    out += [dict(DEFAULT, lens_service=sv) for sv in BATCH_SERVICE]
    return out


def _cache_path() -> Path:
    base = os.environ.get("CTRAJ_CACHE_DIR") or os.path.join(os.path.expanduser("~"), ".cache", "ctraj")
    return Path(base) / "tuning.json"


def workload_key(cb, n: int, device_name: str) -> str:
    h = hashlib.sha256(bytes(cb.elements))
    for t in cb.tables:
        h.update(t.knots.tobytes())
        if t.coef is not None:
            h.update(t.coef.tobytes())
        if t.values is not None:
            h.update(t.values.tobytes())
    # molecule counts within a factor of two share a setting
    return f"{device_name}|{h.hexdigest()[:16]}|{max(0, int(n)).bit_length()}"


def _load_cache() -> dict:
    try:
        return json.loads(_cache_path().read_text())
    except (OSError, ValueError):
        return {}


def _store_cache(cache: dict) -> None:
    try:
        p = _cache_path()
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
        tmp.replace(p)
    except OSError:
        pass  # read-only home: tune again next time


def batch_measure(engine, cb, n: int, run_kwargs: dict, runs: int = 8, l2_flush_bytes: int = 0):
    """A measure for the batch axis: ms per run of ``runs`` runs of n molecules
    as one pipelined ctraj_run_batch (CUDA events on the current stream, which
    the engine must launch on), with ``l2_flush_bytes`` written before each run."""
    import torch

    kw = {k: v for k, v in run_kwargs.items() if k not in ("seed",)}
    kw["l2_flush_bytes"] = l2_flush_bytes
    seeds = [int(run_kwargs.get("seed", 0)) + 1 + k for k in range(runs)]
    stream = torch.cuda.current_stream()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def measure():
        ev0.record(stream)
        engine.run_batch(cb, n, seeds, **kw)
        ev1.record(stream)
        ev1.synchronize()
        return ev0.elapsed_time(ev1) / runs

    return measure


def autotune(engine, cb, n: int, run_kwargs: dict, device_name: str = "gpu", repeats: int = 2,
             use_cache: bool = True, cands=None, measure=None, key_extra: str = "", batch=None) -> dict:
    """Pick the fastest knob setting for this workload; returns {"tuning", "ms", "trials", ...}.

    By default a setting is timed as ``engine.run(cb, n, **run_kwargs)``
    (front + lens kernel time); ``measure`` (a callable returning
    milliseconds under the engine's current tuning) times something else,
    e.g. a batched sweep, and ``key_extra`` keeps its cache entry apart.
    ``cands`` replaces the axis search by an explicit list of settings.
    ``batch`` (a callable like ``batch_measure(...)``) adds the batch axes
    (batch_group x batch_lens_threads, then lens_service, which the batch's
    lens passes share with single runs), timed with it after the per-run
    knobs are fixed."""
    key = workload_key(cb, n, device_name) + key_extra + ("|batch" if batch is not None else "")
    cache = _load_cache() if use_cache else {}
    if use_cache and key in cache:
        engine.set_tuning(**cache[key]["tuning"])
        return dict(cache[key], cached=True)

    def timed(setting, fn):
        engine.set_tuning(**setting)
        best = float("inf")
        for _ in range(repeats):
            if fn is None:
                r = engine.run(cb, n, timing=True, **run_kwargs)
                best = min(best, r.extra["front_ms"] + r.extra["lens_ms"])
            else:
                best = min(best, float(fn()))
        return best

    trials = []
    if cands is not None:
        for cand in cands:
            trials.append((timed(cand, measure), cand))
        trials.sort(key=lambda x: x[0])
        ms, best = trials[0]
    else:
        best, ms = dict(DEFAULT), None
        for axis in axes():
            results = []
            for v in axis:
                setting = dict(best, **v)
                t = timed(setting, measure)
                trials.append((t, setting))
                results.append((t, setting))
            ms, best = min(results, key=lambda x: x[0])
    default_ms = next((t for t, c in trials if c == DEFAULT), None)
    result = {"tuning": best, "ms": ms, "trials": len(trials), "default_ms": default_ms}
    if batch is not None:
        results = []
        for g in BATCH_GROUPS:
            for t in BATCH_LENS_THREADS:
                setting = dict(best, batch_group=g, batch_lens_threads=t)
                results.append((timed(setting, batch), setting))
        bms, best = min(results, key=lambda x: x[0])
        service = []
        for sv in BATCH_SERVICE:
            setting = dict(best, lens_service=sv)
            service.append((bms if sv == best["lens_service"] else timed(setting, batch), setting))
        bms, best = min(service, key=lambda x: x[0])
        result.update(tuning=best, batch_ms_per_run=bms, trials=len(trials) + len(results) + len(service),
                      batch_trials={f"{s['batch_group']}x{s['batch_lens_threads']}": t for t, s in results},
                      batch_service_trials={str(s["lens_service"]): t for t, s in service})
    engine.set_tuning(**best)
    if use_cache:
        cache[key] = result
        _store_cache(cache)
    return dict(result, cached=False)
