"""Autotuner for the engine's launch knobs.

The knobs (``ctraj_set_tuning``): which FP32 lens pass runs (one persistent
launch that refills lanes and compacts the last molecules every
``lens_interval`` steps, or chunked launches), the length of the first lens
chunk, the growth of later chunks and their maximum (how often molecules still
inside a lens are compacted into full warps in chunked mode, which FP64 runs
always use), and the size of the front kernel's grid.
The best setting depends on the beamline: how fast molecules are lost inside
the lens and how long the survivors stay.  ``autotune`` times every candidate
on the actual workload with CUDA events (kernel time of the front and lens
passes), keeps the fastest, applies it to the engine and caches it per
(beamline, molecule count, GPU) in a JSON file.
"""
from __future__ import annotations

import hashlib
import itertools
import json
import os
from pathlib import Path

DEFAULT = dict(chunk_first=64, chunk_growth=200, chunk_max=1024, front_waves=4, lens_mode=0, lens_interval=256)


def candidates():
    """Knob settings to try: the chunked lens pass with each chunk schedule,
    the persistent one with each compaction interval, the front grid."""
    out = []
    for cf, g, cm in itertools.product((32, 64, 128), (150, 200, 300), (256, 512, 1024, 2048)):
        if cm >= cf:
            out.append(dict(DEFAULT, chunk_first=cf, chunk_growth=g, chunk_max=cm, lens_mode=1))
    for iv in (64, 128, 256, 512, 1024):
        out.append(dict(DEFAULT, lens_interval=iv))
    for fw in (1, 2, 8):
        out.append(dict(DEFAULT, front_waves=fw))
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


def autotune(engine, cb, n: int, run_kwargs: dict, device_name: str = "gpu", repeats: int = 2,
             use_cache: bool = True, cands=None, measure=None, key_extra: str = "") -> dict:
    """Pick the fastest knob setting for this workload; returns {"tuning", "ms", "trials"}.

    By default a candidate is timed as ``engine.run(cb, n, **run_kwargs)``;
    ``measure`` (a callable returning milliseconds under the engine's current
    tuning) times something else, e.g. a batched sweep, and ``key_extra``
    keeps its cache entry apart."""
    key = workload_key(cb, n, device_name) + key_extra
    cache = _load_cache() if use_cache else {}
    if use_cache and key in cache:
        engine.set_tuning(**cache[key]["tuning"])
        return dict(cache[key], cached=True)
    trials = []
    for cand in (cands or candidates()):
        engine.set_tuning(**cand)
        best = float("inf")
        for _ in range(repeats):
            if measure is None:
                r = engine.run(cb, n, timing=True, **run_kwargs)
                best = min(best, r.extra["front_ms"] + r.extra["lens_ms"])
            else:
                best = min(best, float(measure()))
        trials.append((best, cand))
    trials.sort(key=lambda x: x[0])
    ms, tuning = trials[0]
    engine.set_tuning(**tuning)
    result = {"tuning": tuning, "ms": ms, "trials": len(trials),
              "default_ms": next((t for t, c in trials if c == DEFAULT), None)}
    if use_cache:
        cache[key] = result
        _store_cache(cache)
    return dict(result, cached=False)
