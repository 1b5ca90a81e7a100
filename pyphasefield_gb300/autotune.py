"""Launch-shape autotuner with a persistent JSON cache.

A tuning problem is a key (kernel family, grid shape, dtype, device name)
and a list of candidate configurations. Each candidate is timed with CUDA
events over a few launches on the caller's stream (after warm-up) and the
fastest is cached in the JSON file named by $PPF_AUTOTUNE_CACHE (default
~/.cache/pyphasefield_gb300/autotune.json), so the search runs once per
machine. Candidates run on scratch copies of the state: tuning never changes
the simulation.
"""
from __future__ import annotations

import json
import os
import threading
from pathlib import Path

import torch

_lock = threading.Lock()
# choices made in this process (per cache file and key): consulted first, so
# that a cache file that cannot be written (read-only home) does not make two
# engines of the same key pick differently
_memory: dict = {}


def cache_path() -> Path:
    p = os.environ.get("PPF_AUTOTUNE_CACHE")
    if p:
        return Path(p)
    return Path.home() / ".cache" / "pyphasefield_gb300" / "autotune.json"


def _load() -> dict:
    p = cache_path()
    try:
        return json.loads(p.read_text())
    except (OSError, ValueError):
        return {}


def _store(cache: dict) -> None:
    p = cache_path()
    try:
        p.parent.mkdir(parents=True, exist_ok=True)
        tmp = p.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1, sort_keys=True))
        os.replace(tmp, p)
    except OSError:
        pass  # a read-only home only costs a re-tune next time


def make_key(family: str, shape, dtype, extra: str = "") -> str:
    dev = torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"
    return f"{family}|{tuple(int(n) for n in shape)}|{dtype}|{dev}|{extra}"


def time_candidate(run, stream: torch.cuda.Stream, warmup: int = 2, reps: int = 10) -> float:
    """Seconds per call of run() on `stream` (CUDA events)."""
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            run()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(reps):
            run()
        e1.record(stream)
    e1.synchronize()
    return e0.elapsed_time(e1) / 1e3 / reps


def pick(key: str, candidates: list, measure) -> dict:
    """Return the cached best candidate for `key`, or time every candidate
    with measure(candidate) -> seconds per unit of work and cache the best."""
    mkey = (str(cache_path()), key)
    with _lock:
        hit = _memory.get(mkey)
        if hit is None:
            hit = _load().get(key)
        if hit is not None and hit.get("config") in candidates:
            _memory[mkey] = hit
            return hit["config"]
    results = []
    for cand in candidates:
        try:
            results.append((measure(cand), cand))
        except Exception:  # a shape the kernel rejects is simply not a candidate
            continue
    if not results:
        raise RuntimeError(f"no autotune candidate ran for {key}")
    best_t, best = min(results, key=lambda r: r[0])
    entry = {"config": best, "seconds": best_t,
             "tried": [{"config": c, "seconds": t} for t, c in results]}
    with _lock:
        _memory[mkey] = entry
        cache = _load()
        cache[key] = entry
        _store(cache)
    return best
