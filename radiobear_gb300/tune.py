"""Autotuner for the absorption line sums.

The line-sum kernel's tiling (frequency slots per thread M, warps per CTA W,
lines per work item) trades shared-record reuse against occupancy and load
balance, and the best choice depends on the number of frequencies, layers
and lines.  ``tune_alpha`` times a caller-supplied step (any sequence of
library calls on the engine, e.g. one batched forward + adjoint, or one
image) for each candidate tiling with CUDA events and leaves the fastest
one set on the engine.

Results are cached per key -- the device, the kind of step, the number of
frequencies, the layer range, the line counts per family and the rays --
in memory and in a JSON file (``RB_TUNING_CACHE``, default
``~/.cache/radiobear_gb300/tuning.json``), so a later process on the same
kind of GPU and workload skips the search.
"""
from __future__ import annotations

import itertools
import json
import os

_CACHE = {}

DEFAULT_CANDIDATES = tuple(itertools.product((2, 4), (1, 2, 4), (512, 1024)))


def cache_path():
    return os.environ.get('RB_TUNING_CACHE') or os.path.join(
        os.path.expanduser('~'), '.cache', 'radiobear_gb300', 'tuning.json')


def _device_name():
    try:
        import torch
        return torch.cuda.get_device_name()
    except Exception:
        return 'unknown'


def workload_key(kind, wl, rays, layers=None):
    """Cache key of a step: kind, frequencies, layer range, line counts per
    catalogue, rays.  ``wl`` is a synthetic workload (freqs, gas, lines) or
    any object with those entries; ``layers`` overrides the layer range
    (e.g. (300, 1200) for a batch)."""
    nL = layers if layers is not None else (int(wl['gas'].shape[1]),) * 2
    counts = {name: int(len(next(iter(tab.values())))) for name, tab in sorted(wl['lines'].items())
              if isinstance(tab, dict) and tab}
    return dict(kind=kind, nf=int(len(wl['freqs'])), layers=[int(nL[0]), int(nL[1])], lines=counts,
                rays=int(rays))


def _key_str(key):
    return json.dumps(dict(key, device=_device_name()), sort_keys=True)


def _load():
    try:
        with open(cache_path()) as fp:
            return json.load(fp)
    except (OSError, ValueError):
        return {}


def _store(k, best, times):
    path = cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        data = _load()
        data[k] = dict(best=list(best), ms={'{},{},{}'.format(*c): v for c, v in times.items()})
        tmp = path + '.tmp'
        with open(tmp, 'w') as fp:
            json.dump(data, fp, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass                       # a read-only home: the in-memory cache still holds it


def tune_alpha(engine, step, key=None, candidates=DEFAULT_CANDIDATES, reps=3, stream=None):
    """Time ``step()`` for each (M, W, item_lines) candidate; set and return
    the fastest.  ``step`` must enqueue its work on ``stream`` (default: the
    current torch stream).  ``key`` (a dict from :func:`workload_key`, or
    None for no caching) selects the cache entry.  Returns (best,
    {candidate: ms}); a cached result returns the times it was chosen by."""
    import torch
    k = _key_str(key) if key is not None else None
    if k is not None:
        hit = _CACHE.get(k)
        if hit is None:
            rec = _load().get(k)
            if rec is not None:
                hit = (tuple(rec['best']),
                       {tuple(int(v) for v in c.split(',')): t for c, t in rec['ms'].items()})
                _CACHE[k] = hit
        if hit is not None:
            engine.set_alpha_tiling(*hit[0])
            return hit
    stream = stream or torch.cuda.current_stream()
    times = {}
    for cand in candidates:
        engine.set_alpha_tiling(*cand)
        step()                       # plan + warm-up
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(reps)]
        for s, e in ev:
            s.record(stream)
            step()
            e.record(stream)
        torch.cuda.synchronize()
        times[cand] = min(s.elapsed_time(e) for s, e in ev)
    best = min(times, key=times.get)
    engine.set_alpha_tiling(*best)
    if k is not None:
        _CACHE[k] = (best, times)
        _store(k, best, times)
    return best, times
