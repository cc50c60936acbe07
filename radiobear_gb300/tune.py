"""Autotuner for the kernels' launch shapes.

The line-sum kernel's tiling (frequency slots per thread M, warps per CTA W,
lines per work item) trades shared-record reuse against occupancy and load
balance, and the best choice depends on the number of frequencies, layers
and lines.  ``tune_alpha`` times a caller-supplied step (any sequence of
library calls on the engine, e.g. one batched forward + adjoint, or one
image) for each candidate tiling with CUDA events and leaves the fastest
one set on the engine; ``tune_adjoint`` does the same for the adjoint's
JVP launch shape (frequencies per CTA, resident CTAs per SM) and
``tune_scan`` for the brightness scan's lanes per (ray, chunk) item.

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
        data[k] = dict(best=list(best), ms={','.join(str(x) for x in c): v for c, v in times.items()})
        # one temporary file per process: replicas tuning at once each move a
        # whole file into place (the last one wins; no reader sees a torn one)
        tmp = '{}.{}.tmp'.format(path, os.getpid())
        with open(tmp, 'w') as fp:
            json.dump(data, fp, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass                       # a read-only home: the in-memory cache still holds it


def _search(apply, step, candidates, key, reps, stream):
    """Time ``step()`` under each candidate (``apply(c)`` sets it), keep the
    fastest; cached per key (memory and JSON)."""
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
            apply(hit[0])
            return hit
    stream = stream or torch.cuda.current_stream()
    times = {}
    for cand in candidates:
        cand = tuple(int(v) for v in cand)
        apply(cand)
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
    apply(best)
    if k is not None:
        _CACHE[k] = (best, times)
        _store(k, best, times)
    return best, times


def tune_alpha(engine, step, key=None, candidates=DEFAULT_CANDIDATES, reps=3, stream=None):
    """Time ``step()`` for each (M, W, item_lines) line-sum tiling; set and
    return the fastest.  ``step`` must enqueue its work on ``stream``
    (default: the current torch stream).  ``key`` (a dict from
    :func:`workload_key`, or None for no caching) selects the cache entry.
    Returns (best, {candidate: ms}); a cached result returns the times it
    was chosen by."""
    key = None if key is None else dict(key, knob='alpha_tiling')
    return _search(lambda c: engine.set_alpha_tiling(*c), step, candidates, key, reps, stream)


# (frequencies per CTA, resident CTAs per SM at 256 threads, threads per CTA)
# of the absorption JVP
JVP_CANDIDATES = ((128, 5, 128), (128, 4, 128), (128, 6, 128), (128, 3, 256), (64, 3, 256),
                  (64, 4, 256), (64, 4, 128), (32, 3, 256), (32, 5, 128))


def tune_adjoint(engine, step, key=None, candidates=JVP_CANDIDATES, reps=1, stream=None):
    """The adjoint's JVP launch shape: frequencies per CTA, resident CTAs
    per SM and threads per CTA (rb_set_tuning), timed on the caller's
    forward + adjoint step.  Candidates with more frequencies per CTA than
    the step has are skipped by the caller's choice of list."""
    key = None if key is None else dict(key, knob='jvp')

    def apply(c):
        engine.set_tuning(jvp_freqs=c[0], jvp_ctas=c[1], jvp_threads=c[2] if len(c) > 2 else 0)
    return _search(apply, step, candidates, key, reps, stream)


def tune_scan(engine, step, key=None, candidates=((4,), (8,), (16,)), reps=2, stream=None):
    """Frequency-pair lanes per (ray, chunk) item of the brightness scan."""
    key = None if key is None else dict(key, knob='scan_lanes')
    return _search(lambda c: engine.set_tuning(scan_lanes=c[0]), step, candidates, key, reps, stream)
