"""Autotuner for the absorption line sums.

The line-sum kernel's tiling (frequency slots per thread M, warps per CTA W,
lines per work item) trades shared-record reuse against occupancy and load
balance, and the best choice depends on the number of frequencies, layers
and lines.  ``tune_alpha`` times a caller-supplied step (any sequence of
library calls on the engine, e.g. one batched forward + adjoint) for each
candidate tiling with CUDA events and leaves the fastest one set on the
engine.  Results are cached per key (e.g. the workload shape) for the
process.
"""
from __future__ import annotations

import itertools

_CACHE = {}

DEFAULT_CANDIDATES = tuple(itertools.product((2, 4), (1, 2, 4), (512, 1024)))


def tune_alpha(engine, step, key=None, candidates=DEFAULT_CANDIDATES, reps=3, stream=None):
    """Time ``step()`` for each (M, W, item_lines) candidate; set and return
    the fastest.  ``step`` must enqueue its work on ``stream`` (default: the
    current torch stream).  Returns (best, {candidate: ms})."""
    import torch
    if key is not None and key in _CACHE:
        best = _CACHE[key][0]
        engine.set_alpha_tiling(*best)
        return _CACHE[key]
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
    if key is not None:
        _CACHE[key] = (best, times)
    return best, times
