"""CPU: the autotuner's JSON cache (keyed by device, step kind,
frequencies, layer range, line counts and rays) is written and read back,
and a cached key sets its tiling without timing anything."""
import json

import numpy as np
import pytest

pytest.importorskip('torch')

from radiobear_gb300 import tune   # noqa: E402


class FakeEngine:
    def __init__(self):
        self.tiling = None
        self.tuning = {}

    def set_alpha_tiling(self, M=0, W=0, item_lines=0):
        self.tiling = (M, W, item_lines)

    def set_tuning(self, **kw):
        self.tuning.update(kw)


def test_workload_key_and_json_cache(tmp_path, monkeypatch):
    monkeypatch.setenv('RB_TUNING_CACHE', str(tmp_path / 'tuning.json'))
    monkeypatch.setattr(tune, '_CACHE', {})
    wl = dict(freqs=np.ones(8), gas=np.zeros((16, 1000)),
              lines=dict(ammonia=dict(fo=np.ones(1500)), h2o=dict(f_o=np.ones(500))))
    key = tune.workload_key('image', wl, 65536)
    assert key == dict(kind='image', nf=8, layers=[1000, 1000], lines=dict(ammonia=1500, h2o=500),
                       rays=65536)
    k = tune._key_str(dict(key, knob='alpha_tiling'))
    tune._store(k, (2, 1, 1024), {(2, 1, 1024): 1.0, (4, 1, 1024): 1.5})
    on_disk = json.loads((tmp_path / 'tuning.json').read_text())
    assert on_disk[k]['best'] == [2, 1, 1024]

    def never():
        raise AssertionError('a cached key must not time the step')

    eng = FakeEngine()
    best, times = tune.tune_alpha(eng, never, key=key)
    assert best == (2, 1, 1024) and eng.tiling == (2, 1, 1024)
    assert times[(4, 1, 1024)] == 1.5
    other = tune.workload_key('batch', dict(freqs=np.ones(128), lines=wl['lines']), 32,
                              layers=(300, 1200))
    assert tune._key_str(other) not in on_disk


def test_jvp_and_scan_knobs_are_cached_separately(tmp_path, monkeypatch):
    monkeypatch.setenv('RB_TUNING_CACHE', str(tmp_path / 'tuning.json'))
    monkeypatch.setattr(tune, '_CACHE', {})
    key = dict(kind='batch', nf=128, layers=[300, 1200], lines=dict(ammonia=200), rays=32)
    tune._store(tune._key_str(dict(key, knob='jvp')), (64, 4), {(64, 4): 1.0, (128, 3): 2.0})
    tune._store(tune._key_str(dict(key, knob='scan_lanes')), (8,), {(8,): 1.0, (4,): 1.2})

    def never():
        raise AssertionError('a cached key must not time the step')

    eng = FakeEngine()
    assert tune.tune_adjoint(eng, never, key=key)[0] == (64, 4)
    assert tune.tune_scan(eng, never, key=key)[0] == (8,)
    assert eng.tuning == dict(jvp_freqs=64, jvp_ctas=4, jvp_threads=0, scan_lanes=8)


def _write_keys(path, tag, n):
    import os
    os.environ['RB_TUNING_CACHE'] = path
    from radiobear_gb300 import tune as T
    for i in range(n):
        T._store('{}-{}'.format(tag, i), (2, 1, 512), {(2, 1, 512): float(i)})


def test_cache_written_by_replicas_at_once(tmp_path):
    """Replicas under torchrun tune at once and write the same cache: each
    moves a whole file of its own into place, so the file always parses and
    no temporary files are left (entries may be lost to the last writer)."""
    import multiprocessing as mp
    path = str(tmp_path / 'tuning.json')
    ctx = mp.get_context('spawn')
    procs = [ctx.Process(target=_write_keys, args=(path, 'r{}'.format(r), 40)) for r in range(3)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    data = json.loads((tmp_path / 'tuning.json').read_text())
    assert any(k.endswith('-39') for k in data)
    assert sorted(f.name for f in tmp_path.iterdir()) == ['tuning.json']
