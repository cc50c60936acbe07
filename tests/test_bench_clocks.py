"""bench.py's clock record (CPU): samples of a stand-in nvidia-smi, the
throttle reasons found in them, the timed-region filter and the fallback
period when 50 ms samples are refused."""
import os
import stat
import sys
import textwrap
import time

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402

FAKE = textwrap.dedent('''\
    #!{python}
    import datetime, sys, time
    period = int(sys.argv[sys.argv.index('-lms') + 1])
    if period < {min_period}:
        sys.exit(2)
    i = 0
    while True:
        ts = datetime.datetime.now().strftime('%Y/%m/%d %H:%M:%S.%f')[:-3]
        slow = 'Active' if i == {slow_at} else 'Not Active'
        print('{{}}, 0, {{}}, 2070, 900.5, 0x0, {{}}, Not Active, Not Active, Not Active'.format(
            ts, 2070 if i else 960, slow), flush=True)
        i += 1
        time.sleep(period / 1000.0)
    ''')


def _fake_smi(tmp_path, monkeypatch, min_period=0, slow_at=-1):
    d = tmp_path / 'bin'
    d.mkdir()
    p = d / 'nvidia-smi'
    p.write_text(FAKE.format(python=sys.executable, min_period=min_period, slow_at=slow_at))
    p.chmod(p.stat().st_mode | stat.S_IXUSR)
    monkeypatch.setenv('PATH', str(d) + os.pathsep + os.environ.get('PATH', ''))


def _sample(seconds):
    with bench.ClockSampler(0) as clk:
        t0 = time.time()
        time.sleep(seconds)
        clk.region(t0, time.time())
    return clk.summary()


def test_samples_inside_the_timed_region(tmp_path, monkeypatch):
    _fake_smi(tmp_path, monkeypatch)
    s = _sample(0.3)
    assert s['in_timed_region'] and s['samples'] >= 3
    assert s['sm_mhz'] == 2070.0 and s['sm_max_mhz'] == 2070.0
    assert s['reasons'] == []


def test_hw_slowdown_is_reported(tmp_path, monkeypatch):
    _fake_smi(tmp_path, monkeypatch, slow_at=2)
    s = _sample(0.4)
    assert 'hw_slowdown' in s['reasons']


def test_refused_period_falls_back_to_200_ms(tmp_path, monkeypatch):
    _fake_smi(tmp_path, monkeypatch, min_period=100)
    s = _sample(0.5)
    assert s['samples'] >= 1 and s['sm_mhz'] == 2070.0


def test_no_nvidia_smi(tmp_path, monkeypatch):
    empty = tmp_path / 'empty'
    empty.mkdir()
    monkeypatch.setenv('PATH', str(empty))
    s = _sample(0.0)
    assert s['sm_mhz'] is None and s['reasons'] == ['nvidia-smi unavailable']
