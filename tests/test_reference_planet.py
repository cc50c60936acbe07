"""The reference's own Planet.run, routed to the GPU by dropin.install().

Runs the unmodified reference (installed under ``baseline/_ref``) on its
``scripts/benchmark.py`` case in a child process (``tests/ref_planet_run.py``)
twice: as shipped (CPU) and after ``install()``.  After install the whole b
loop is one ``rb_bright_run`` call; the Tb table matches the benchmark's
expected values (``scripts/benchmark.py:20-24``, float32) and the CPU run at
1 mK, including an off-planet ray (T_cmb) and an off-equator ray, and the
per-ray state the loop leaves on ``Planet.bright`` (the last ray's tau
profile, path and integrated weights) is there.
"""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from tests import goldio as G

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF = os.path.join(ROOT, 'baseline', '_ref')
EXTRA_B = [[0.3, 0.4], [0.99, 0.5]]      # off the equator; off the planet


def _run(gpu):
    if not os.path.isdir(os.path.join(REF, 'radiobear')):
        pytest.skip('the reference is not installed under baseline/_ref')
    cmd = [sys.executable, os.path.join(ROOT, 'tests', 'ref_planet_run.py'), '--ref', REF,
           '--extra-b', json.dumps(EXTRA_B)] + (['--gpu'] if gpu else [])
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-3000:]
    return json.loads(r.stdout.strip().splitlines()[-1])


@pytest.mark.gpu
def test_reference_planet_run_after_install():
    gpu = _run(True)
    cpu = _run(False)
    tg, tc = np.array(gpu['Tb']), np.array(cpu['Tb'])
    assert tg.shape == tc.shape == (6, 6)
    assert gpu['bright_run_calls'] == 1          # every numeric ray of the loop in one call
    assert np.max(np.abs(tg - tc)) < 1e-3
    T_rb = G.load('benchmark')['T_rb']
    assert np.max(np.abs(tg[:4] - T_rb)) < 1e-3 + 1e-4
    assert np.all(tg[5] == 2.725) and np.all(tc[5] == 2.725)
    assert gpu['last_ray']['tau_shape'] == cpu['last_ray']['tau_shape']
    assert gpu['last_ray']['nseg'] == cpu['last_ray']['nseg']
    assert np.allclose(gpu['last_ray']['intW'], cpu['last_ray']['intW'], rtol=0, atol=1e-5)
