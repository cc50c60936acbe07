"""Run the reference's own ``Planet.run`` on its ``scripts/benchmark.py`` case
(Jupiter, ``Jupiter/config_benchmark.par``, 6 frequencies x 4 equatorial
rays, ``scripts/benchmark.py:10-15``), optionally after
``radiobear_gb300.dropin.install()``, and print one JSON line with the Tb
table, the wall time of the run and the number of ``rb_bright_run`` calls.

    python tests/ref_planet_run.py --ref <folder holding radiobear> [--gpu]

Test tooling: run as a child process by ``tests/test_reference_planet.py``
so the reference's module-level state (formalism modules imported under bare
names, patched classes) stays out of the test process.  It runs in a scratch
working directory that holds the benchmark's ``Jupiter/`` inputs, as the
reference resolves ``<Planet>/<config>`` against the working directory.
"""
import argparse
import json
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(HERE, 'golden'))

FREQS = [0.6, 1.25, 2.6, 5.2, 10, 21.9]                  # scripts/benchmark.py:14


def main():
    p = argparse.ArgumentParser()
    p.add_argument('--ref', required=True)
    p.add_argument('--gpu', action='store_true')
    p.add_argument('--extra-b', default='[]',
                   help='JSON list of further impact parameters after the four of the benchmark')
    a = p.parse_args()
    import refharness as H
    H.set_reference(os.path.abspath(a.ref))
    rb = H.import_reference()
    calls = {'bright_run': 0}
    if a.gpu:
        from radiobear_gb300 import _native, dropin
        eng = _native.Engine(0)
        orig = eng.bright_run

        def counted(*args, **kw):
            calls['bright_run'] += 1
            return orig(*args, **kw)
        eng.bright_run = counted
        dropin.install(rb, engine_=eng)
    b = [[np.sin(np.radians(15.0 * k)), 0.0] for k in range(4)]   # scripts/benchmark.py:15
    b += [list(map(float, v)) for v in json.loads(a.extra_b)]
    cwd = os.getcwd()
    with tempfile.TemporaryDirectory() as work:
        H.benchmark_planet_dir(work)
        os.chdir(work)
        try:
            j = H.make_planet('config_benchmark.par')
            t0 = time.perf_counter()
            j.run(FREQS, b=b, reuse_override='False')
            t1 = time.perf_counter()
            tb = np.array(j.Tb, dtype=np.float64)
            last = dict(tau_shape=list(np.shape(j.bright.tau)),
                        intW=[float(v) for v in np.atleast_1d(j.bright.integrated_W)],
                        nseg=len(j.bright.travel.ds or []))
        finally:
            os.chdir(cwd)
    print(json.dumps(dict(Tb=tb.tolist(), seconds=t1 - t0, bright_run_calls=calls['bright_run'],
                          last_ray=last)))


if __name__ == '__main__':
    main()
