"""Loading helpers for the committed golden fixtures (tests/golden/*.npz)."""
import functools
import os

import numpy as np

from radiobear_gb300 import synth

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), 'golden')
C = {k: i for i, k in enumerate(synth.GAS_COLUMNS)}
REQ, RPOL = synth.JUPITER['Req'], synth.JUPITER['Rpol']


@functools.lru_cache(maxsize=None)
def load(name):
    z = np.load(os.path.join(HERE, name + '.npz'))
    return {k: z[k] for k in z.files}


@functools.lru_cache(maxsize=None)
def real_catalogues():
    z = load('catalogs_real')
    out = {}
    for k, v in z.items():
        cat, col = k.split('__', 1)
        out.setdefault(cat, {})[col] = v
    return out


def gas_table(z):
    """Reference-layout gas table [len(GAS_COLUMNS), nL] from a fixture."""
    g = np.zeros((len(synth.GAS_COLUMNS), len(z['gas_P'])))
    for k in ('Z', 'T', 'P', 'H2', 'HE', 'CH4', 'NH3', 'H2O', 'H2S', 'PH3'):
        g[C[k]] = z['gas_' + k]
    return g


def benchmark_lines():
    c = real_catalogues()
    return dict(ammonia=c['ammonia'], nh3=c['nh3'], h2o=c['h2o'], h2s=c['h2s'],
                ph3=c['ph3'], ph3wgt=c['ph3wgt'])


def c0_lines():
    z = load('c0')
    c = real_catalogues()
    amm = {k[len('ammonia__'):]: v for k, v in z.items() if k.startswith('ammonia__')}
    nh3 = {k[len('nh3__'):]: v for k, v in z.items() if k.startswith('nh3__')}
    return dict(ammonia=amm, nh3=nh3, h2o=c['h2o'], h2s=c['h2s'], ph3=c['ph3'], ph3wgt=c['ph3wgt'])


def c1_workload():
    """Configuration 1 regenerated from its seed, with the real PH3 lines."""
    c = real_catalogues()
    wl = synth.make_workload(1, real=c)
    wl['lines']['ph3wgt'] = c['ph3wgt']
    return wl


def c0_workload():
    c = real_catalogues()
    wl = synth.make_workload(0, real=c)
    wl['lines']['ph3wgt'] = c['ph3wgt']
    return wl
