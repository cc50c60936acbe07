"""Edge cases of the GPU path against the oracle / reference fixtures:
continua only (no line items), frequency counts from 1 to several tiles
(odd counts take the scalar scan), unsorted frequencies straddling 30 GHz
(the nh3_hs output order), a formalism switched on with an empty
catalogue, rays that all miss the planet, and the host-side rejections."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import goldio as G

pytestmark = pytest.mark.gpu

ALPHA_RTOL = 1e-5
TB_ATOL = 1e-3


def _rel(a, b, floor=1e-300):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


@pytest.fixture(scope='module')
def engine():
    from radiobear_gb300 import _native
    e = _native.Engine(0)
    yield e
    e.close()


def _c0():
    z = G.load('c0')
    return z, G.gas_table(z)


def _X(g):
    from radiobear_gb300._native import x_matrix
    return x_matrix(g, G.C)


def _load(engine, lines, nh3='nh3_hs_sjs', h2=True, h2o=True, h2s=True, ph3=True):
    from radiobear_gb300 import catalog
    catalog.upload(engine, lines)
    engine.set_formalisms(nh3, h2, h2o, h2s, ph3, 'e')
    engine.set_co_clouds(co=False)


def test_continua_only(engine):
    """No line family on: the plan has no line items and the assembly
    kernel alone writes H2 CIA."""
    z, g = _c0()
    _load(engine, G.c0_lines(), nh3='off', h2o=False, h2s=False, ph3=False)
    freqs = z['freqs']
    lay, gas = engine.alpha(g[G.C['P']], g[G.C['T']], _X(g), freqs, per_gas=True)
    per = O.alpha_per_gas(freqs, g, G.C, G.c0_lines(), constituents=('h2',))
    assert _rel(gas[:, :, 0], per[:, :, 0]) < ALPHA_RTOL
    assert _rel(lay, per[:, :, 0].T) < ALPHA_RTOL


@pytest.mark.parametrize('nf', [1, 2, 3, 33, 700])
def test_frequency_counts(engine, nf):
    """Absorption and Tb of two rays at nf frequencies (700 spans several
    slot tiles)."""
    z, g = _c0()
    lines = G.c0_lines()
    _load(engine, lines)
    freqs = np.exp(np.linspace(np.log(0.8), np.log(90.0), nf)) if nf > 1 else np.array([22.2])
    out = engine.forward(g[G.C['P']], g[G.C['T']], _X(g), z['prop_R'], z['prop_N'], freqs,
                         [[0.0, 0.0], [0.6, 0.2]], G.REQ, G.RPOL, want_layers=True)
    per = O.alpha_per_gas(freqs, g, G.C, lines)
    layers, _ = O.total_alpha(per, O.layer_scale(False, g.shape[1]))
    assert _rel(out['layers'], layers, 1e-7 * np.abs(layers).max(axis=1, keepdims=True)) < ALPHA_RTOL
    tbs, _, _ = O.forward(g, G.C, z['prop_R'], z['prop_N'], freqs, [[0.0, 0.0], [0.6, 0.2]], lines,
                          G.REQ, G.RPOL)
    assert np.max(np.abs(out['Tb'] - tbs)) < TB_ATOL


def test_unsorted_frequencies_reference_order(engine):
    """Frequencies out of order and straddling 30 GHz: nh3_hs returns the
    <= 30 GHz block then the > 30 GHz block (nh3_hs.py:70-88); the
    reference's own get_layers output is the fixture."""
    s = G.load('scale_cases')
    z, g = _c0()
    _load(engine, G.c0_lines())
    lay, _ = engine.alpha(g[G.C['P']], g[G.C['T']], _X(g), s['unsorted_freqs'])
    assert _rel(lay, s['unsorted'], 1e-7 * np.abs(s['unsorted']).max()) < ALPHA_RTOL


def test_family_on_with_empty_catalogue(engine):
    """h2s_ddb on with no H2S lines uploaded contributes zero (the
    reference's loop over an empty line list)."""
    z, g = _c0()
    lines = dict(G.c0_lines())
    lines.pop('h2s')
    _load(engine, lines)
    _, gas = engine.alpha(g[G.C['P']], g[G.C['T']], _X(g), z['freqs'], per_gas=True)
    assert np.all(gas[:, :, 2] == 0.0)
    per = O.alpha_per_gas(z['freqs'], g, G.C, G.c0_lines(), constituents=('nh3',))
    assert _rel(gas[:, :, 3], per[:, :, 0], 1e-7 * np.abs(per).max()) < ALPHA_RTOL


def test_rays_all_off_the_planet(engine):
    z, g = _c0()
    _load(engine, G.c0_lines())
    b = [[1.2, 0.0], [0.0, 1.5], [-2.0, 3.0]]
    out = engine.forward(g[G.C['P']], g[G.C['T']], _X(g), z['prop_R'], z['prop_N'], z['freqs'], b,
                         G.REQ, G.RPOL)
    assert np.all(out['Tb'] == 2.725)
    rays = engine.raypath(z['prop_R'], z['prop_N'], b, G.REQ, G.RPOL)
    assert np.all(rays['nseg'] == 0)


def test_host_rejections(engine):
    z, g = _c0()
    _load(engine, G.c0_lines())
    P, T, X = g[G.C['P']], g[G.C['T']], _X(g)
    with pytest.raises(ValueError):
        engine.alpha(P[:0], T[:0], X[:, :0], z['freqs'])
    Pb = P.copy()
    Pb[3] = -1.0
    with pytest.raises(ValueError):
        engine.alpha(Pb, T, X, z['freqs'])
    Xb = X.copy()
    Xb[3, 5] = np.nan
    with pytest.raises(ValueError):
        engine.alpha(P, T, Xb, z['freqs'])
    for bad in (-1.0, np.nan, 2.5e4):     # frequencies in [0, 2e4] GHz
        with pytest.raises(ValueError, match='frequency 1'):
            engine.alpha(P, T, X, np.array([10.0, bad]))
        with pytest.raises(ValueError, match='frequency 1'):
            engine.forward(P, T, X, z['prop_R'], z['prop_N'], np.array([10.0, bad]), [[0.0, 0.0]],
                           G.REQ, G.RPOL)
    with pytest.raises(ValueError):
        engine.set_formalisms('nh3_xyz' if False else 'nh3_hs', True, True, True, True, 'x')
    with pytest.raises(ValueError):
        engine.set_alpha_tiling(3, 2, 128)
    with pytest.raises(ValueError):
        engine.set_lines('H2S', {'f0': np.array([-1.0]), 'I0': np.array([1e-20]),
                                 'E': np.array([1.0]), 'GH2S': np.array([1.0])})
