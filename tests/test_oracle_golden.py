"""Pins the CPU oracle to the reference: its shipped golden table and
fixtures generated by running the unmodified reference (make_golden.py)."""
import numpy as np
import pytest

from oracle import oracle as O
from tests import goldio as G


def _rel(a, b):
    b = np.asarray(b)
    return np.max(np.where(b != 0, np.abs(a - b) / np.maximum(np.abs(b), 1e-300), np.abs(a)))


def test_benchmark_table_reproduced():
    """scripts/benchmark.py:20-24 expected Tb, reproduced at float32."""
    z = G.load('benchmark')
    g = G.gas_table(z)
    per = O.alpha_per_gas(z['freqs'], g, G.C, G.benchmark_lines())
    layers, _ = O.total_alpha(per, O.layer_scale(False, g.shape[1]))
    assert _rel(per, z['alpha_gas']) < 1e-12
    for i, b in enumerate(z['b']):
        ds, lay = O.compute_ds(z['prop_R'], z['prop_N'], b, z['Req'], z['Rpol'])
        assert np.array_equal(lay, z['ray{}_layer'.format(i)])
        assert _rel(ds, z['ray{}_ds'.format(i)]) < 1e-8
        tb, _, _, _ = O.brightness(ds, lay, layers, g[G.C['T']])
        assert np.max(np.abs(tb - z['Tb'][i])) < 1e-6
        assert np.array_equal(tb.astype(np.float32), z['T_rb'][i])


def test_c0_alpha_per_gas():
    z = G.load('c0')
    per = O.alpha_per_gas(z['freqs'], G.gas_table(z), G.C, G.c0_lines())
    assert _rel(per, z['alpha_gas']) < 1e-12


@pytest.mark.parametrize('i', range(12))
def test_c0_rays_and_tb(i):
    z = G.load('c0')
    g = G.gas_table(z)
    layers = z['alpha_layers']
    b = z['rays_b'][i]
    ds, lay = O.compute_ds(z['prop_R'], z['prop_N'], b, G.REQ, G.RPOL)
    ref = z['ray{}_ds'.format(i)]
    if ref.size == 0:
        assert ds is None
    else:
        assert np.array_equal(lay, z['ray{}_layer'.format(i)])
        assert _rel(ds, ref) < 1e-8
    tb, _, _, _ = O.brightness(ds, lay, layers, g[G.C['T']])
    assert np.max(np.abs(tb - z['Tb_rays'][i])) < 1e-6


@pytest.mark.parametrize('i', range(5))
def test_c0_tilted_planet(i):
    z = G.load('c0')
    g = G.gas_table(z)
    b = z['tilt_b'][i]
    ds, lay = O.compute_ds(z['prop_R'], z['prop_N'], b, G.REQ, G.RPOL, orientation=z['tilt_orientation'])
    ref = z['tilt{}_ds'.format(i)]
    if ref.size == 0:
        assert ds is None
    else:
        assert np.array_equal(lay, z['tilt{}_layer'.format(i)])
        assert _rel(ds, ref) < 1e-8
    tb, _, _, _ = O.brightness(ds, lay, z['alpha_layers'], g[G.C['T']])
    assert np.max(np.abs(tb - z['tilt_Tb'][i])) < 1e-6


def test_c0_disc_e2():
    z = G.load('c0')
    g = G.gas_table(z)
    ds, lay = O.compute_ds(z['prop_R'], z['prop_N'], [0.0, 0.0], G.REQ, G.RPOL)
    tb, tau, W, iw = O.brightness(ds, lay, z['alpha_layers'], g[G.C['T']], disc=True)
    assert np.max(np.abs(tb - z['Tb_disc'])) < 1e-6
    assert _rel(tau, z['disc_tau']) < 1e-8
    assert _rel(iw, z['disc_intW']) < 1e-8


def test_scale_semantics():
    s = G.load('scale_cases')
    z = G.load('c0')
    g = G.gas_table(z)
    per = O.alpha_per_gas(s['freqs'], g, G.C, G.c0_lines())
    nL = g.shape[1]
    cases = dict(plain=False, number=0.5, list=s['list_scale'].tolist(),
                 dict={'nh3': s['dict_nh3'].tolist(), 'h2o': s['dict_h2o'].tolist()})
    for name, sc in cases.items():
        L, _ = O.total_alpha(per, O.layer_scale(sc, nL))
        assert _rel(L, s[name]) < 1e-12, name
    _, cube = O.total_alpha(per, O.layer_scale(False, nL))
    assert _rel(cube, s['saved']) < 1e-12
    pu = O.alpha_per_gas(s['unsorted_freqs'], g, G.C, G.c0_lines())
    L, _ = O.total_alpha(pu, O.layer_scale(False, nL))
    assert _rel(L, s['unsorted']) < 1e-12


def test_c1_alpha_subset_including_blend_layers():
    z = G.load('c1_alpha')
    wl = G.c1_workload()
    g = G.gas_table(z)
    sel = z['layers']
    assert np.allclose(g[G.C['P']][sel], wl.gas[G.C['P']][sel], rtol=1e-14)
    per = O.alpha_per_gas(z['freqs'], g[:, sel], G.C, wl.lines)
    assert _rel(per, z['alpha_gas']) < 1e-11
    assert np.any(g[G.C['P']][sel] > 400.0)       # nh3_hs/nh3_sjs blend covered


def test_c1_tb_rays():
    z = G.load('c1_tb')
    wl = G.c1_workload()
    g = G.gas_table(z)
    per = O.alpha_per_gas(z['freqs'], g, G.C, wl.lines)
    layers, _ = O.total_alpha(per, O.layer_scale(False, g.shape[1]))
    for k, b in enumerate(z['b']):
        ds, lay = O.compute_ds(z['prop_R'], z['prop_N'], b, G.REQ, G.RPOL)
        tb, _, _, _ = O.brightness(ds, lay, layers, g[G.C['T']])
        assert np.max(np.abs(tb - z['Tb'][k])) < 1e-6


def test_synthetic_atmosphere_matches_reference_build():
    """The package's computeProp restatement gives the R/N the reference
    derived from the same gas file."""
    from radiobear_gb300 import synth
    z = G.load('c0')
    wl = G.c0_workload()
    LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
    assert _rel(wl.prop[LP['R']], z['prop_R']) < 1e-14
    assert _rel(wl.prop[LP['N']], z['prop_N']) < 1e-14
    assert _rel(wl.gas[G.C['T']], z['gas_T']) < 1e-15
