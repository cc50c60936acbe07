"""GPU parity: the CUDA path through the C ABI against the reference's
golden fixtures and the CPU oracle.

Tolerances (from the forward-model contract): absorption within 1e-5
relative of the reference's float64 value; brightness temperature within
1 mK; ray-path lengths within 5e-7 relative (float32 steps taken from a
double-float along-ray coordinate).
"""
import numpy as np
import pytest

from tests import goldio as G

pytestmark = pytest.mark.gpu

ALPHA_RTOL = 1e-5
TB_ATOL = 1e-3
DS_RTOL = 5e-7   # float32 steps from a double-float along-ray coordinate


@pytest.fixture(scope='module')
def engine():
    from radiobear_gb300 import _native
    e = _native.Engine(0)
    yield e
    e.close()


def _load(engine, lines):
    from radiobear_gb300 import catalog
    catalog.upload(engine, lines)
    engine.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')


def _X(g):
    from radiobear_gb300._native import x_matrix
    return x_matrix(g, G.C)


def _rel(a, b, floor=0.0):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


# Per-gas values are compared relatively down to 1e-30 cm^-1 (absolutely
# below): the device sums in float32, whose normal range ends at ~1e-38, and
# a gas that far below (C0's H2O in its coldest layers, ~1e-33 of the total)
# underflows there.  Every larger value is held to the 1e-5 relative bar.
GAS_ABS_FLOOR = 1e-30


def _per_gas_err(gas_gpu, gas_ref, ordered):
    """Relative error per gas, each entry against max(|ref|, 1e-30 cm^-1)."""
    slots = {'h2': 0, 'h2o': 1, 'h2s': 2, 'nh3': 3, 'ph3': 4}
    out = {}
    for k, name in enumerate(ordered):
        a = gas_gpu[:, :, slots[str(name)]]
        r = gas_ref[:, :, k]
        den = np.maximum(np.abs(r), GAS_ABS_FLOOR)
        out[str(name)] = float(np.max(np.abs(a - r) / den))
    return out


def test_alpha_benchmark_case(engine):
    z = G.load('benchmark')
    _load(engine, G.benchmark_lines())
    g = G.gas_table(z)
    lay, gas = engine.alpha(g[G.C['P']], g[G.C['T']], _X(g), z['freqs'], per_gas=True)
    err = _per_gas_err(gas, z['alpha_gas'], z['ordered_constituents'])
    print('benchmark per-gas rel err', err)
    assert max(err.values()) < ALPHA_RTOL
    assert _rel(lay, z['alpha_layers']) < ALPHA_RTOL


def test_alpha_c0(engine):
    z = G.load('c0')
    _load(engine, G.c0_lines())
    g = G.gas_table(z)
    lay, gas = engine.alpha(g[G.C['P']], g[G.C['T']], _X(g), z['freqs'], per_gas=True)
    err = _per_gas_err(gas, z['alpha_gas'], z['ordered_constituents'])
    print('c0 per-gas rel err', err)
    assert max(err.values()) < ALPHA_RTOL
    assert _rel(lay, z['alpha_layers']) < ALPHA_RTOL


def test_alpha_c1_layers_with_blend(engine):
    z = G.load('c1_alpha')
    wl = G.c1_workload()
    _load(engine, wl.lines)
    g = G.gas_table(z)[:, z['layers']]
    lay, gas = engine.alpha(g[G.C['P']], g[G.C['T']], _X(g), z['freqs'], per_gas=True)
    err = _per_gas_err(gas, z['alpha_gas'], z['ordered_constituents'])
    print('c1 per-gas rel err', err)
    assert max(err.values()) < ALPHA_RTOL
    tot = z['alpha_gas'].sum(axis=2).T
    assert _rel(lay, tot) < ALPHA_RTOL


@pytest.mark.parametrize('tiling', [(2, 1, 128), (2, 2, 256), (2, 4, 512), (4, 1, 128),
                                    (4, 2, 512), (4, 4, 1024)])
def test_alpha_c1_tilings(engine, tiling):
    """Every line-sum tiling (slots per thread, warps per CTA, lines per
    work item) gives the same absorption within the contract."""
    M, W, lines = tiling
    z = G.load('c1_alpha')
    wl = G.c1_workload()
    _load(engine, wl.lines)
    g = G.gas_table(z)[:, z['layers']]
    engine.set_alpha_tiling(M, W, lines)
    try:
        lay, gas = engine.alpha(g[G.C['P']], g[G.C['T']], _X(g), z['freqs'], per_gas=True)
    finally:
        engine.set_alpha_tiling(0, 0, 0)
    err = _per_gas_err(gas, z['alpha_gas'], z['ordered_constituents'])
    print('c1 tiling', tiling, 'per-gas rel err', err)
    assert max(err.values()) < ALPHA_RTOL


@pytest.mark.parametrize('tiling', [(2, 1, 128), (4, 2, 128)])
def test_alpha_benchmark_tilings(engine, tiling):
    z = G.load('benchmark')
    _load(engine, G.benchmark_lines())
    g = G.gas_table(z)
    engine.set_alpha_tiling(*tiling)
    try:
        lay, gas = engine.alpha(g[G.C['P']], g[G.C['T']], _X(g), z['freqs'], per_gas=True)
    finally:
        engine.set_alpha_tiling(0, 0, 0)
    err = _per_gas_err(gas, z['alpha_gas'], z['ordered_constituents'])
    assert max(err.values()) < ALPHA_RTOL


def test_raypaths_c0(engine):
    z = G.load('c0')
    out = engine.raypath(z['prop_R'], z['prop_N'], z['rays_b'], G.REQ, G.RPOL)
    for i in range(len(z['rays_b'])):
        ref = z['ray{}_ds'.format(i)]
        n = out['nseg'][i]
        assert n == ref.size, (i, n, ref.size)
        if n:
            assert np.array_equal(out['layer'][i, :n], z['ray{}_layer'.format(i)])
            assert _rel(out['ds'][i, :n], ref) < DS_RTOL


def test_raypaths_tilted(engine):
    z = G.load('c0')
    out = engine.raypath(z['prop_R'], z['prop_N'], z['tilt_b'], G.REQ, G.RPOL,
                         orientation=tuple(z['tilt_orientation']))
    for i in range(len(z['tilt_b'])):
        ref = z['tilt{}_ds'.format(i)]
        n = out['nseg'][i]
        assert n == ref.size
        if n:
            assert np.array_equal(out['layer'][i, :n], z['tilt{}_layer'.format(i)])
            assert _rel(out['ds'][i, :n], ref) < DS_RTOL


def test_raypaths_benchmark(engine):
    z = G.load('benchmark')
    out = engine.raypath(z['prop_R'], z['prop_N'], z['b'], z['Req'], z['Rpol'])
    for i in range(len(z['b'])):
        ref = z['ray{}_ds'.format(i)]
        n = out['nseg'][i]
        assert n == ref.size
        assert np.array_equal(out['layer'][i, :n], z['ray{}_layer'.format(i)])
        assert _rel(out['ds'][i, :n], ref) < DS_RTOL


def test_brightness_kernel_on_reference_paths(engine):
    """Tb scan alone: reference alpha layers and reference ray paths in."""
    z = G.load('c0')
    g = G.gas_table(z)
    nb = len(z['rays_b'])
    ms = 2 * g.shape[1] + 4
    nseg = np.zeros(nb, dtype=np.int32)
    ds = np.zeros((nb, ms))
    lay = np.zeros((nb, ms), dtype=np.int32)
    for i in range(nb):
        r = z['ray{}_ds'.format(i)]
        nseg[i] = r.size
        ds[i, :r.size] = r
        lay[i, :r.size] = z['ray{}_layer'.format(i)]
    out = engine.brightness(g[G.C['T']], z['alpha_layers'], nseg, ds, lay)
    assert np.max(np.abs(out['Tb'] - z['Tb_rays'])) < TB_ATOL


def test_disc_mode_e2(engine):
    z = G.load('c0')
    g = G.gas_table(z)
    out = engine.raypath(z['prop_R'], z['prop_N'], [[0.0, 0.0]], G.REQ, G.RPOL)
    b = engine.brightness(g[G.C['T']], z['alpha_layers'], out['nseg'], out['ds'], out['layer'],
                          disc=True, profiles=True)
    assert np.max(np.abs(b['Tb'][0] - z['Tb_disc'])) < TB_ATOL
    n = out['nseg'][0]
    assert _rel(b['tau'][0, :, :n], z['disc_tau'], floor=1e-30) < 1e-5
    assert _rel(b['intW'][0], z['disc_intW']) < 1e-5


def test_e2_against_scipy(engine):
    from scipy.special import expn
    x = np.concatenate([[0.0, 1e-12, 1e-6, 1e-3], np.linspace(0.01, 1.0, 50),
                        np.linspace(1.0001, 30.0, 80), [50.0, 200.0, 700.0]])
    got = engine.debug_e2(x)
    ref = expn(2, x)
    assert np.max(np.abs(got - ref) / np.maximum(ref, 1e-300)) < 1e-13


def test_e1_against_scipy(engine):
    """E1 = -dE2/dx, the derivative the disc-mode adjoint takes."""
    from scipy.special import exp1
    x = np.concatenate([[1e-12, 1e-6, 1e-3], np.linspace(0.01, 1.0, 50),
                        np.linspace(1.0001, 30.0, 80), [50.0, 200.0, 700.0]])
    got = engine.debug_e1(x)
    ref = exp1(x)
    assert np.max(np.abs(got - ref) / np.maximum(ref, 1e-300)) < 1e-13


def test_forward_benchmark_golden_table(engine):
    """scripts/benchmark.py:20-24 through the fused GPU forward model."""
    z = G.load('benchmark')
    _load(engine, G.benchmark_lines())
    g = G.gas_table(z)
    out = engine.forward(g[G.C['P']], g[G.C['T']], _X(g), z['prop_R'], z['prop_N'], z['freqs'],
                         z['b'], z['Req'], z['Rpol'])
    assert np.max(np.abs(out['Tb'] - z['Tb'])) < TB_ATOL
    assert np.max(np.abs(out['Tb'] - z['T_rb'].astype(np.float64))) < TB_ATOL + 1e-4


def test_forward_c0_rays_and_disc(engine):
    z = G.load('c0')
    _load(engine, G.c0_lines())
    g = G.gas_table(z)
    args = (g[G.C['P']], g[G.C['T']], _X(g), z['prop_R'], z['prop_N'], z['freqs'])
    out = engine.forward(*args, z['rays_b'], G.REQ, G.RPOL)
    assert np.max(np.abs(out['Tb'] - z['Tb_rays'])) < TB_ATOL
    d = engine.forward(*args, [[0.0, 0.0]], G.REQ, G.RPOL, disc=True)
    assert np.max(np.abs(d['Tb'][0] - z['Tb_disc'])) < TB_ATOL


def test_forward_c1_rays(engine):
    z = G.load('c1_tb')
    wl = G.c1_workload()
    _load(engine, wl.lines)
    g = G.gas_table(z)
    out = engine.forward(g[G.C['P']], g[G.C['T']], _X(g), z['prop_R'], z['prop_N'], z['freqs'],
                         z['b'], G.REQ, G.RPOL)
    err = np.max(np.abs(out['Tb'] - z['Tb']))
    print('c1 max |dTb| =', err)
    assert err < TB_ATOL


def test_forward_c1_disc_average_against_oracle(engine):
    """Disc average over the 64-point Gauss-Legendre quadrature: the CPU
    oracle's sum of per-ray Tb against the GPU's fused average."""
    from oracle import oracle as O
    wl = G.c1_workload()
    _load(engine, wl.lines)
    LP = {k: i for i, k in enumerate(__import__('radiobear_gb300.synth', fromlist=['x']).PROPERTY_COLUMNS)}
    R, N = wl.prop[LP['R']], wl.prop[LP['N']]
    g = wl.gas
    out = engine.forward(g[G.C['P']], g[G.C['T']], _X(g), R, N, wl.freqs, wl.b, G.REQ, G.RPOL,
                         weights=wl.weights, want_layers=True)
    per = O.alpha_per_gas(wl.freqs, g, G.C, wl.lines)
    layers, _ = O.total_alpha(per, O.layer_scale(False, g.shape[1]))
    assert _rel(out['layers'], layers) < ALPHA_RTOL
    sel = [0, 7, 31, 63]
    tbs = []
    for k in sel:
        ds, lay = O.compute_ds(R, N, wl.b[k], G.REQ, G.RPOL)
        tb, _, _, _ = O.brightness(ds, lay, layers, g[G.C['T']])
        tbs.append(tb)
    assert np.max(np.abs(out['Tb'][sel] - np.array(tbs))) < TB_ATOL
    avg = np.tensordot(wl.weights, out['Tb'], axes=1)
    # the disc average is a compensated float32 sum over rays
    assert np.max(np.abs(out['Tb_avg'] - avg)) < 2e-5
