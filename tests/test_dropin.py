"""Drop-in classes with the reference's signatures (radiobear_gb300.dropin).

CPU: scale semantics and errors of Alpha.get_layer_scale /
total_layer_alpha (alpha.py:151-259), the alpha cache format
(alpha.py:110-149) and install().  GPU: get_layers, get_alpha_from_calc,
compute_ds and Brightness.single against the reference fixtures, and the
memory / file cache round trips.
"""
import sys
import types
from argparse import Namespace

import numpy as np
import pytest

from radiobear_gb300 import dropin, synth
from tests import goldio as G

LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}


class FakeEngine:
    def set_formalisms(self, *a, **k):
        self.formalisms = (a, k)

    def set_co_clouds(self, *a, **k):
        self.co_clouds = (a, k)


def cpu_alpha(tmp_path=None):
    cfg = Namespace(constituent_alpha=dict(dropin.DEFAULT_CONSTITUENTS), h2state='e',
                    scratch_directory=str(tmp_path) if tmp_path else 'Scratch')
    return dropin.Alpha(config=cfg, engine_=FakeEngine())


def test_layer_scale_semantics():
    a = cpu_alpha()
    assert a.ordered_constituents == ['h2', 'h2o', 'h2s', 'nh3', 'ph3']
    assert a.get_layer_scale(2, 3) == [2.0, 2.0, 2.0]
    assert a.get_layer_scale(False, 2) == [1.0, 1.0]
    assert list(a.get_layer_scale([1.0, 2.0], 2)) == [1.0, 2.0]
    d = a.get_layer_scale({'nh3': [1.0, 0.5]}, 2)
    assert d == [{'nh3': 1.0}, {'nh3': 0.5}]
    with pytest.raises(ValueError, match='Incorrect number of scale layers'):
        a.get_layer_scale([1.0], 2)
    with pytest.raises(ValueError, match='not found as constituent'):
        a.get_layer_scale({'co': [1.0, 1.0]}, 2)
    with pytest.raises(ValueError, match='Incorrect scale for nh3'):
        a.get_layer_scale({'nh3': [1.0]}, 2)


def test_neptune_formalisms_and_other_dict():
    """nh3_dbs_sjs, co_ddb and clouds_idp: sorted constituents and the
    other_dict entries copied from the configuration (alpha.py:80-102);
    CH4 clouds stay off ('ch4_p' is copied, clouds_idp tests 'ch4')."""
    ca = dict(dropin.DEFAULT_CONSTITUENTS, nh3='nh3_dbs_sjs', co='co_ddb', clouds='clouds_idp')
    cfg = Namespace(constituent_alpha=ca, h2state='e', scratch_directory='Scratch', coshape='voigt',
                    water_p=1e-4, ice_p=1e-4, nh4sh_p=0.0, nh3ice_p=1e-4, h2sice_p=1e-4, ch4_p=1e-4)
    eng = FakeEngine()
    a = dropin.Alpha(config=cfg, engine_=eng)
    assert a.ordered_constituents == ['clouds', 'co', 'h2', 'h2o', 'h2s', 'nh3', 'ph3']
    assert a.other_dict['co'] == {'coshape': 'voigt'}
    assert a.other_dict['clouds']['ch4_p'] == 1e-4
    assert eng.formalisms[0][0] == 'nh3_dbs_sjs'
    k = eng.co_clouds[1]
    assert k['co'] is True and k['coshape'] == 'voigt' and k['clouds'] is a.other_dict['clouds']
    from radiobear_gb300 import _native
    mask = sum(b for key, b in _native.CLOUD_BITS.items() if k['clouds'].get(key, 0) > 0)
    assert mask == _native.CLOUD_BITS['water_p'] | _native.CLOUD_BITS['ice_p'] | \
        _native.CLOUD_BITS['nh3ice_p'] | _native.CLOUD_BITS['h2sice_p']
    m = a._scale_matrix([{'co': 2.0, 'clouds': 0.5}])
    assert m[0, _native.GASES.index('co')] == 2.0 and m[0, _native.GASES.index('clouds')] == 0.5
    with pytest.raises(ValueError, match='not on the GPU path'):
        dropin.Alpha(config=Namespace(constituent_alpha={'hcn': 'hcn_x'}), engine_=FakeEngine())


def test_scale_matrix_and_total():
    a = cpu_alpha()
    m = a._scale_matrix([2.0, {'nh3': 0.5, 'h2o': 3.0}])
    assert np.all(m[0] == 2.0)
    assert m[1, 3] == 0.5 and m[1, 1] == 3.0 and m[1, 0] == 1.0
    a._save_alpha_memfil = False
    absorb = np.arange(10.0).reshape(2, 5)
    assert np.allclose(a.total_layer_alpha(absorb, 2.0), 2.0 * absorb.sum(axis=1))
    want = (absorb * np.array([1, 3.0, 1, 0.5, 1])).sum(axis=1)
    assert np.allclose(a.total_layer_alpha(absorb, {'nh3': 0.5, 'h2o': 3.0}), want)


def test_alpha_cache_format(tmp_path):
    a = cpu_alpha(tmp_path)
    a.freqs = np.array([1.0, 2.0])
    a.P = np.array([0.1, 1.0, 10.0])
    a.tosave = list(np.random.default_rng(0).random((3, 2, 5)))
    a.save_alpha_data('file')
    z = np.load(a.alphafile)
    assert sorted(z.files) == ['P', 'alpha_data', 'freqs', 'ordered_constituents']
    assert z['alpha_data'].shape == (3, 2, 5)
    b = cpu_alpha(tmp_path)
    b.read_alpha_data('file')
    assert np.array_equal(b.alpha_data, z['alpha_data'])
    a.save_alpha_data('memory')
    assert a.memory.alpha_data.shape == (3, 2, 5)


def test_install_patches_package():
    pkg = types.ModuleType('fakerb')
    pkg.__file__ = '/nonexistent/fakerb/__init__.py'
    al = types.ModuleType('fakerb.alpha')
    rp = types.ModuleType('fakerb.raypath')
    br = types.ModuleType('fakerb.brightness')
    al.Alpha = type('Alpha', (), {'get_layers': lambda self: None})
    rp.Ray = dropin.Ray
    rp.compute_ds = lambda *a: None
    br.Brightness = type('Brightness', (), {'single': lambda self: None})
    br.ray = rp
    saved = {k: sys.modules.get(k) for k in ('fakerb', 'fakerb.alpha', 'fakerb.raypath', 'fakerb.brightness')}
    sys.modules.update({'fakerb': pkg, 'fakerb.alpha': al, 'fakerb.raypath': rp, 'fakerb.brightness': br})
    try:
        out = dropin.install(pkg, lines={}, engine_=FakeEngine())
    finally:
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    assert al.Alpha.get_layers.__name__ == 'get_layers' and rp.compute_ds is out['compute_ds']
    assert br.ray.compute_ds is out['compute_ds']
    assert br.Brightness.single.__name__ == 'single'


# ------------------------------------------------------------------ GPU
def bench_atm():
    z = G.load('benchmark')
    gas = G.gas_table(z)
    prop = np.zeros((len(synth.PROPERTY_COLUMNS), gas.shape[1]))
    prop[LP['R']] = z['prop_R']
    prop[LP['N']] = z['prop_N']
    cfg = Namespace(C=G.C, LP=LP, Req=float(z['Req']), Rpol=float(z['Rpol']), gtype='ellipse',
                    orientation=[0.0, 0.0])
    return z, Namespace(gas=gas, property=prop, config=cfg)


@pytest.fixture(scope='module')
def gpu_alpha():
    from radiobear_gb300 import _native
    e = _native.Engine(0)
    cfg = Namespace(constituent_alpha=dict(dropin.DEFAULT_CONSTITUENTS), h2state='e')
    a = dropin.Alpha(config=cfg, engine_=e, lines=G.benchmark_lines())
    yield a, e
    e.close()


@pytest.mark.gpu
def test_get_layers_benchmark(gpu_alpha):
    a, _ = gpu_alpha
    z, atm = bench_atm()
    lay = a.get_layers(z['freqs'], atm)
    assert lay.shape == z['alpha_layers'].shape
    assert np.max(np.abs(lay - z['alpha_layers']) / np.abs(z['alpha_layers'])) < 1e-5


@pytest.mark.gpu
def test_get_alpha_from_calc_one_layer(gpu_alpha):
    a, _ = gpu_alpha
    z, atm = bench_atm()
    L = 7
    g = a.get_alpha_from_calc(z['freqs'], atm.gas[G.C['T'], L], atm.gas[G.C['P'], L], atm.gas[:, L],
                              G.C, None, None)
    ref = z['alpha_gas'][L]      # [nf, nC] in the reference's ordered constituents
    order = [list(z['ordered_constituents']).index(c) for c in a.ordered_constituents]
    refo = ref[:, order]
    tot = np.abs(ref).sum(axis=1, keepdims=True)
    assert np.max(np.abs(g - refo) / np.maximum(np.abs(refo), 1e-7 * tot)) < 1e-5


@pytest.mark.gpu
def test_alpha_cache_round_trips(gpu_alpha, tmp_path):
    a, _ = gpu_alpha
    z, atm = bench_atm()
    nL = atm.gas.shape[1]
    scale = {'nh3': np.linspace(0.5, 1.5, nL), 'h2o': np.full(nL, 2.0)}
    calc = a.get_layers(z['freqs'], atm, scale=scale, save_alpha='memory')
    again = a.get_layers(z['freqs'], atm, scale=1.0, get_alpha='memory')
    assert np.allclose(again, calc, rtol=1e-12, atol=0)      # stored data are already scaled
    a.alphafile = str(tmp_path / 'alpha0000.npz')
    a.get_layers(z['freqs'], atm, save_alpha='file')
    from_file = a.get_layers(z['freqs'], atm, get_alpha='file')
    plain = a.get_layers(z['freqs'], atm)
    assert np.allclose(from_file, plain, rtol=1e-12, atol=0)


@pytest.mark.gpu
def test_compute_ds_and_brightness_benchmark(gpu_alpha):
    a, e = gpu_alpha
    z, atm = bench_atm()
    for i, b in enumerate(z['b']):
        ray = dropin.compute_ds(atm, b, engine_=e)
        assert np.array_equal(np.array(ray.layer4ds), z['ray{}_layer'.format(i)])
        assert np.max(np.abs(np.array(ray.ds) - z['ray{}_ds'.format(i)]) / z['ray{}_ds'.format(i)]) < 5e-7
    a.get_layers(z['freqs'], atm)
    br = dropin.Brightness(engine_=e)
    for i, b in enumerate(z['b']):
        tb = br.single(b, z['freqs'], atm, a)
        assert np.max(np.abs(np.array(tb) - z['Tb'][i])) < 1e-3


class FakeRayEngine:
    """Stands in for the GPU engine: rays with |b| < 0.9 have a 3-segment
    path, the others miss; Tb = 100 + 10 b_x + f."""

    def __init__(self):
        self.calls = []

    def bright_run(self, T, R, N, layers, b, Req, Rpol, orientation=(0.0, 0.0), gtype='ellipse',
                   limb='shape'):
        self.calls.append(('bright_run', len(b)))
        nf = layers.shape[0]
        hit = np.hypot(b[:, 0], b[:, 1]) < 0.9
        Tb = np.where(hit[:, None], 100.0 + 10.0 * b[:, :1] + np.arange(nf)[None, :], 2.725)
        return dict(Tb=Tb, intW=np.ones((len(b), nf)), nseg=np.where(hit, 3, 0).astype(np.int32))

    def raypath(self, R, N, b, Req, Rpol, orientation=(0.0, 0.0), gtype='ellipse', extras=False):
        self.calls.append(('raypath', len(b)))
        ms = 2 * len(R) + 4
        out = dict(nseg=np.array([3], dtype=np.int32), ds=np.zeros((1, ms)),
                   layer=np.zeros((1, ms), dtype=np.int32), r4ds=np.zeros((1, ms)))
        out['ds'][0, :3] = [1.0, 2.0, 3.0]
        out['layer'][0, :3] = [0, 1, 2]
        return out

    def brightness(self, T, layers, nseg, ds, lay, disc=False, profiles=False):
        self.calls.append(('brightness', len(nseg)))
        nf, ms = layers.shape[0], ds.shape[1]
        prof = np.full((1, nf, ms), 0.5)
        return dict(Tb=np.full((1, nf), 123.0), intW=np.ones((1, nf)), tau=prof, W=prof, TbL=prof)


def test_batched_planet_loop_serves_single_and_materialises_lazily():
    """install()'s b-loop batching on a stand-in engine: one bright_run for
    the whole loop, Brightness.single served from it in the loop's order,
    the per-ray path/profiles evaluated only when read, and off-planet rays
    leaving the previous ray's profiles in place (brightness.py:45-50)."""
    eng = FakeRayEngine()
    bright_cls = type('Brightness', (), {'config': None, 'verbose': False})
    for k in dropin._RAY_STATE:
        setattr(bright_cls, k, dropin._RayState(k))
    bright = bright_cls()
    nL = 4
    gas = np.zeros((len(synth.GAS_COLUMNS), nL))
    gas[G.C['T']] = [100.0, 150.0, 200.0, 250.0]
    gas[G.C['P']] = [0.1, 1.0, 10.0, 100.0]
    prop = np.zeros((len(synth.PROPERTY_COLUMNS), nL))
    prop[LP['R']] = [71000.0, 70990.0, 70980.0, 70970.0]
    prop[LP['N']] = 1.0
    cfg = Namespace(C=G.C, LP=LP, Req=71492.0, Rpol=66854.0, gtype='ellipse', orientation=[0.0, 0.0])
    atm = Namespace(gas=gas, property=prop, config=cfg)
    alpha = Namespace(layers=np.full((2, nL), 1e-6), freqs=[1.0, 2.0])
    planet = Namespace(b=[[0.0, 0.0], [0.5, 0.0], [0.95, 0.0]], atmos=[atm], alpha=[alpha],
                       config=Namespace(orientation=[0.0, 0.0]), bright=bright,
                       map_b_to_atm=lambda b: 0)
    dropin._run_batches(planet, eng)
    assert eng.calls == [('bright_run', 3)]
    for bv, want in zip(planet.b, ([100.0, 101.0], [105.0, 106.0], [2.725, 2.725])):
        assert dropin._from_batch(bright, bv, [1.0, 2.0], atm, alpha, None, eng)
        assert np.allclose(bright.Tb, want)
        if bv[0] == 0.5:
            assert eng.calls == [('bright_run', 3)]          # nothing evaluated yet
            assert bright.tau.shape == (2, 3)                # read -> one ray evaluated
            assert [c[0] for c in eng.calls[1:]] == ['raypath', 'brightness']
            assert bright.travel.layer4ds == [0, 1, 2]
    assert bright.travel.ds is None                          # the off-planet ray's empty path
    assert bright.tau.shape == (2, 3)                        # profiles of the previous ray stay
    assert not dropin._from_batch(bright, [0.1, 0.1], [1.0, 2.0], atm, alpha, None, eng)
