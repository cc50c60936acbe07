"""Formalisms beside the Jupiter set: nh3_dbs, nh3_dbs_sjs, co_ddb (every
coshape) and clouds_idp (every particle kind).

Pinning: ``tests/golden/f2.npz`` holds the reference's own output
(``Alpha.get_alpha_from_calc`` per layer with its other_dict and cloud
dispatch, plus direct ``co_ddb.alpha`` / ``clouds_idp.alpha`` calls; made by
``tests/golden/make_golden.py f2``).  The CPU tests pin the oracle to it;
the GPU tests hold the CUDA path to it.

Tolerances: the line gases (float32 line sums) within 1e-5 relative, as
for the Jupiter set; co_ddb and clouds_idp are evaluated in float64 on the
device and agree to 1e-10 relative (co 'diff', a difference of two sums
that cancel, is measured against the size of the VVW sum).
"""
import numpy as np
import pytest

from oracle import oracle as O
from radiobear_gb300 import synth
from tests import goldio as G

C = G.C
CL = {k: i for i, k in enumerate(synth.CLOUD_COLUMNS)}
ALPHA_RTOL = 1e-5
EXTRA_RTOL = 1e-10
CLOUD_KEYS = ('water_p', 'ice_p', 'nh4sh_p', 'nh3ice_p', 'h2sice_p', 'ch4_p')
RUNS = (('A', 'nh3_dbs_sjs'), ('B', 'nh3_dbs'))


def f2():
    return G.load('f2')


def f2_lines():
    z = f2()
    lines = dict(G.c0_lines())
    lines['co'] = {k: z['co__' + k] for k in ('f0', 'I0', 'E')}
    return lines


def run_setup(run):
    z = f2()
    ordered = tuple(str(x) for x in z['run{}_ordered'.format(run)])
    other = {'co': {'coshape': str(z['run{}_coshape'.format(run)])},
             'clouds': {k: float(z['run{}_{}'.format(run, k)]) for k in CLOUD_KEYS}}
    return ordered, other


def rel_err(a, r, floor):
    den = np.maximum(np.abs(r), floor)
    return float(np.max(np.where(den > 0, np.abs(a - r) / np.where(den > 0, den, 1.0),
                                 np.abs(a - r))))


# Line gases are compared entry by entry against max(|ref|, 1e-30 cm^-1):
# below that the float32 product of a tiny abundance and a tiny line sum can
# underflow, and such entries are ~1e-30 of any layer total anyway.
GAS_ABS_FLOOR = 1e-30


def gas_errors(per, ref, ordered):
    """Per constituent: line gases against max(|ref|, 1e-30 cm^-1);
    co / clouds against max(|ref|, 1e-12 x their max)."""
    out = {}
    for k, c in enumerate(ordered):
        r, a = ref[:, :, k], per[:, :, k]
        floor = 1e-12 * np.max(np.abs(r)) if c in ('co', 'clouds') else GAS_ABS_FLOOR
        out[c] = rel_err(a, r, floor)
    return out


# ------------------------------------------------------------------ CPU: oracle pin
@pytest.mark.parametrize('run,nh3', RUNS)
def test_oracle_matches_reference_runs(run, nh3):
    z = f2()
    ordered, other = run_setup(run)
    per = O.alpha_per_gas(z['freqs'], z['gas'], C, f2_lines(), constituents=ordered, nh3=nh3,
                          cloud=z['cloud'], Cl=CL, other=other)
    errs = gas_errors(per, z['run{}_alpha'.format(run)], ordered)
    assert max(errs.values()) < 1e-12, errs


@pytest.mark.parametrize('shape', ['vvw', 'diff'])
def test_oracle_co_shapes(shape):
    z = f2()
    g = z['gas']
    a = O.alpha_co_ddb(z['freqs'], g[C['T']], g[C['P']], g[C['H2']], g[C['HE']], g[C['CO']],
                       f2_lines()['co'], coshape=shape)
    r = z['co_' + shape]
    assert rel_err(a, r, 1e-12 * np.max(np.abs(r))) < 1e-12


def test_oracle_clouds_ch4_key():
    """clouds_idp tests the key 'ch4' (not the 'ch4_p' that Alpha copies
    from the configuration), so CH4 clouds only act when called so."""
    z = f2()
    a = O.alpha_clouds_idp(z['freqs'], z['gas'][C['T']], z['cloud'], CL, {'ch4': 1.0})
    r = z['clouds_ch4key']
    assert np.max(r) > 0.0
    assert rel_err(a, r, 1e-300) < 1e-12


def test_water_dielectric_branches():
    """Debye above 0 C, the ice table below, with its extrapolation below
    1e8 Hz and above 1e11 Hz (clouds_idp.py:88-100)."""
    e_warm = O.water_dielectric(10.0, 300.0)
    assert e_warm.real > 4.9 and e_warm.imag < 0.0
    for f in (0.05, 5.0, 150.0):
        e = O.water_dielectric(f, 200.0)
        assert e.real == 3.17 and e.imag < 0.0


# ------------------------------------------------------------------ GPU parity
@pytest.fixture(scope='module')
def engine():
    from radiobear_gb300 import _native
    e = _native.Engine(0)
    yield e
    e.close()


def _gpu_per_gas(engine, run, nh3, coshape=None, clouds=None, units_db=False):
    from radiobear_gb300 import _native, catalog
    z = f2()
    ordered, other = run_setup(run)
    catalog.upload(engine, f2_lines())
    engine.set_formalisms(nh3 if 'nh3' in ordered else 'off', 'h2' in ordered, 'h2o' in ordered,
                          'h2s' in ordered, 'ph3' in ordered, 'e')
    engine.set_co_clouds(co='co' in ordered, coshape=coshape or other['co']['coshape'],
                         clouds=(clouds if clouds is not None else other['clouds'])
                         if 'clouds' in ordered else None)
    g = z['gas']
    X = _native.x_matrix(g, C, z['cloud'], CL)
    lay, gas = engine.alpha(g[C['P']], g[C['T']], X, z['freqs'], per_gas=True, units_db=units_db)
    cols = [_native.GASES.index(c) for c in ordered]
    return ordered, lay, gas[:, :, cols]


@pytest.mark.gpu
@pytest.mark.parametrize('run,nh3', RUNS)
def test_gpu_runs_match_reference(engine, run, nh3):
    z = f2()
    ordered, lay, per = _gpu_per_gas(engine, run, nh3)
    ref = z['run{}_alpha'.format(run)]
    errs = gas_errors(per, ref, ordered)
    for c, e in errs.items():
        assert e < (EXTRA_RTOL if c in ('co', 'clouds') else ALPHA_RTOL), (c, errs)
    tot = ref.sum(axis=2).T
    assert rel_err(lay, tot, GAS_ABS_FLOOR) < ALPHA_RTOL


@pytest.mark.gpu
@pytest.mark.parametrize('shape', ['vvw', 'diff'])
def test_gpu_co_shapes(engine, shape):
    z = f2()
    ordered, _, per = _gpu_per_gas(engine, 'B', 'nh3_dbs', coshape=shape)
    r = z['co_' + shape]
    a = per[:, :, ordered.index('co')]
    # 'diff' = Voigt - VVW cancels where the shapes agree: its rounding is
    # relative to the size of the terms (the VVW sum), not to the difference
    floor = np.abs(z['co_vvw']) if shape == 'diff' else 1e-12 * np.max(np.abs(r))
    assert rel_err(a, r, floor) < EXTRA_RTOL


@pytest.mark.gpu
def test_gpu_clouds_ch4_key(engine):
    z = f2()
    ordered, _, per = _gpu_per_gas(engine, 'B', 'nh3_dbs', clouds={'ch4': 1.0})
    r = z['clouds_ch4key']
    a = per[:, :, ordered.index('clouds')]
    assert rel_err(a, r, 1e-300) < EXTRA_RTOL


@pytest.mark.gpu
def test_gpu_units_db(engine):
    """dB/km output: every gas times 434294.5 (the reference multiplies
    each formalism's result)."""
    z = f2()
    ordered, _, per = _gpu_per_gas(engine, 'A', 'nh3_dbs_sjs', units_db=True)
    ref = z['runA_alpha'] * 434294.5
    errs = gas_errors(per, ref, ordered)
    for c, e in errs.items():
        assert e < (EXTRA_RTOL if c in ('co', 'clouds') else ALPHA_RTOL), (c, errs)


@pytest.mark.gpu
def test_gpu_co_needs_lines(engine):
    from radiobear_gb300 import _native, catalog
    z = f2()
    lines = dict(G.c0_lines())
    catalog.upload(engine, lines)             # no 'co': CO family cleared
    engine.set_formalisms('nh3_dbs', False, False, False, False, 'e')
    engine.set_co_clouds(co=True)
    g = z['gas']
    with pytest.raises(_native.RBError):
        engine.alpha(g[C['P']], g[C['T']], _native.x_matrix(g, C), z['freqs'])
    engine.set_co_clouds(co=False)


# ------------------------------------------------------------------ adjoint
@pytest.mark.gpu
def test_gpu_adjoint_with_co_and_clouds(engine):
    """dTb/dT and dTb/dP with co_ddb ('std' shape) and clouds_idp switched
    on: directional derivatives against central differences of the float64
    oracle (the co / cloud terms are differentiated in float64)."""
    from oracle import adjoint as A
    from radiobear_gb300 import _native, catalog
    z = f2()
    nL = 40
    gas = synth.make_gas_table(nL, 1.0e-3, 700.0)
    gas[C['CO']] = 1.0e-6
    T, P = gas[C['T']], gas[C['P']]
    cloud = np.zeros((len(synth.CLOUD_COLUMNS), nL))
    rng = np.random.default_rng(8)
    cloud[CL['H2O']] = np.where((P > 2.0) & (T < 273.0), 10.0 ** rng.uniform(-5, -3, nL), 0.0)
    cloud[CL['SOLN']] = np.where(T >= 273.0, 10.0 ** rng.uniform(-5, -3, nL), 0.0)
    cloud[CL['NH4SH']] = np.where((P > 1.0) & (P < 10.0), 1e-4, 0.0)
    other = {'co': {'coshape': 'std'}, 'clouds': {'water_p': 1e-4, 'ice_p': 1e-4, 'nh4sh_p': 1e-4}}
    ordered = ('clouds', 'co', 'h2', 'h2o', 'h2s', 'nh3', 'ph3')
    prop = synth.compute_properties(gas)
    LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
    R, N = prop[LP['R']], prop[LP['N']]
    freqs = np.array([1.4, 5.0, 12.0, 22.2, 33.0, 60.0, 115.0])
    b, w = synth.gauss_legendre_disc(3)
    lines = f2_lines()
    catalog.upload(engine, lines)
    engine.set_formalisms('nh3_dbs_sjs', True, True, True, True, 'e')
    engine.set_co_clouds(co=True, coshape='std', clouds=other['clouds'])
    grad = rng.normal(size=freqs.size)
    X = _native.x_matrix(gas, C, cloud, CL)
    out = engine.adjoint(P, T, X, R, N, freqs, b, G.REQ, G.RPOL, grad, weights=w)
    kw = dict(constituents=ordered, nh3='nh3_dbs_sjs', cloud=cloud, Cl=CL, other=other)
    _, _, avg = O.forward(gas, C, R, N, freqs, b, lines, G.REQ, G.RPOL, weights=w, **kw)
    assert np.max(np.abs(out['Tb_avg'] - avg)) < 1e-3
    for k in range(6):
        d = dict(T=rng.normal(0.0, 5.0, nL), P=0.01 * P * rng.normal(0.0, 1.0, nL))
        fd = A.directional_fd(gas, C, R, N, freqs, b, lines, G.REQ, G.RPOL, w, grad, d, h=1e-4, **kw)
        ad = np.dot(out['dT'], d['T']) + np.dot(out['dP'], d['P'])
        assert abs(ad - fd) <= 3e-3 * abs(fd) + 1e-7, (k, ad, fd)
    engine.set_co_clouds(co=False)
    engine.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')


@pytest.mark.gpu
def test_gpu_dropin_get_alpha_from_calc(engine):
    """dropin.Alpha with the Neptune-style formalisms: get_alpha_from_calc
    (gas and cloud columns of one layer) equals the reference's."""
    from argparse import Namespace
    from radiobear_gb300 import dropin
    z = f2()
    ordered, other = run_setup('A')
    ca = dict(nh3='nh3_dbs_sjs', co='co_ddb', clouds='clouds_idp', h2='h2_jj_ddb', h2o='h2o_bk',
              h2s='h2s_ddb', ph3='ph3_jh')
    cfg = Namespace(constituent_alpha=ca, h2state='e', scratch_directory='Scratch',
                    coshape=other['co']['coshape'], **other['clouds'])
    a = dropin.Alpha(config=cfg, engine_=engine, lines=f2_lines())
    assert tuple(a.ordered_constituents) == ordered
    g, cl = z['gas'], z['cloud']
    for L in (0, 10, 30, 47):
        got = a.get_alpha_from_calc(z['freqs'], g[C['T'], L], g[C['P'], L], g[:, L], C, cl[:, L], CL)
        ref = z['runA_alpha'][L]
        errs = gas_errors(got[None], ref[None], ordered)
        for c, e in errs.items():
            assert e < (EXTRA_RTOL if c in ('co', 'clouds') else ALPHA_RTOL), (L, c, errs)
    engine.set_co_clouds(co=False)
