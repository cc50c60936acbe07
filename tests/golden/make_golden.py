"""Generate the golden fixtures in this folder by running the reference.

Run from the repository root with ``RADIOBEAR_REF`` naming the folder that
holds the reference's ``radiobear`` package (its source tree or an install):

    RADIOBEAR_REF=<path> python tests/golden/make_golden.py            # all fixtures
    RADIOBEAR_REF=<path> python tests/golden/make_golden.py bench c0   # a subset

Fixtures (all float64, ``numpy.savez_compressed``):

``catalogs_real.npz``
    The real catalogues as the reference's loaders prepare them (default
    Jupiter truncation): ``ammonia.npz``, ``nh3.npz``, ``h2s.npz`` (121
    lines), ``ph3jh.npz`` + ``PH3WGT.npz`` (33 lines) and the 15 built-in
    ``h2o_bk`` lines.  Keys are ``<catalogue>__<column>``.
``benchmark.npz``
    ``scripts/benchmark.py``: Jupiter, ``Jupiter/config_benchmark.par``,
    6 freqs x 4 equatorial rays.  Holds the regridded atmosphere the
    reference built (gas + R, N), its alpha layers and per-gas alpha, the
    float64 Tb it computed, the float32 expected table ``T_rb`` quoted in
    ``scripts/benchmark.py:20-24`` and the ray paths.
``c0.npz``
    Configuration 0 (synthetic, 200 layers, 21 freqs, 200 NH3 lines): inputs,
    per-gas alpha for every layer, Tb for b=[0,0] and for 'disc', ray paths
    for nadir, off-nadir, oblique and limb rays (tangent/egress restored by
    the sqrt patch), with orientation (0,0) and (10,25) deg.
``c1_alpha.npz``
    Configuration 1 line lists (2000 NH3, 500 H2O, 200 H2S, 33 PH3) and
    256 freqs: per-gas alpha for 40 layers including the 400-500 bar
    nh3_hs/nh3_sjs blend layers.
``c1_tb.npz``
    Configuration 1: Tb of 6 Gauss-Legendre rays (incl. the two outermost)
    from the reference's full 1000-layer alpha.
``scale_cases.npz``
    ``Alpha.get_layers`` with number, list and dict scales on the C0
    atmosphere, plus the ``save_alpha='memory'`` cube.
``f2.npz``
    The formalisms beside the Jupiter set: nh3_dbs, nh3_dbs_sjs, co_ddb
    (every coshape) and clouds_idp (every particle kind), through the
    reference's ``Alpha.get_alpha_from_calc`` per layer (its own
    other_dict / cloud dispatch) and direct module calls, on a 48-layer
    synthetic atmosphere from 1e-4 to 2500 bar with CO and a cloud table,
    the C0 NH3 line lists and the real CO lines.
``f3.npz``
    ``AtmosphereBase.computeProp`` and ``regrid.regrid`` (interpolation
    inside the table, inward dry-adiabat and outward slope extrapolation)
    on an 80-layer synthetic gas + cloud table.
``f4.npz``
    ``set_utils.set_b`` b lists (float grids with image blocks, a stamp,
    line requests with and without an angle) and the text files
    ``fileIO.FileIO.write`` produces for image, spectrum, profile and disc
    data (frequency and wavelength axes).
"""
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import refharness as rh  # noqa: E402
from radiobear_gb300 import synth  # noqa: E402

GAS_KEEP = ['Z', 'T', 'P', 'H2', 'HE', 'CH4', 'NH3', 'H2O', 'H2S', 'PH3']


def _flatten(prefix, d):
    return {'{}__{}'.format(prefix, k): np.asarray(v, dtype=np.float64) for k, v in d.items()}


def real_catalogues():
    path = os.path.join(HERE, 'catalogs_real.npz')
    if os.path.exists(path):
        z = np.load(path)
        out = {}
        for k in z.files:
            cat, col = k.split('__', 1)
            out.setdefault(cat, {})[col] = z[k]
        return out
    cats = rh.load_real_catalogues()
    flat = {}
    for cat, d in cats.items():
        flat.update(_flatten(cat, d))
    np.savez_compressed(path, **flat)
    print('wrote', path, {c: len(next(iter(d.values()))) for c, d in cats.items()})
    return cats


def _ray_record(ray):
    if ray.ds is None:
        return np.zeros(0), np.zeros(0, dtype=np.int64), np.zeros(0)
    return (np.asarray(ray.ds, dtype=np.float64), np.asarray(ray.layer4ds, dtype=np.int64),
            np.asarray(ray.r4ds, dtype=np.float64))


def _gas_arrays(atm):
    C = atm.config.C
    return {('gas_' + k): np.asarray(atm.gas[C[k]], dtype=np.float64) for k in GAS_KEEP}


def _prop_arrays(atm):
    LP = atm.config.LP
    return {'prop_R': np.asarray(atm.property[LP['R']]), 'prop_N': np.asarray(atm.property[LP['N']])}


def golden_benchmark():
    rh.import_reference()
    rh.reset_lines()
    rh.patch_limb_sqrt(False)
    import radiobear.raypath as rp
    work = tempfile.mkdtemp(prefix='rbgold_bench_')
    rh.benchmark_planet_dir(work)
    cwd = os.getcwd()
    os.chdir(work)
    try:
        j = rh.make_planet('config_benchmark.par')
        freqs = [0.6, 1.25, 2.6, 5.2, 10, 21.9]
        b = [[0.0, 0.0], [np.sin(np.radians(15)), 0.0], [np.sin(np.radians(30)), 0.0],
             [np.sin(np.radians(45)), 0.0]]
        rv = j.run(freqs, b=b, reuse_override='False', save_alpha='memory')
        atm = j.atmos[0]
        out = dict(freqs=np.array(freqs, dtype=np.float64), b=np.array(b),
                   Tb=np.array(j.Tb, dtype=np.float64), Tb_f32=np.asarray(rv.Tb),
                   alpha_layers=np.asarray(j.alpha[0].layers),
                   alpha_gas=np.asarray(j.alpha[0].memory.alpha_data),
                   Req=j.config.Req, Rpol=j.config.Rpol)
        out.update(_gas_arrays(atm))
        out.update(_prop_arrays(atm))
        out['T_rb'] = np.array(
            [[805.38385, 424.58337, 298.74915, 227.0338, 179.9148, 147.3627],
             [790.66736, 420.24728, 296.62033, 225.69223, 179.22531, 147.24104],
             [745.55975, 407.28714, 290.07492, 221.56863, 177.13437, 146.8625],
             [668.4528, 385.59015, 278.51672, 214.30847, 173.56506, 146.17966]], dtype=np.float32)
        for i, bv in enumerate(b):
            ds, lay, r4 = _ray_record(rp.compute_ds(atm, bv))
            out['ray{}_ds'.format(i)] = ds
            out['ray{}_layer'.format(i)] = lay
        out['ordered_constituents'] = np.array(j.alpha[0].ordered_constituents)
    finally:
        os.chdir(cwd)
    dev = np.max(np.abs(out['Tb'].astype(np.float32) - out['T_rb']))
    print('benchmark: max |Tb(f32) - T_rb| =', dev)
    assert dev <= 1e-3, dev
    path = os.path.join(HERE, 'benchmark.npz')
    np.savez_compressed(path, **out)
    print('wrote', path)


def _synth_planet(work, wl, orientation=(0.0, 0.0), name='config_synth.par'):
    rh.scratch_planet_dir(work, wl.gas, synth.GAS_COLUMNS, config_name=name,
                          orientation=orientation)
    return rh.make_planet(name)


C0_RAYS = [[0.0, 0.0], [0.3, 0.0], [0.7, 0.0], [0.95, 0.0], [0.0, 0.5], [0.4, 0.4],
           [0.997, 0.0], [0.9985, 0.0], [0.99, 0.05], [0.0, 0.92], [0.5, -0.6], [1.2, 0.0]]


def golden_c0():
    cats = real_catalogues()
    rh.import_reference()
    import radiobear.raypath as rp
    wl = synth.make_workload(0, real=cats)
    rh.reset_lines()
    lines = dict(wl.lines)
    lines['ph3wgt'] = cats['ph3wgt']
    work = tempfile.mkdtemp(prefix='rbgold_c0_')
    cwd = os.getcwd()
    os.chdir(work)
    out = {}
    try:
        j = _synth_planet(work, wl)
        rh.inject_lines(lines)
        rh.patch_limb_sqrt(False)
        freqs = '1:100:5'
        j.run(freqs, b=[0.0, 0.0], reuse_override='False', save_alpha='memory')
        out['Tb_nadir'] = np.array(j.Tb[0], dtype=np.float64)
        out['alpha_layers'] = np.asarray(j.alpha[0].layers)
        out['alpha_gas'] = np.asarray(j.alpha[0].memory.alpha_data)
        out['freqs'] = np.asarray(j.freqs, dtype=np.float64)
        j.run(freqs, b='disc', reuse_override='False')
        out['Tb_disc'] = np.array(j.Tb[0], dtype=np.float64)
        bri = j.bright
        out['disc_tau'] = np.asarray(bri.tau)
        out['disc_W'] = np.asarray(bri.W)
        out['disc_intW'] = np.asarray(bri.integrated_W)
        atm = j.atmos[0]
        out.update(_gas_arrays(atm))
        out.update(_prop_arrays(atm))
        # rays: unpatched for on-disc, patched (tangent branch restored) for all
        rh.patch_limb_sqrt(True)
        tbs = []
        for i, bv in enumerate(C0_RAYS):
            ds, lay, r4 = _ray_record(rp.compute_ds(atm, bv))
            out['ray{}_ds'.format(i)] = ds
            out['ray{}_layer'.format(i)] = lay
            out['ray{}_r4ds'.format(i)] = r4
            tb = j.bright.single(bv, out['freqs'].tolist(), atm, j.alpha[0], j.config.orientation)
            tbs.append(np.array(tb, dtype=np.float64))
        out['Tb_rays'] = np.array(tbs)
        out['rays_b'] = np.array(C0_RAYS)
        rh.patch_limb_sqrt(False)
    finally:
        os.chdir(cwd)
    # tilted planet: orientation (10, 25) deg
    work2 = tempfile.mkdtemp(prefix='rbgold_c0o_')
    os.chdir(work2)
    try:
        j2 = _synth_planet(work2, wl, orientation=(10.0, 25.0), name='config_tilt.par')
        rh.inject_lines(lines)
        rh.patch_limb_sqrt(True)
        atm2 = j2.atmos[0]
        j2.alpha[0].get_layers(out['freqs'].tolist(), atm2)
        tilt_rays = [[0.0, 0.0], [0.3, 0.2], [-0.5, 0.6], [0.9, -0.3], [0.999, 0.0]]
        tbs = []
        for i, bv in enumerate(tilt_rays):
            ds, lay, r4 = _ray_record(rp.compute_ds(atm2, bv))
            out['tilt{}_ds'.format(i)] = ds
            out['tilt{}_layer'.format(i)] = lay
            tb = j2.bright.single(bv, out['freqs'].tolist(), atm2, j2.alpha[0], j2.config.orientation)
            tbs.append(np.array(tb, dtype=np.float64))
        out['tilt_Tb'] = np.array(tbs)
        out['tilt_b'] = np.array(tilt_rays)
        out['tilt_orientation'] = np.array([10.0, 25.0])
        rh.patch_limb_sqrt(False)
    finally:
        os.chdir(cwd)
    # synthetic inputs, so the fixture is self-contained
    for k, v in wl.lines['ammonia'].items():
        out['ammonia__' + k] = v
    for k, v in wl.lines['nh3'].items():
        out['nh3__' + k] = v
    out['ordered_constituents'] = np.array(j.alpha[0].ordered_constituents)
    path = os.path.join(HERE, 'c0.npz')
    np.savez_compressed(path, **out)
    print('wrote', path)


C1_LAYERS = None


def c1_layer_subset(P):
    idx = set(np.linspace(0, len(P) - 1, 24).astype(int).tolist())
    idx.update(np.nonzero(P >= 380.0)[0].tolist())
    return np.array(sorted(idx))


def golden_c1_alpha():
    cats = real_catalogues()
    rh.import_reference()
    wl = synth.make_workload(1, real=cats)
    rh.reset_lines()
    lines = dict(wl.lines)
    lines['ph3wgt'] = cats['ph3wgt']
    work = tempfile.mkdtemp(prefix='rbgold_c1_')
    cwd = os.getcwd()
    os.chdir(work)
    try:
        j = _synth_planet(work, wl)
        rh.inject_lines(lines)
        atm = j.atmos[0]
        C = atm.config.C
        P = atm.gas[C['P']]
        sel = c1_layer_subset(P)
        freqs = wl.freqs.tolist()
        t0 = time.time()
        per = []
        for layer in sel:
            a = j.alpha[0].get_alpha_from_calc(freqs, atm.gas[C['T']][layer], P[layer],
                                               atm.gas[:, layer], C, atm.cloud[:, layer],
                                               atm.config.Cl, units='invcm')
            per.append(np.asarray(a, dtype=np.float64))
        print('c1 alpha subset: {} layers in {:.1f} s'.format(len(sel), time.time() - t0))
        out = dict(layers=sel, alpha_gas=np.array(per), freqs=wl.freqs,
                   ordered_constituents=np.array(j.alpha[0].ordered_constituents))
        out.update(_gas_arrays(atm))
    finally:
        os.chdir(cwd)
    path = os.path.join(HERE, 'c1_alpha.npz')
    np.savez_compressed(path, **out)
    print('wrote', path)


def golden_c1_tb():
    cats = real_catalogues()
    rh.import_reference()
    wl = synth.make_workload(1, real=cats)
    rh.reset_lines()
    lines = dict(wl.lines)
    lines['ph3wgt'] = cats['ph3wgt']
    work = tempfile.mkdtemp(prefix='rbgold_c1tb_')
    cwd = os.getcwd()
    os.chdir(work)
    try:
        j = _synth_planet(work, wl)
        rh.inject_lines(lines)
        rh.patch_limb_sqrt(True)
        atm = j.atmos[0]
        t0 = time.time()
        j.alpha[0].get_layers(wl.freqs.tolist(), atm)
        print('c1 full alpha: {:.1f} s'.format(time.time() - t0))
        ray_idx = np.array([0, 1, 2, 20, 40, 63])
        tbs = []
        for k in ray_idx:
            tb = j.bright.single(wl.b[k].tolist(), wl.freqs.tolist(), atm, j.alpha[0],
                                 j.config.orientation)
            tbs.append(np.array(tb, dtype=np.float64))
        rh.patch_limb_sqrt(False)
        out = dict(ray_idx=ray_idx, b=wl.b[ray_idx], Tb=np.array(tbs), freqs=wl.freqs)
        out.update(_gas_arrays(atm))
        out.update(_prop_arrays(atm))
    finally:
        os.chdir(cwd)
    path = os.path.join(HERE, 'c1_tb.npz')
    np.savez_compressed(path, **out)
    print('wrote', path)


def golden_scale_cases():
    cats = real_catalogues()
    rh.import_reference()
    wl = synth.make_workload(0, real=cats)
    rh.reset_lines()
    lines = dict(wl.lines)
    lines['ph3wgt'] = cats['ph3wgt']
    work = tempfile.mkdtemp(prefix='rbgold_scale_')
    cwd = os.getcwd()
    os.chdir(work)
    try:
        j = _synth_planet(work, wl)
        rh.inject_lines(lines)
        atm = j.atmos[0]
        nL = atm.gas.shape[1]
        P = atm.gas[atm.config.C['P']]
        freqs = [1.0, 5.0, 22.0, 31.0, 60.0]
        al = j.alpha[0]
        out = dict(freqs=np.array(freqs))
        al.get_layers(freqs, atm, scale=False, save_alpha='memory')
        out['plain'] = np.asarray(al.layers)
        out['saved'] = np.asarray(al.memory.alpha_data)
        al.get_layers(freqs, atm, scale=0.5)
        out['number'] = np.asarray(al.layers)
        ramp = (2.0 * (P[-1] - P / 1.5) / P[-1])
        al.get_layers(freqs, atm, scale=ramp.tolist())
        out['list'] = np.asarray(al.layers)
        out['list_scale'] = ramp
        dscale = {'nh3': np.where(P > 1.0, 0.25, 2.0).tolist(),
                  'h2o': np.where(P > 10.0, 0.5, 1.0e-4).tolist()}
        al.get_layers(freqs, atm, scale=dscale)
        out['dict'] = np.asarray(al.layers)
        out['dict_nh3'] = np.array(dscale['nh3'])
        out['dict_h2o'] = np.array(dscale['h2o'])
        # reuse of the saved cube with a dict scale (scripts/demo_batch.py path)
        al.get_layers(freqs, atm, scale=False, save_alpha='memory')
        al.get_layers(freqs, atm, scale=dscale, get_alpha='memory')
        out['dict_from_memory'] = np.asarray(al.layers)
        # unsorted frequencies straddling 30 GHz (nh3_hs output ordering)
        fun = [40.0, 10.0, 22.2, 35.0, 2.0]
        al.get_layers(fun, atm)
        out['unsorted_freqs'] = np.array(fun)
        out['unsorted'] = np.asarray(al.layers)
        assert out['plain'].shape == (len(freqs), nL)
    finally:
        os.chdir(cwd)
    path = os.path.join(HERE, 'scale_cases.npz')
    np.savez_compressed(path, **out)
    print('wrote', path)


F2_FREQS = [0.05, 0.6, 1.4, 5.0, 12.0, 22.2, 24.0, 29.9, 30.1, 33.0, 44.0, 60.0, 115.0,
            115.271, 150.0, 230.0]


def f2_atmosphere(nL=48):
    """Gas and cloud tables of the f2 fixture (CO 1e-6; cloud decks of every
    kind, ice / liquid water on either side of 273 K)."""
    gas = synth.make_gas_table(nL, 1.0e-4, 2500.0)
    C = {k: i for i, k in enumerate(synth.GAS_COLUMNS)}
    gas[C['CO']] = 1.0e-6
    Cl = {k: i for i, k in enumerate(synth.CLOUD_COLUMNS)}
    cloud = np.zeros((len(synth.CLOUD_COLUMNS), nL))
    for k in ('Z', 'T', 'P'):
        cloud[Cl[k]] = gas[C[k]]
    T, P = gas[C['T']], gas[C['P']]
    rng = np.random.default_rng(21)
    dens = 10.0 ** rng.uniform(-6.0, -3.0, nL)
    cloud[Cl['H2O']] = np.where((T < 273.0) & (P > 1.0), dens, 0.0)
    cloud[Cl['SOLN']] = np.where(T >= 250.0, dens[::-1], 0.0)
    cloud[Cl['NH4SH']] = np.where((P > 1.0) & (P < 30.0), 0.3 * dens, 0.0)
    cloud[Cl['NH3']] = np.where((P > 0.3) & (P < 3.0), 2.0 * dens, 0.0)
    cloud[Cl['H2S']] = np.where((P > 0.1) & (P < 10.0), 0.5 * dens, 0.0)
    cloud[Cl['CH4']] = np.where(P < 1.0, 0.1 * dens, 0.0)
    return gas, C, cloud, Cl


def golden_f2():
    cats = real_catalogues()
    rh.import_reference()
    rh.reset_lines()
    import importlib
    from argparse import Namespace
    import radiobear.alpha as ralpha
    z = np.load(os.path.join(HERE, 'c0.npz'))
    amm = {k[len('ammonia__'):]: z[k] for k in z.files if k.startswith('ammonia__')}
    nh3 = {k[len('nh3__'):]: z[k] for k in z.files if k.startswith('nh3__')}
    lines = dict(ammonia=amm, nh3=nh3, h2o=cats['h2o'], h2s=cats['h2s'], ph3=cats['ph3'],
                 ph3wgt=cats['ph3wgt'])
    rh.inject_lines(lines)
    dbs = importlib.import_module('radiobear.constituents.nh3.nh3_dbs')
    dbs.data = {k: np.asarray(v, dtype=np.float64) for k, v in amm.items()}
    gas, C, cloud, Cl = f2_atmosphere()
    nL = gas.shape[1]
    freqs = list(F2_FREQS)
    work = tempfile.mkdtemp(prefix='rbgold_f2_')
    out = dict(freqs=np.array(freqs), gas=gas, cloud=cloud)
    full = {'nh3': 'nh3_dbs_sjs', 'co': 'co_ddb', 'clouds': 'clouds_idp', 'h2': 'h2_jj_ddb',
            'h2o': 'h2o_bk', 'h2s': 'h2s_ddb', 'ph3': 'ph3_jh'}
    runs = dict(
        A=(full, dict(coshape='voigt', water_p=1.0e-4, ice_p=1.0e-4, nh4sh_p=1.0e-4,
                      nh3ice_p=1.0e-4, h2sice_p=1.0e-4, ch4_p=1.0e-4)),
        B=({'nh3': 'nh3_dbs', 'co': 'co_ddb', 'clouds': 'clouds_idp'},
           dict(coshape='std', water_p=1.0e-4, ice_p=1.0e-4, nh4sh_p=0.0, nh3ice_p=0.0,
                h2sice_p=0.0, ch4_p=0.0)))
    for name, (ca, other) in runs.items():
        cfg = Namespace(constituent_alpha=ca, truncate_method={}, scratch_directory=work,
                        h2state='e', h2newset=False, **other)
        al = ralpha.Alpha(config=cfg, verbose=False)
        if 'nh3_dbs' in sys.modules:      # the bare module the dispatcher imported for 'nh3_dbs'
            sys.modules['nh3_dbs'].data = dbs.data
        per = np.zeros((nL, len(freqs), len(al.ordered_constituents)))
        for L in range(nL):
            per[L] = al.get_alpha_from_calc(freqs, gas[C['T']][L], gas[C['P']][L], gas[:, L], C,
                                            cloud[:, L], Cl, units='invcm')
        out['run{}_alpha'.format(name)] = per
        out['run{}_ordered'.format(name)] = np.array(al.ordered_constituents)
        for k, v in other.items():
            out['run{}_{}'.format(name, k)] = np.array(v)
    co = sys.modules['co_ddb']
    for shape in ('vvw', 'diff'):
        a = np.zeros((nL, len(freqs)))
        for L in range(nL):
            a[L] = co.alpha(freqs, gas[C['T']][L], gas[C['P']][L], gas[:, L], C,
                            {'coshape': shape}, units='invcm', path=rh.constituents_dir('co'),
                            verbose=False)
        out['co_' + shape] = a
    cl = sys.modules['clouds_idp']
    a = np.zeros((nL, len(freqs)))
    for L in range(nL):
        a[L] = cl.alpha(freqs, gas[C['T']][L], gas[C['P']][L], cloud[:, L], Cl, {'ch4': 1.0},
                        units='invcm', verbose=False)
    out['clouds_ch4key'] = a
    for k, v in co.data.items():
        out['co__' + k] = np.asarray(v, dtype=np.float64)
    path = os.path.join(HERE, 'f2.npz')
    np.savez_compressed(path, **out)
    print('wrote', path)


class _GridSpacing(float):
    """A float grid request whose len() is 1: lets the reference's set_b
    return its b list (its own imSize line takes len() of the float and
    raises TypeError, set_utils.py:78)."""

    def __len__(self):
        return 1


F4_SETB = dict(grid_a=(0.1, [1, 1]), grid_b=(0.1, [2, 4]), grid_c=(0.05, [3, 3]),
               grid_d=(0.25, [1, 1]))
F4_STRINGS = dict(stamp='stamp:0.1:-0.2,0.2,-0.3,0.3', line_angle='0:1.2:0.1<30',
                  line_csv='0.1,0.5,0.9,0.999', line_flat='0:1:0.25', disc='disc')


def golden_f4():
    """set_b requests and the FileIO text formats from the reference."""
    rh.import_reference()
    from argparse import Namespace
    from radiobear import set_utils, fileIO
    out = {}
    for name, (spacing, block) in F4_SETB.items():
        rv = set_utils.set_b(_GridSpacing(spacing), block)
        out['setb_' + name] = np.asarray(rv.b, dtype=np.float64)
    for name, req in F4_STRINGS.items():
        rv = set_utils.set_b(req, [1, 1], Rpol=66854.0, Req=71492.0)
        out['setb_' + name] = np.asarray(rv.b if name != 'disc' else [[0.0, 0.0]], dtype=np.float64)
        out['setb_' + name + '_type'] = np.array(rv.data_type)
    rng = np.random.default_rng(44)
    work = tempfile.mkdtemp(prefix='rbgold_f4_')
    cwd = os.getcwd()
    os.chdir(work)
    os.makedirs('Scratch', exist_ok=True)
    try:
        hdr = {'b': '# b request:  0.25  [1, 1]', 'freqs': '# freqs request: 22.0 GHz'}
        cases = dict(
            image=Namespace(type='image', header=hdr, f=[22.0], freqUnit='GHz',
                            b=[[0.0, 0.0]] * 25, Tb=(100.0 + 200.0 * rng.random((5, 5))).tolist()),
            spectrum=Namespace(type='spectrum', header=hdr, f=[1.4, 5.0, 22.0], freqUnit='GHz',
                               b=[[0.0, 0.0], [0.25, 0.1]],
                               Tb=(100.0 + 300.0 * rng.random((2, 3))).tolist()),
            profile=Namespace(type='profile', header=hdr, f=[1.4, 22.0], freqUnit='GHz',
                              b=[[0.1 * i, 0.0] for i in range(12)],
                              Tb=(100.0 + 300.0 * rng.random((12, 2))).tolist()),
            disc=Namespace(type='spectrum', header=hdr, f=[1.4, 5.0], freqUnit='GHz', b=['disc'],
                           Tb=(100.0 + 300.0 * rng.random((1, 2))).tolist()))
        for name, data in cases.items():
            for xaxis in ('frequency', 'wavelength'):
                if name == 'image' and xaxis == 'wavelength':
                    continue
                path = os.path.join(work, '{}_{}.dat'.format(name, xaxis))
                fileIO.FileIO().write(path, data, xaxis=xaxis)
                with open(path) as fp:
                    out['file_{}_{}'.format(name, xaxis)] = np.array(fp.read())
            out['data_{}_Tb'.format(name)] = np.asarray(data.Tb, dtype=np.float64)
            out['data_{}_f'.format(name)] = np.asarray(data.f, dtype=np.float64)
    finally:
        os.chdir(cwd)
    path = os.path.join(HERE, 'f4.npz')
    np.savez_compressed(path, **out)
    print('wrote', path)


def f3_tables(nL=80, Pmin=1.0e-2, Pmax=300.0):
    """Gas and cloud tables of the f3 fixture (the C1 recipe, cloud decks)."""
    gas = synth.make_gas_table(nL, Pmin, Pmax)
    C = {k: i for i, k in enumerate(synth.GAS_COLUMNS)}
    gas[C['CO']] = 1.0e-7
    Cl = {k: i for i, k in enumerate(synth.CLOUD_COLUMNS)}
    cloud = np.zeros((len(synth.CLOUD_COLUMNS), nL))
    for k in ('Z', 'T', 'P'):
        cloud[Cl[k]] = gas[C[k]]
    P = gas[C['P']]
    cloud[Cl['NH3']] = np.where((P > 0.4) & (P < 1.0), 2.0e-4, 0.0)
    cloud[Cl['H2O']] = np.where((P > 4.0) & (P < 8.0), 5.0e-4, 0.0)
    cloud[Cl['DZ']] = np.append(0.0, np.abs(np.diff(cloud[Cl['Z']])) * 1e5)
    return gas, C, cloud, Cl


def golden_f3():
    """AtmosphereBase.computeProp and regrid.regrid on synthetic tables,
    run through the reference's own functions bound to a minimal atmosphere
    object (gas, cloud, config)."""
    rh.import_reference()
    import types
    from argparse import Namespace
    import radiobear.regrid as rregrid
    from radiobear.atm_base import AtmosphereBase
    LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
    J = synth.JUPITER
    out = {}

    def make_atm(gas, C, cloud, Cl):
        atm = Namespace(gas=np.array(gas), cloud=np.array(cloud),
                        config=Namespace(C=C, Cl=Cl, LP=LP, p_ref=J['p_ref'], Req=J['Req'],
                                         GM_ref=J['GM_ref'], regridType='none', path='.'))
        atm.computeProp = types.MethodType(AtmosphereBase.computeProp, atm)
        atm._renorm_z = types.MethodType(AtmosphereBase._renorm_z, atm)
        return atm

    gas, C, cloud, Cl = f3_tables()
    out['gas_in'] = gas
    out['cloud_in'] = cloud
    atm = make_atm(gas, C, cloud, Cl)
    atm.computeProp()
    out['prop_in'] = np.asarray(atm.property, dtype=np.float64)
    cases = dict(inside=(200, 0, 0), extend=(250, 3.0e-3, 1000.0), deeper=(120, 1.0e-2, 2000.0))
    for name, (n, pmin, pmax) in cases.items():
        atm = make_atm(gas, C, cloud, Cl)
        rregrid.regrid(atm, regridType=n, Pmin=pmin or None, Pmax=pmax or None)
        out['gas_' + name] = np.asarray(atm.gas, dtype=np.float64)
        out['cloud_' + name] = np.asarray(atm.cloud, dtype=np.float64)
        atm.computeProp()
        out['prop_' + name] = np.asarray(atm.property, dtype=np.float64)
        out['case_' + name] = np.array([n, pmin, pmax], dtype=np.float64)
    path = os.path.join(HERE, 'f3.npz')
    np.savez_compressed(path, **out)
    print('wrote', path)


JOBS = dict(cats=real_catalogues, bench=golden_benchmark, c0=golden_c0,
            c1a=golden_c1_alpha, c1tb=golden_c1_tb, scale=golden_scale_cases, f2=golden_f2,
            f3=golden_f3, f4=golden_f4)

if __name__ == '__main__':
    which = sys.argv[1:] or list(JOBS)
    for name in which:
        t0 = time.time()
        JOBS[name]()
        print('[{}] {:.1f} s'.format(name, time.time() - t0))
