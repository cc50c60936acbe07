"""Harness that drives the unmodified radioBEAR reference in this container.

Used by ``make_golden.py`` to produce the committed golden fixtures, and by
``tests/ref_planet_run.py`` / the bench's stock-reference figure to run an
installed copy of the reference.  The reference tree is named by the
``RADIOBEAR_REF`` environment variable (or ``set_reference``): the folder
that holds the ``radiobear`` package.  The package itself never imports
this file.

What it does to run the reference (none of it edits reference files):

* stubs ``matplotlib`` (imported by ``radiobear/atm_modify.py:8`` on the
  ``Atmosphere.std`` path) because matplotlib is not installed;
* runs in a scratch working directory holding a ``Jupiter/`` folder, since
  the reference resolves ``<Planet>/config.par`` relative to the cwd
  (``radiobear/planet_base.py:52``, ``radiobear/config.py:76``);
* injects line lists by setting the module-global ``data`` of the formalism
  module objects the dispatcher actually calls (bare names for
  ``h2o_bk``/``h2s_ddb``/``ph3_jh``, ``alpha.py:63-67``; package paths for
  ``nh3_hs``/``nh3_sjs``, ``nh3_hs_sjs.py:1-2``);
* optionally patches ``radiobear.raypath.np.sqrt`` to raise ``ValueError`` on
  negative scalars, which restores the tangent / egress branch of
  ``compute_ds`` (``raypath.py:191-209``); unpatched, numpy returns NaN there.
"""
import os
import shutil
import sys
import types

import numpy as np

REF = os.environ.get('RADIOBEAR_REF')


def set_reference(path):
    """Use the reference tree at ``path`` (the folder holding ``radiobear``)."""
    global REF
    REF = path


def _ref():
    if not REF:
        raise RuntimeError('set RADIOBEAR_REF to the folder that holds the radiobear package')
    return REF


def _stub_matplotlib():
    if 'matplotlib' in sys.modules:
        return
    mpl = types.ModuleType('matplotlib')
    plt = types.ModuleType('matplotlib.pyplot')
    cm = types.ModuleType('matplotlib.cm')
    mpl.pyplot = plt
    mpl.cm = cm
    mpl.use = lambda *a, **k: None
    sys.modules['matplotlib'] = mpl
    sys.modules['matplotlib.pyplot'] = plt
    sys.modules['matplotlib.cm'] = cm


def import_reference():
    _stub_matplotlib()
    if _ref() not in sys.path:
        sys.path.insert(0, _ref())
    import radiobear  # noqa: F401
    import radiobear.planet  # noqa: F401
    import radiobear.raypath  # noqa: F401
    import radiobear.alpha  # noqa: F401
    return sys.modules['radiobear']


class _SqrtRaises:
    """Proxy for ``numpy`` whose ``sqrt`` raises on a negative scalar."""

    def __init__(self, np_mod):
        self._np = np_mod

    def __getattr__(self, name):
        return getattr(self._np, name)

    def sqrt(self, x):
        if np.ndim(x) == 0 and x < 0.0:
            raise ValueError('math domain error')
        return self._np.sqrt(x)


def patch_limb_sqrt(enable=True):
    import radiobear.raypath as rp
    rp.np = _SqrtRaises(np) if enable else np


def constituents_dir(c):
    return os.path.join(_ref(), 'radiobear', 'constituents', c)


def load_real_catalogues():
    """Real catalogues as the reference's own loaders prepare them with the
    default Jupiter truncation (h2s/ph3 strength > 1e-22)."""
    from argparse import Namespace
    import_reference()
    out = {}
    am = np.load(os.path.join(constituents_dir('nh3'), 'ammonia.npz'))
    out['ammonia'] = {k: np.array(am[k]) for k in am.files}
    n3 = np.load(os.path.join(constituents_dir('nh3'), 'nh3.npz'))
    out['nh3'] = {k: np.array(n3[k]) for k in n3.files}
    for c, mod in (('h2s', 'h2s_ddb'), ('ph3', 'ph3_jh'), ('h2o', 'h2o_bk')):
        if constituents_dir(c) not in sys.path:
            sys.path.append(constituents_dir(c))
        m = __import__(mod)
        trunc = 1.0e-22 if c in ('h2s', 'ph3') else None
        par = Namespace(path=constituents_dir(c), verbose=False,
                        truncate_strength=trunc, truncate_freq=None, units='invcm')
        m.data = None
        m.readInputFiles(par)
        out[c] = {k: np.array(v) for k, v in m.data.items()}
        if c == 'ph3':
            out['ph3wgt'] = {k: np.array(v) for k, v in m.data_wgt.items()}
        m.data = None
    return out


def inject_lines(lines):
    """Point every formalism the dispatcher uses at the given line lists."""
    import_reference()
    import importlib
    for c, mod in (('h2s', 'h2s_ddb'), ('ph3', 'ph3_jh'), ('h2o', 'h2o_bk')):
        if constituents_dir(c) not in sys.path:
            sys.path.append(constituents_dir(c))
        importlib.import_module(mod)
    hs = importlib.import_module('radiobear.constituents.nh3.nh3_hs')
    sjs = importlib.import_module('radiobear.constituents.nh3.nh3_sjs')
    if 'ammonia' in lines:
        hs.data = {k: np.asarray(v, dtype=np.float64) for k, v in lines['ammonia'].items()}
    if 'nh3' in lines:
        sjs.data = {k: np.asarray(v, dtype=np.float64) for k, v in lines['nh3'].items()}
    if 'h2o' in lines:
        sys.modules['h2o_bk'].data = {k: np.asarray(v, dtype=np.float64) for k, v in lines['h2o'].items()}
    if 'h2s' in lines:
        sys.modules['h2s_ddb'].data = {k: np.asarray(v, dtype=np.float64) for k, v in lines['h2s'].items()}
    if 'ph3' in lines:
        m = sys.modules['ph3_jh']
        m.data = {k: np.asarray(v, dtype=np.float64) for k, v in lines['ph3'].items()}
        m.data_wgt.clear()
        m.data_wgt.update({k: np.asarray(v, dtype=np.float64) for k, v in lines['ph3wgt'].items()})


def reset_lines():
    """Drop injected/cached catalogues so the next call reloads from disk."""
    import importlib
    for name in ('radiobear.constituents.nh3.nh3_hs', 'radiobear.constituents.nh3.nh3_sjs',
                 'h2o_bk', 'h2s_ddb', 'ph3_jh'):
        if name in sys.modules:
            sys.modules[name].data = None
    if 'ph3_jh' in sys.modules:
        sys.modules['ph3_jh'].data_wgt.clear()
    importlib.invalidate_caches()


CONFIG_TEMPLATE = """gasfile {gas}
constituents Z T P H2 HE CH4 NH3 H2O H2S SOLN OTHER PH3 CO CO13 HCN DZ
cloudfile {cloud}
clouds Z T P SOLN H2O NH4SH NH3 H2S CH4 AR PH3 DZ
tweakmodule NoTweakSynth
regridtype none
alpha nh3:nh3_hs_sjs h2s:h2s_ddb h2o:h2o_bk ph3:ph3_jh h2:h2_jj_ddb cloud:none
truncate_method h2s:none ph3:none
h2state e
distance 5.2 AU
orientation {orient0} {orient1}
gtype    {gtype}
limb     {limb}
doppler 0
"""

NO_TWEAK = '''def modify(gas, cloud, C, Cl):
    return "no tweak", gas, cloud
'''


def scratch_planet_dir(workdir, gas_table, gas_columns, config_name='config_synth.par',
                       orientation=(0.0, 0.0), gtype='ellipse', limb='shape'):
    """Write a Jupiter/ folder (gas + empty cloud file + config + no-op tweak)."""
    jdir = os.path.join(workdir, 'Jupiter')
    os.makedirs(jdir, exist_ok=True)
    with open(os.path.join(jdir, 'synth.gas'), 'w') as fp:
        fp.write('# synthetic gas table: ' + ' '.join(gas_columns[:-1]) + '\n')
        for i in range(gas_table.shape[1]):
            fp.write(' '.join(repr(float(gas_table[k, i])) for k in range(len(gas_columns) - 1)))
            fp.write('\n')
    with open(os.path.join(jdir, 'synth.cloud'), 'w') as fp:
        fp.write('# empty clouds\n')
        for i in range(gas_table.shape[1]):
            z, T, P = gas_table[0, i], gas_table[1, i], gas_table[2, i]
            fp.write('{} {} {} 0 0 0 0 0 0 0 0\n'.format(repr(float(z)), repr(float(T)), repr(float(P))))
    with open(os.path.join(jdir, 'NoTweakSynth.py'), 'w') as fp:
        fp.write(NO_TWEAK)
    with open(os.path.join(jdir, config_name), 'w') as fp:
        fp.write(CONFIG_TEMPLATE.format(gas='synth.gas', cloud='synth.cloud',
                                        orient0=orientation[0], orient1=orientation[1],
                                        gtype=gtype, limb=limb))
    zonal_src = os.path.join(_ref(), 'radiobear', 'Jupiter', 'zonalJupiter.dat')
    shutil.copy(zonal_src, os.path.join(jdir, 'zonalJupiter.dat'))
    return jdir


def benchmark_planet_dir(workdir):
    """Copy the reference's benchmark inputs into workdir/Jupiter."""
    jdir = os.path.join(workdir, 'Jupiter')
    os.makedirs(jdir, exist_ok=True)
    src = os.path.join(_ref(), 'radiobear', 'Jupiter')
    for f in ('config_benchmark.par', 'jupiter.benchmark_gas', 'jupiter.benchmark_nocloud',
              'JupiterNoTweak.py', 'zonalJupiter.dat'):
        shutil.copy(os.path.join(src, f), os.path.join(jdir, f))
    return jdir


def make_planet(config_file, **kw):
    import radiobear.planet as rbp
    return rbp.Planet('jupiter', config_file=config_file, plot_atm=False, plot_bright=False,
                      verbose=False, **kw)


# ------------------------------------------------------------ stock timing
# Workers of a spawn pool that time the unmodified reference's own hot-path
# calls on the synthetic C1 workload (1000 layers, 256 freqs, 64 disc rays):
# Alpha.get_alpha_from_calc per layer (the call Alpha.get_layers loops
# over, alpha.py:261-305) and Brightness.single per ray (the call of
# Planet.run's b loop, planet_base.py:268).  Each worker builds its own
# Planet in a scratch folder once (untimed).
_STOCK = {}


def stock_init(ref, root):
    import tempfile
    if root not in sys.path:
        sys.path.insert(0, root)
    os.environ['OMP_NUM_THREADS'] = '1'
    set_reference(ref)
    import_reference()
    from radiobear_gb300 import synth
    from tests import goldio
    cats = goldio.real_catalogues()
    wl = synth.make_workload(1, real=cats)
    lines = dict(wl.lines)
    lines['ph3wgt'] = cats['ph3wgt']
    work = tempfile.mkdtemp(prefix='rbstock_')
    os.chdir(work)
    scratch_planet_dir(work, wl.gas, synth.GAS_COLUMNS)
    reset_lines()
    j = make_planet('config_synth.par')
    inject_lines(lines)
    patch_limb_sqrt(True)
    atm = j.atmos[0]
    j.alpha[0].layers = np.full((len(wl.freqs), atm.gas.shape[1]), 1.0e-6)
    _STOCK.update(j=j, atm=atm, freqs=wl.freqs.tolist(), b=wl.b)


def stock_alpha_job(layers):
    import time
    j, atm, freqs = _STOCK['j'], _STOCK['atm'], _STOCK['freqs']
    C = atm.config.C
    t0 = time.perf_counter()
    for layer in layers:
        j.alpha[0].get_alpha_from_calc(freqs, atm.gas[C['T']][layer], atm.gas[C['P']][layer],
                                       atm.gas[:, layer], C, atm.cloud[:, layer], atm.config.Cl,
                                       units='invcm')
    return time.perf_counter() - t0


def stock_ray_job(k):
    import time
    j, atm = _STOCK['j'], _STOCK['atm']
    t0 = time.perf_counter()
    j.bright.single(_STOCK['b'][k].tolist(), _STOCK['freqs'], atm, j.alpha[0], j.config.orientation)
    return time.perf_counter() - t0
