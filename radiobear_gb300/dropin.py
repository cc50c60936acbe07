"""Drop-in replacements for radioBEAR's hot-path calls.

Same names, signatures, argument meaning, results and errors as

  * ``radiobear.alpha.Alpha`` -- ``get_layers``, ``get_alpha_from_calc``,
    ``get_single_layer``, ``total_layer_alpha``, ``get_layer_scale``,
    ``save_alpha_data`` / ``read_alpha_data`` (the ``Scratch/alphaNNNN.npz``
    cache: keys ``ordered_constituents``, ``alpha_data`` [nL, nf, nC],
    ``freqs``, ``P``) (alpha.py:13-305);
  * ``radiobear.raypath.compute_ds`` -> ``Ray`` (raypath.py:20-273);
  * ``radiobear.brightness.Brightness.single`` (brightness.py:30-126),

computed on the GPU through the C ABI (``_native.Engine``).  An ``atm``
argument is anything with the reference Atmosphere's attributes used on
this path: ``gas`` [nC, nL], ``config.C`` (gas row index by name),
``property`` with ``config.LP`` (rows ``R`` and ``N``), ``config.Req``,
``config.Rpol``, ``config.gtype``, ``config.orientation``.

``install()`` routes an importable ``radiobear`` package's own classes to
these implementations, and makes ``Planet.run``'s b loop one GPU call per
atmosphere (all rays' paths and scans together, the absorption uploaded
once).
"""
from __future__ import annotations

import os
from argparse import Namespace

import numpy as np

from . import _native, catalog

T_CMB = 2.725   # radiobear/utils.py:77

# Jupiter's default absorbers (radiobear default_config.json)
DEFAULT_CONSTITUENTS = {'nh3': 'nh3_hs_sjs', 'h2o': 'h2o_bk', 'h2s': 'h2s_ddb',
                        'ph3': 'ph3_jh', 'h2': 'h2_jj_ddb'}
_NH3_FORMALISMS = ('nh3_hs', 'nh3_sjs', 'nh3_hs_sjs', 'nh3_dbs', 'nh3_dbs_sjs')
_SUPPORTED = {'h2o': 'h2o_bk', 'h2s': 'h2s_ddb', 'ph3': 'ph3_jh', 'h2': 'h2_jj_ddb', 'co': 'co_ddb',
              'clouds': 'clouds_idp'}
# config attributes Alpha.setup_formalisms copies into other_dict (alpha.py:90-102)
_OTHER_TO_COPY = {'h2': ['h2state', 'h2newset'],
                  'clouds': ['water_p', 'ice_p', 'nh4sh_p', 'nh3ice_p', 'h2sice_p', 'ch4_p'],
                  'co': ['coshape']}
_GAS_SLOT = {g: i for i, g in enumerate(_native.GASES)}

_ENGINES = {}


def engine(device=0):
    """One shared Engine per device (catalogues and formalisms are set by
    the Alpha that uses it)."""
    if device not in _ENGINES:
        _ENGINES[device] = _native.Engine(device)
    return _ENGINES[device]


def _isanynum(v):
    """utils.isanynum (radiobear/utils.py:33-41): bools, dicts and lists are
    not numbers; anything float() accepts is; a ValueError means no (other
    errors propagate, as there)."""
    if isinstance(v, (bool, dict, list)):
        return False
    try:
        float(v)
    except ValueError:
        return False
    return True


def _cfg(config, name, default=None):
    return getattr(config, name, default) if config is not None else default


class Alpha:
    """Layer absorption (radiobear/alpha.py:13), on the GPU."""

    def __init__(self, idnum=0, config=None, log=None, load_formal=True, verbose=True,
                 engine_=None, lines=None, **kwargs):
        self.verbose = verbose
        self.log = log
        self.config = config
        self.idnum = idnum
        self.engine = engine_ or engine(0)
        self.lines = lines
        self.reset_layers()
        scratch = _cfg(config, 'scratch_directory', 'Scratch')
        self.alphafile = os.path.join(scratch, 'alpha{:04d}.npz'.format(self.idnum))
        self.saved_fields = ['ordered_constituents', 'alpha_data', 'freqs', 'P']
        self.memory = Namespace()
        if load_formal:
            self.setup_formalisms()

    def setup_formalisms(self):
        """Formalism choice (alpha.py:49-102) -> rb_set_formalisms; the line
        catalogues (given, or loaded as the formalism modules load them)
        -> rb_set_lines."""
        ca = dict(_cfg(self.config, 'constituent_alpha', None) or DEFAULT_CONSTITUENTS)
        self.constituent = {}
        for c, absorber in ca.items():
            if absorber is None:
                continue
            if c == 'nh3' and absorber in _NH3_FORMALISMS:
                self.constituent[c] = absorber
            elif _SUPPORTED.get(c) == absorber:
                self.constituent[c] = absorber
            else:
                raise ValueError('absorber {} for {} is not on the GPU path'.format(absorber, c))
        self.ordered_constituents = sorted(self.constituent.keys())
        self.other_dict = {}
        for absorber in self.ordered_constituents:
            self.other_dict[absorber] = {}
            for oc in _OTHER_TO_COPY.get(absorber, []):
                if self.config is not None and hasattr(self.config, oc):
                    self.other_dict[absorber][oc] = getattr(self.config, oc)
        self.engine.set_formalisms(self.constituent.get('nh3') or 'off',
                                   h2='h2' in self.constituent, h2o='h2o' in self.constituent,
                                   h2s='h2s' in self.constituent, ph3='ph3' in self.constituent,
                                   h2state=_cfg(self.config, 'h2state', 'e'))
        co = self.other_dict.get('co', {})
        self.engine.set_co_clouds(co='co' in self.constituent, coshape=co.get('coshape', 'voigt'),
                                  clouds=self.other_dict.get('clouds'))
        if self.lines is not None:
            catalog.upload(self.engine, self.lines)

    def reset_layers(self):
        self.P = None
        self.freqs = None
        self.layers = None

    # -------------------------------------------------------------- cache
    def save_alpha_data(self, save_type):
        """alpha.py:110-130: 'file' -> self.alphafile, 'memory' -> self.memory."""
        self.tosave = np.array(self.tosave)
        if save_type == 'file':
            np.savez(self.alphafile, ordered_constituents=self.ordered_constituents,
                     alpha_data=self.tosave, freqs=self.freqs, P=self.P)
        elif save_type == 'memory':
            self.memory.ordered_constituents = self.ordered_constituents
            self.memory.alpha_data = self.tosave
            self.memory.freqs = self.freqs
            self.memory.P = self.P

    def read_alpha_data(self, save_type):
        """alpha.py:132-149."""
        if save_type == 'file':
            alphain = np.load(self.alphafile)
            for sf in self.saved_fields:
                setattr(self, sf, alphain[sf])
        elif save_type == 'memory':
            for sf in self.saved_fields:
                setattr(self, sf, getattr(self.memory, sf))

    # -------------------------------------------------------------- scaling
    def total_layer_alpha(self, absorb, lscale):
        """alpha.py:151-192: sum of one layer's per-constituent absorption
        [nf, nC] with a number or per-constituent dict scale."""
        absorb = np.asarray(absorb, dtype=np.float64)
        if _isanynum(lscale):
            scaled = absorb * float(lscale)
        else:
            m = np.array([float(lscale[c]) if c in lscale else 1.0 for c in self.ordered_constituents])
            scaled = absorb * m[None, :]
        if self._save_alpha_memfil:
            self.tosave.append(scaled)
        return scaled.sum(axis=1)

    def get_layer_scale(self, scale, N):
        """alpha.py:235-259."""
        layer_scale = []
        if isinstance(scale, dict):
            for k, v in scale.items():
                if k not in self.ordered_constituents:
                    raise ValueError("{} not found as constituent for alpha".format(k))
                if len(v) != N:
                    raise ValueError("Incorrect scale for {}:  N {} vs {}".format(k, len(v), N))
            for lyr in range(N):
                layer_scale.append({k: v[lyr] for k, v in scale.items()})
        elif isinstance(scale, (list, np.ndarray)):
            if len(scale) != N:
                raise ValueError("Incorrect number of scale layers.")
            layer_scale = scale
        else:
            scale_val = float(scale) if _isanynum(scale) else 1.0
            layer_scale = [scale_val] * N
        return layer_scale

    def _scale_matrix(self, lscale):
        """Per-layer scale entries -> the C ABI's [nL][RB_NGAS] gas multipliers."""
        nL = len(lscale)
        m = np.ones((nL, len(_native.GASES)))
        for lyr, s in enumerate(lscale):
            if _isanynum(s):
                m[lyr, :] = float(s)
            else:
                for c, v in s.items():
                    m[lyr, _GAS_SLOT[c]] = float(v)
        return m

    # -------------------------------------------------------------- absorption
    def _per_gas(self, freqs, gas, C, cloud=None, Cl=None, scale_matrix=None):
        """[nL, nf, nC] per-constituent absorption (cm^-1) of gas [nC_gas, nL]
        and cloud [nC_cloud, nL]."""
        X = _native.x_matrix(gas, C, cloud, Cl)
        _, g = self.engine.alpha(gas[C['P']], gas[C['T']], X, freqs, scale=scale_matrix,
                                 per_gas=True, layers=False)
        cols = [_GAS_SLOT[c] for c in self.ordered_constituents]
        return g[:, :, cols]

    def get_alpha_from_calc(self, freqs, T, P, gas, gas_dict, cloud, cloud_dict, units='invcm'):
        """alpha.py:194-216: one layer, [nf, nC]."""
        if units not in ('invcm', '1/cm', 'cm^-1'):
            raise ValueError('units {} not supported on the GPU path (cm^-1)'.format(units))
        g = np.asarray(gas, dtype=np.float64).reshape(-1, 1).copy()
        g[gas_dict['T'], 0] = T
        g[gas_dict['P'], 0] = P
        cl = None if cloud is None else np.asarray(cloud, dtype=np.float64).reshape(-1, 1)
        return self._per_gas(np.atleast_1d(np.asarray(freqs, dtype=np.float64)), g, gas_dict,
                             cl, cloud_dict)[0]

    def get_single_layer(self, freqs, layer, atm, lscale, units='invcm'):
        """alpha.py:218-233."""
        if self._get_alpha_memfil:
            absorb = self.alpha_data[layer]
        else:
            C = atm.config.C
            cloud, Cl = _clouds(atm)
            absorb = self.get_alpha_from_calc(freqs, atm.gas[C['T']][layer], atm.gas[C['P']][layer],
                                              atm.gas[:, layer], C,
                                              None if cloud is None else cloud[:, layer], Cl, units)
        return self.total_layer_alpha(absorb=absorb, lscale=lscale)

    def get_layers(self, freqs, atm, scale=False, get_alpha='calc', save_alpha='none'):
        """alpha.py:261-305: every layer in one device call."""
        self.reset_layers()
        self.alpha_data = []
        self.tosave = []
        self.freqs = freqs
        C = atm.config.C
        self.P = atm.gas[C['P']]
        self._get_alpha_memfil = get_alpha in ['memory', 'file']
        self._save_alpha_memfil = save_alpha in ['memory', 'file']
        if self._get_alpha_memfil:
            self.read_alpha_data(get_alpha)
        numLayers = len(atm.gas[0])
        lscale = self.get_layer_scale(scale, numLayers)
        if self._get_alpha_memfil:
            layer_alpha = [self.get_single_layer(freqs, i, atm, lscale[i]) for i in range(numLayers)]
            self.layers = np.array(layer_alpha).transpose()
        else:
            f = np.atleast_1d(np.asarray(freqs, dtype=np.float64))
            sm = self._scale_matrix(lscale)
            X = _native.x_matrix(atm.gas, C, *_clouds(atm))
            lay, g = self.engine.alpha(atm.gas[C['P']], atm.gas[C['T']], X, f, scale=sm,
                                       per_gas=self._save_alpha_memfil)
            self.layers = lay
            if self._save_alpha_memfil:
                cols = [_GAS_SLOT[c] for c in self.ordered_constituents]
                self.tosave = list(g[:, :, cols])
        if self._save_alpha_memfil:
            self.save_alpha_data(save_alpha)
        del lscale, self.alpha_data, self.tosave
        return self.layers


def _clouds(atm):
    """(atm.cloud, atm.config.Cl) when the atmosphere carries clouds."""
    cloud = getattr(atm, 'cloud', None)
    Cl = getattr(atm.config, 'Cl', None)
    if cloud is None or Cl is None:
        return None, None
    return np.asarray(cloud, dtype=np.float64), Cl


# ------------------------------------------------------------------ ray paths
class Ray:
    """raypath.py:20-36."""

    allowed_parameters = ['ds', 'layer4ds', 'r4ds', 'P4ds', 'doppler', 'tip', 'rotate', 'rNorm']

    def __init__(self):
        for k in self.allowed_parameters:
            setattr(self, k, None)

    def update(self, **kwargs):
        for k, v in kwargs.items():
            if k in self.allowed_parameters:
                setattr(self, k, v)
            else:
                raise ValueError('{} not allowed Ray parameter'.format(k))


_GTYPE = {'ellipse': 'ellipse', 'sphere': 'sphere'}


def _geometry(atm, orientation, gtype):
    cfg = atm.config
    gtype = gtype if gtype is not None else getattr(cfg, 'gtype', 'ellipse')
    if gtype not in _GTYPE:
        raise ValueError('gtype {} not on the GPU path (ellipse, sphere)'.format(gtype))
    orientation = orientation if orientation is not None else getattr(cfg, 'orientation', [0.0, 0.0])
    R = atm.property[cfg.LP['R']]
    N = atm.property[cfg.LP['N']]
    Req = getattr(cfg, 'Req', R[0])
    Rpol = getattr(cfg, 'Rpol', Req)
    return R, N, float(Req), float(Rpol), (float(orientation[0]), float(orientation[1])), gtype


def compute_ds(atm, b, orientation=None, gtype=None, verbose=False, engine_=None):
    """raypath.py:108-273 for one impact parameter; off-planet rays return
    an empty Ray (ds None)."""
    R, N, Req, Rpol, orient, gtype = _geometry(atm, orientation, gtype)
    path = Ray()
    if b[0] ** 2 + b[1] ** 2 >= 1.0:
        return path
    eng = engine_ or engine(0)
    out = eng.raypath(R, N, np.array([b], dtype=np.float64), Req, Rpol, orientation=orient,
                      gtype=gtype, extras=True)
    n = int(out['nseg'][0])
    if n == 0:
        return path
    lay = out['layer'][0, :n]
    C = atm.config.C
    P = atm.gas[C['P']]
    tip, rotate = _aspect(orient, Req, Rpol)
    path.update(ds=list(out['ds'][0, :n]), layer4ds=list(lay), r4ds=list(out['r4ds'][0, :n]),
                P4ds=list(P[lay]), tip=tip, rotate=rotate, rNorm=R[0])
    return path


def _aspect(orientation, Req, Rpol):
    """computeAspect (raypath.py:39-44): the 'tip' to north and the
    sub-earth planetocentric latitude, radians."""
    f = 1.0 - Rpol / Req
    tip = -orientation[0] * np.pi / 180.0
    rotate = -np.arctan(np.tan(orientation[1] * np.pi / 180.0) * (1.0 - f) ** 2)
    return tip, rotate


# ------------------------------------------------------------------ brightness
class Brightness:
    """brightness.py:13-126."""

    def __init__(self, config=None, log=None, verbose=True, engine_=None, **kwargs):
        self.verbose = verbose
        self.log = log
        self.config = config
        self.engine = engine_ or engine(0)

    def single(self, b, freqs, atm, alpha, orientation=None, taulimit=20.0):
        """One ray (or 'disc': the nadir ray with E2 weighting); returns the
        Tb list and sets tau, W, Tb_lyr, integrated_W, travel, P, z."""
        disc_average = isinstance(b, str) and b.lower().startswith('dis')
        if disc_average:
            b = [0.0, 0.0]
        self.alpha = alpha
        self.freqs = freqs
        self.b = b
        if alpha.layers is None:
            alpha.get_layers(freqs, atm)
        travel = compute_ds(atm, b, orientation, gtype=None, engine_=self.engine)
        self.travel = travel
        nf = len(np.atleast_1d(freqs))
        if travel.ds is None:
            self.Tb = [T_CMB] * nf
            return self.Tb
        C = atm.config.C
        n = len(travel.ds)
        ds = np.array(travel.ds, dtype=np.float64)[None, :]
        lay = np.array(travel.layer4ds, dtype=np.int32)[None, :]
        out = self.engine.brightness(atm.gas[C['T']], np.asarray(alpha.layers, dtype=np.float64),
                                     np.array([n], dtype=np.int32), ds, lay, disc=disc_average,
                                     profiles=True)
        self.Tb = list(out['Tb'][0])
        self.tau = out['tau'][0][:, :n]
        self.W = out['W'][0][:, :n]
        self.Tb_lyr = out['TbL'][0][:, :n]
        self.integrated_W = out['intW'][0]
        P = atm.gas[C['P']]
        z = atm.gas[C['Z']] if 'Z' in C else np.zeros_like(P)
        l = np.array(travel.layer4ds)
        self.P = np.concatenate([[P[l[0]]], (P[l[:-1]] + P[l[1:]]) / 2.0])
        self.z = np.concatenate([[z[l[0]]], (z[l[:-1]] + z[l[1:]]) / 2.0])
        return self.Tb


# ------------------------------------------------------------------ binding
_RAY_STATE = ('travel', 'tau', 'W', 'Tb_lyr', 'P', 'z')


class _RayState:
    """Class attribute of the installed Brightness for the per-ray results
    that Planet.run's batched b loop does not compute up front (the path,
    tau, W, Tb_lyr, P, z of brightness.py:30-126).  A ray served from the
    batch leaves a pending record; the first read of any of these names
    evaluates that one ray on the GPU (path + profiles) and stores them.
    Assignments store directly."""

    def __init__(self, name):
        self.name = name

    def __get__(self, obj, owner=None):
        if obj is None:
            return self
        d = obj.__dict__
        if self.name not in d and d.get('_rb_pending') is not None:
            _materialise(obj)
        try:
            return d[self.name]
        except KeyError:
            raise AttributeError(self.name) from None

    def __set__(self, obj, value):
        obj.__dict__[self.name] = value


def _materialise(bright):
    """Path and profiles of the pending ray of a batched run (one GPU call)."""
    atm, alpha, b, freqs, orientation, eng = bright.__dict__.pop('_rb_pending')
    gb = Brightness(bright.config, verbose=False, engine_=eng)
    gb.single(b, freqs, atm, alpha, orientation)
    for k in _RAY_STATE:
        if hasattr(gb, k) and k not in bright.__dict__:   # an off-planet ray since set travel
            bright.__dict__[k] = getattr(gb, k)


def _run_batches(planet, eng):
    """All numeric rays of Planet.run's b list (planet.py:118-133), grouped
    by atmosphere (map_b_to_atm), through one rb_bright_run per atmosphere
    with the absorption its Alpha computed; results kept on planet.bright
    for the loop's Brightness.single calls."""
    batches = {}
    groups = {}
    for bv in planet.b:
        if isinstance(bv, str):
            continue
        groups.setdefault(planet.map_b_to_atm(bv), []).append(bv)
    orientation = planet.config.orientation
    for j, bl in groups.items():
        atm, alpha = planet.atmos[j], planet.alpha[j]
        if alpha.layers is None:
            continue
        R, N, Req, Rpol, orient, gtype = _geometry(atm, orientation, None)
        bb = np.array([[float(v[0]), float(v[1])] for v in bl])
        out = eng.bright_run(atm.gas[atm.config.C['T']], R, N, np.asarray(alpha.layers, dtype=np.float64),
                             bb, Req, Rpol, orientation=orient, gtype=gtype)
        rows = {}
        for k in range(len(bl)):
            rows[(bb[k, 0], bb[k, 1])] = (out['Tb'][k], out['intW'][k], int(out['nseg'][k]))
        batches[(id(atm), id(alpha))] = dict(rows=rows, layers=alpha.layers, orient=orient)
    planet.bright.__dict__['_rb_batches'] = batches


def _from_batch(bright, b, freqs, atm, alpha, orientation, eng):
    """Serve Brightness.single from the run's batch: True if it did."""
    batches = bright.__dict__.get('_rb_batches')
    if not batches or isinstance(b, str):
        return False
    ent = batches.get((id(atm), id(alpha)))
    if ent is None or ent['layers'] is not alpha.layers:
        return False
    R, N, Req, Rpol, orient, gtype = _geometry(atm, orientation, None)
    if orient != ent['orient']:
        return False
    row = ent['rows'].get((float(b[0]), float(b[1])))
    if row is None or len(row[0]) != len(np.atleast_1d(freqs)):
        return False
    tb, iw, nseg = row
    bright.alpha, bright.freqs, bright.b = alpha, freqs, b
    if nseg == 0:                      # off the planet (brightness.py:45-50): tau, W, ... stay
        bright.__dict__['travel'] = Ray()
        bright.Tb = [T_CMB] * len(tb)
        return True
    for k in _RAY_STATE:
        bright.__dict__.pop(k, None)
    bright.__dict__['_rb_pending'] = (atm, alpha, b, freqs, orientation, eng)
    bright.Tb = list(tb)
    bright.integrated_W = np.array(iw)
    return True


def _reference_lines(ref_alpha, cdir):
    """The catalogues a reference Alpha would load: the shipped .npz files
    with the instance's truncation (alpha.py:72-78, the loaders of
    h2s_ddb.py:14-39 and ph3_jh.py:18-61), and the h2o_bk lines its module
    builds (h2o_bk.py:17-62) with that truncation."""
    ts = {k: v for k, v in (getattr(ref_alpha, 'truncate_strength', None) or {}).items() if v is not None}
    tf = {k: v for k, v in (getattr(ref_alpha, 'truncate_freq', None) or {}).items() if v is not None}
    out = catalog.load_reference_catalogues(cdir, truncate_strength=ts, truncate_freq=tf)
    m = (getattr(ref_alpha, 'absorptionModule', None) or {}).get('h2o')
    if m is not None and hasattr(m, 'readInputFiles'):
        if getattr(m, 'data', None) is None:
            m.readInputFiles(Namespace(verbose=False, truncate_strength=ts.get('h2o'),
                                       truncate_freq=tf.get('h2o'), path=os.path.join(cdir, 'h2o'),
                                       units='invcm'))
        out['h2o'] = {k: np.array(v, dtype=np.float64) for k, v in m.data.items()}
    return out


def install(radiobear_pkg=None, lines=None, device=0, engine_=None):
    """Route an importable radiobear package to the GPU implementations:
    Alpha.get_layers, raypath.compute_ds and Brightness.single of the
    package are replaced, and Planet.init_run (called by Planet.run just
    before its b loop, planet.py:122) runs every ray of the loop in one
    rb_bright_run per atmosphere, which the loop's Brightness.single calls
    then read.  The Alpha's formalism choice and catalogues are taken from
    the instance; the catalogues are ``lines`` or, when None, the ones the
    instance would load itself (its truncation, its h2o_bk lines)."""
    if radiobear_pkg is None:
        import radiobear as radiobear_pkg   # noqa: F811
    from importlib import import_module
    ra = import_module(radiobear_pkg.__name__ + '.alpha')
    rr = import_module(radiobear_pkg.__name__ + '.raypath')
    rbm = import_module(radiobear_pkg.__name__ + '.brightness')
    try:
        rpl = import_module(radiobear_pkg.__name__ + '.planet')
    except ImportError:
        rpl = None
    eng = engine_ or engine(device)
    cdir = os.path.join(os.path.dirname(radiobear_pkg.__file__), 'constituents')
    state = {}

    def get_layers(self, freqs, atm, scale=False, get_alpha='calc', save_alpha='none'):
        gpu = self.__dict__.get('_rb_gpu')
        if gpu is None:
            own = lines if lines is not None else _reference_lines(self, cdir)
            gpu = Alpha(self.idnum, config=self.config, engine_=eng, lines=own)
            self._rb_gpu = gpu
        elif state.get('active') is not gpu:
            gpu.setup_formalisms()       # the engine last served another Alpha
        state['active'] = gpu
        gpu.alphafile, gpu.memory = self.alphafile, self.memory
        out = gpu.get_layers(freqs, atm, scale=scale, get_alpha=get_alpha, save_alpha=save_alpha)
        self.freqs, self.P, self.layers = gpu.freqs, gpu.P, gpu.layers
        return out

    def compute_ds_gpu(atm, b, orientation=None, gtype=None, verbose=False):
        path = compute_ds(atm, b, orientation, gtype, verbose, engine_=eng)
        ref = rr.Ray()
        ref.update(**{k: getattr(path, k) for k in path.allowed_parameters if getattr(path, k) is not None})
        return ref

    def single(self, b, freqs, atm, alpha, orientation=None, taulimit=20.0):
        if _from_batch(self, b, freqs, atm, alpha, orientation, eng):
            return self.Tb
        self.__dict__.pop('_rb_pending', None)
        gb = Brightness(self.config, engine_=eng)
        tb = gb.single(b, freqs, atm, alpha, orientation, taulimit)
        for k in ('alpha', 'freqs', 'b', 'travel', 'Tb', 'tau', 'W', 'Tb_lyr', 'integrated_W', 'P', 'z'):
            if hasattr(gb, k):
                setattr(self, k, getattr(gb, k))
        return tb

    ra.Alpha.get_layers = get_layers
    rr.compute_ds = compute_ds_gpu
    rbm.ray.compute_ds = compute_ds_gpu
    rbm.Brightness.single = single
    for k in _RAY_STATE:
        setattr(rbm.Brightness, k, _RayState(k))
    out = dict(alpha=ra.Alpha, compute_ds=compute_ds_gpu, brightness=rbm.Brightness)
    if rpl is not None and hasattr(rpl, 'Planet'):
        init_run0 = rpl.Planet.init_run

        def init_run(self):
            init_run0(self)
            _run_batches(self, eng)

        rpl.Planet.init_run = init_run
        out['planet'] = rpl.Planet
    return out
