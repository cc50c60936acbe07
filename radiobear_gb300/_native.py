"""ctypes binding of the C ABI in ``include/radiobear_gb300.h``.

The shared library is built in-tree by :mod:`radiobear_gb300.build`.  There
is no CPU fallback: if the library cannot be loaded, or no CUDA device is
present, every compute call raises.
"""
from __future__ import annotations

import ctypes
import os
import threading

import numpy as np

from . import build as _build

LIB_PATH = _build.LIB
ABI_VERSION = 3      # RB_ABI_VERSION of include/radiobear_gb300.h

RB_OK = 0
FAM = dict(NH3_INV=0, NH3_ROT=1, NH3_V2=2, NH3_SJS=3, H2O=4, H2S=5, PH3=6, CO=7)
NH3_MODE = dict(off=0, nh3_hs=1, nh3_sjs=2, nh3_hs_sjs=3, nh3_dbs=4, nh3_dbs_sjs=5)
GASES = ('h2', 'h2o', 'h2s', 'nh3', 'ph3', 'co', 'clouds')        # RB_GAS_* order
# RB_X_* order: gas mole fractions (gas table columns), then cloud densities
# (cloud table columns, prefixed 'cl:')
X_ROWS = ('H2', 'HE', 'CH4', 'NH3', 'H2O', 'H2S', 'PH3', 'CO',
          'cl:H2O', 'cl:SOLN', 'cl:NH4SH', 'cl:NH3', 'cl:H2S', 'cl:CH4')
COSHAPE = dict(voigt=0, vvw=1, diff=2)              # anything else: 3 (blended, 'std')
# clouds_idp other_dict keys -> RB_CLOUD_* bits (clouds_idp.py:16-49 tests
# 'ice_p', 'water_p', 'nh4sh_p', 'nh3ice_p', 'h2sice_p' and 'ch4')
CLOUD_BITS = dict(ice_p=1, water_p=2, nh4sh_p=4, nh3ice_p=8, h2sice_p=16, ch4=32)
GTYPE = dict(ellipse=0, sphere=1, circle=1)
LIMB = dict(shape=0, sec=1)

# column order per family (the reference catalogue keys)
FAMILY_COLUMNS = {
    'NH3_INV': ('fo', 'Io', 'Eo', 'gammaNH3o'),
    'NH3_ROT': ('fo_rot', 'Io_rot', 'Eo_rot', 'gNH3_rot', 'gH2_rot', 'gHe_rot'),
    'NH3_V2': ('fo_v2', 'Io_v2', 'Eo_v2'),
    'NH3_SJS': ('f0', 'I0', 'E', 'G0'),
    'H2O': ('f_o', 'I_o', 'E_o', 'w_s', 'x_s', 'w_h2', 'w_he', 'x_h2', 'x_he', 'SR'),
    'H2S': ('f0', 'I0', 'E', 'GH2S'),
    'PH3': ('f0', 'I0', 'E', 'WgtI0', 'WgtFGB', 'WgtSB'),
    'CO': ('f0', 'I0', 'E'),
}

EXPORTS = ('rb_abi_version', 'rb_last_error', 'rb_create', 'rb_destroy', 'rb_set_lines',
           'rb_set_formalisms', 'rb_alpha', 'rb_raypath', 'rb_brightness', 'rb_forward',
           'rb_forward_device', 'rb_last_launch_count', 'rb_set_profiling', 'rb_phase_times',
           'rb_probe_fp32_peak', 'rb_debug_e2', 'rb_set_alpha_tiling', 'rb_adjoint',
           'rb_adjoint_device', 'rb_forward_batch_device', 'rb_adjoint_batch_device',
           'rb_set_co_clouds', 'rb_atm_props', 'rb_atm_props_device', 'rb_regrid',
           'rb_regrid_device', 'rb_bright_run', 'rb_debug_e1', 'rb_set_tuning')

_lib = None
_lock = threading.Lock()

_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int32)
_vp = ctypes.c_void_p


class RBError(RuntimeError):
    """A non-zero status from the C ABI."""


def load_library(path=None):
    """Load (once) and return the ctypes library with typed prototypes."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = path or LIB_PATH
        if not os.path.exists(p):
            raise RBError('radiobear_gb300 CUDA library not built ({}); run '
                          '`python -m radiobear_gb300.build`'.format(p))
        lib = ctypes.CDLL(p)
        c_int, c_double = ctypes.c_int, ctypes.c_double
        lib.rb_abi_version.restype = c_int
        lib.rb_last_error.restype = ctypes.c_char_p
        lib.rb_create.argtypes = [ctypes.POINTER(_vp), c_int]
        lib.rb_destroy.argtypes = [_vp]
        lib.rb_set_lines.argtypes = [_vp, c_int, c_int, c_int, _d]
        lib.rb_set_formalisms.argtypes = [_vp, c_int, c_int, c_int, c_int, c_int, c_int]
        lib.rb_set_co_clouds.argtypes = [_vp, c_int, c_int, c_int, c_int]
        _ip32 = ctypes.POINTER(ctypes.c_int32)
        lib.rb_atm_props.argtypes = [_vp, c_int, c_int, _ip32, _d, _d, c_double, c_double, c_double, _d]
        lib.rb_atm_props_device.argtypes = [_vp, _vp, c_int, _ip32, c_int, _ip32, _d, _vp, c_double,
                                            c_double, c_double, _vp]
        lib.rb_regrid.argtypes = [_vp, c_int, c_int, _ip32, _d, _d, c_int, _ip32, _d, c_int, _d,
                                  c_double, c_double, c_double, _d, _d]
        lib.rb_regrid_device.argtypes = [_vp, _vp, c_int, _ip32, c_int, _ip32, _d, _vp, c_int, _ip32,
                                         _vp, c_int, _vp, c_int, c_double, c_double, c_double, _vp,
                                         _vp]
        lib.rb_alpha.argtypes = [_vp, c_int, _d, _d, _d, c_int, _d, _d, c_int, _d, _d]
        lib.rb_raypath.argtypes = [_vp, c_int, _d, _d, c_double, c_double, c_double, c_double,
                                   c_int, c_int, c_int, _d, c_int, _i, _d, _i, _d, _d, _i]
        lib.rb_brightness.argtypes = [_vp, c_int, _d, c_int, _d, c_int, _i, _d, _i, c_int, c_int,
                                      _d, _d, _d, _d, _d]
        lib.rb_bright_run.argtypes = [_vp, c_int, _d, _d, _d, c_double, c_double, c_double, c_double,
                                      c_int, c_int, c_int, _d, c_int, _d, _d, _d, _i]
        # host arrays as addresses (numpy .ctypes.data): cheaper per call than pointer objects
        lib.rb_forward.argtypes = [_vp, c_int, _vp, _vp, _vp, _vp, _vp, c_int, _vp, _vp, c_double,
                                   c_double, c_double, c_double, c_int, c_int, c_int, _vp, _vp,
                                   c_int, _vp, _vp, _vp]
        lib.rb_forward_device.argtypes = [_vp, _vp, c_int, _vp, _vp, _vp, _vp, _vp, c_int, _d, _vp,
                                          c_double, c_double, c_double, c_double, c_int, c_int,
                                          c_int, _vp, _vp, c_int, _vp, _vp]
        lib.rb_last_launch_count.argtypes = [_vp]
        lib.rb_debug_e2.argtypes = [_vp, c_int, _d, _d]
        lib.rb_debug_e1.argtypes = [_vp, c_int, _d, _d]
        lib.rb_set_profiling.argtypes = [_vp, c_int]
        lib.rb_phase_times.argtypes = [_vp, _d, c_int]
        lib.rb_probe_fp32_peak.argtypes = [_vp, _d]
        lib.rb_set_alpha_tiling.argtypes = [_vp, c_int, c_int, c_int]
        lib.rb_set_tuning.argtypes = [_vp, c_int, c_int]
        lib.rb_adjoint.argtypes = [_vp, c_int, _vp, _vp, _vp, _vp, _vp, c_int, _vp, _vp, c_double,
                                   c_double, c_double, c_double, c_int, c_int, c_int, _vp, _vp, c_int,
                                   _vp, _vp, _vp, _vp, _vp, _vp]
        _ip = ctypes.POINTER(ctypes.c_int32)
        lib.rb_forward_batch_device.argtypes = [_vp, _vp, c_int, _ip, _vp, _vp, _vp, _vp, _vp, c_int, _d,
                                                _vp, c_double, c_double, c_double, c_double, c_int,
                                                c_int, c_int, _vp, _vp, _vp]
        lib.rb_adjoint_batch_device.argtypes = [_vp, _vp, c_int, _ip, _vp, _vp, _vp, _vp, _vp, c_int, _d,
                                                _vp, c_double, c_double, c_double, c_double, c_int,
                                                c_int, c_int, _vp, _vp, _vp, _vp, _vp, _vp, _vp]
        lib.rb_adjoint_device.argtypes = [_vp, _vp, c_int, _vp, _vp, _vp, _vp, _vp, c_int, _d, _vp,
                                          c_double, c_double, c_double, c_double, c_int, c_int,
                                          c_int, _vp, _vp, c_int, _vp, _vp, _vp, _vp, _vp, _vp]
        for name in EXPORTS:
            getattr(lib, name).restype = getattr(lib, name).restype or c_int
        lib.rb_last_error.restype = ctypes.c_char_p
        if lib.rb_abi_version() != ABI_VERSION:
            raise RBError('{} has ABI version {}, this binding expects {}; rebuild it with '
                          '`python -m radiobear_gb300.build`'.format(p, lib.rb_abi_version(),
                                                                     ABI_VERSION))
        _lib = lib
        return lib


def _ptr(a, ctype=ctypes.c_double):
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _addr(a):
    """Address of a contiguous numpy array (None stays None)."""
    return None if a is None else a.ctypes.data


def _check(lib, rc, what):
    if rc != RB_OK:
        msg = lib.rb_last_error().decode(errors='replace')
        if rc == 1:
            raise ValueError('{}: {}'.format(what, msg))
        raise RBError('{} failed (status {}): {}'.format(what, rc, msg))


class Engine:
    """One device handle: catalogues, formalism switches and workspaces."""

    def __init__(self, device=0):
        self.lib = load_library()
        h = _vp()
        _check(self.lib, self.lib.rb_create(ctypes.byref(h), int(device)), 'rb_create')
        self._h = h
        self.device = device
        self.families = {}

    def close(self):
        if getattr(self, '_h', None):
            self.lib.rb_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------ catalogues
    def set_lines(self, family, table):
        """Upload a family from a dict with the reference's catalogue keys."""
        cols = FAMILY_COLUMNS[family]
        if table is None:
            n = 0
            arr = np.zeros(len(cols))
        else:
            n = len(np.asarray(table[cols[0]]))
            arr = np.concatenate([_f64(table[c]).reshape(-1) for c in cols]) if n else np.zeros(len(cols))
        _check(self.lib, self.lib.rb_set_lines(self._h, FAM[family], n, len(cols), _ptr(arr)),
               'rb_set_lines')
        self.families[family] = n

    def set_formalisms(self, nh3='nh3_hs_sjs', h2=True, h2o=True, h2s=True, ph3=True, h2state='e'):
        _check(self.lib, self.lib.rb_set_formalisms(self._h, NH3_MODE[nh3 or 'off'], int(h2), int(h2o),
                                                    int(h2s), int(ph3), ord(h2state)),
               'rb_set_formalisms')

    def set_co_clouds(self, co=False, coshape='voigt', clouds=None):
        """co_ddb on/off with its line shape (other_dict['coshape']), and
        clouds_idp: None (off) or its other_dict (particle switches)."""
        mask = 0
        if clouds is not None:
            for k, bit in CLOUD_BITS.items():
                if k in clouds and clouds[k] > 0.0:
                    mask |= bit
        _check(self.lib, self.lib.rb_set_co_clouds(self._h, int(bool(co)), COSHAPE.get(coshape, 3),
                                                   int(clouds is not None), mask),
               'rb_set_co_clouds')

    # ------------------------------------------------------------ compute
    def alpha(self, P, T, X, freqs, scale=None, units_db=False, per_gas=False, layers=True):
        """Absorption: returns (layers [nf, nL] or None, gas [nL, nf, RB_NGAS] or None)."""
        P, T, X, f = _f64(P), _f64(T), _f64(X), _f64(freqs)
        nL, nf = P.size, f.size
        sc = None if scale is None else _f64(scale)
        lay = np.empty((nf, nL)) if layers else None
        gas = np.empty((nL, nf, len(GASES))) if per_gas else None
        rc = self.lib.rb_alpha(self._h, nL, _ptr(P), _ptr(T), _ptr(X), nf, _ptr(f), _ptr(sc),
                               int(units_db), _ptr(lay), _ptr(gas))
        _check(self.lib, rc, 'rb_alpha')
        return lay, gas

    def raypath(self, R, N, b, Req, Rpol, orientation=(0.0, 0.0), gtype='ellipse', limb='shape',
                max_seg=None, extras=False):
        R, N = _f64(R), _f64(N)
        b = _f64(np.atleast_2d(b))
        nL, nb = R.size, b.shape[0]
        ms = max_seg or 2 * nL + 4
        nseg = np.zeros(nb, dtype=np.int32)
        ds = np.zeros((nb, ms))
        lay = np.zeros((nb, ms), dtype=np.int32)
        r4 = np.zeros((nb, ms)) if extras else None
        ll = np.zeros((nb, ms + 1, 2)) if extras else None
        end = np.zeros(nb, dtype=np.int32)
        rc = self.lib.rb_raypath(self._h, nL, _ptr(R), _ptr(N), float(Req), float(Rpol),
                                 float(orientation[0]), float(orientation[1]), GTYPE[gtype],
                                 LIMB[limb], nb, _ptr(b), ms, _ptr(nseg, ctypes.c_int32), _ptr(ds),
                                 _ptr(lay, ctypes.c_int32), _ptr(r4), _ptr(ll),
                                 _ptr(end, ctypes.c_int32))
        _check(self.lib, rc, 'rb_raypath')
        out = dict(nseg=nseg, ds=ds, layer=lay, end=end, max_seg=ms)
        if extras:
            out.update(r4ds=r4, latlng=ll)
        return out

    def brightness(self, T, layers, nseg, ds, layer, disc=False, profiles=False):
        T, layers = _f64(T), _f64(layers)
        nf, nL = layers.shape
        nseg = np.ascontiguousarray(nseg, dtype=np.int32)
        ds = _f64(ds)
        layer = np.ascontiguousarray(layer, dtype=np.int32)
        nb, ms = ds.shape
        Tb = np.empty((nb, nf))
        iw = np.empty((nb, nf))
        tau = W = tbl = None
        if profiles:
            tau, W, tbl = (np.empty((nb, nf, ms)) for _ in range(3))
        rc = self.lib.rb_brightness(self._h, nL, _ptr(T), nf, _ptr(layers), nb,
                                    _ptr(nseg, ctypes.c_int32), _ptr(ds),
                                    _ptr(layer, ctypes.c_int32), ms, int(disc), _ptr(Tb), _ptr(iw),
                                    _ptr(tau), _ptr(W), _ptr(tbl))
        _check(self.lib, rc, 'rb_brightness')
        return dict(Tb=Tb, intW=iw, tau=tau, W=W, TbL=tbl)

    def bright_run(self, T, R, N, layers, b, Req, Rpol, orientation=(0.0, 0.0), gtype='ellipse',
                   limb='shape'):
        """Every ray of b[nb, 2] through one atmosphere with the given
        absorption layers [nf, nL] (rb_bright_run): returns Tb [nb, nf],
        intW [nb, nf] and nseg [nb]."""
        T, R, N, layers = _f64(T), _f64(R), _f64(N), _f64(layers)
        b = _f64(np.atleast_2d(b))
        nf, nL = layers.shape
        nb = b.shape[0]
        Tb = np.empty((nb, nf))
        iw = np.empty((nb, nf))
        nseg = np.zeros(nb, dtype=np.int32)
        rc = self.lib.rb_bright_run(self._h, nL, _ptr(T), _ptr(R), _ptr(N), float(Req), float(Rpol),
                                    float(orientation[0]), float(orientation[1]), GTYPE[gtype],
                                    LIMB[limb], nf, _ptr(layers), nb, _ptr(b), _ptr(Tb), _ptr(iw),
                                    _ptr(nseg, ctypes.c_int32))
        _check(self.lib, rc, 'rb_bright_run')
        return dict(Tb=Tb, intW=iw, nseg=nseg)

    def forward(self, P, T, X, R, N, freqs, b, Req, Rpol, orientation=(0.0, 0.0),
                gtype='ellipse', limb='shape', weights=None, disc=False, scale=None,
                want_layers=False, want_rays=True):
        P, T, X, R, N, f = (_f64(v) for v in (P, T, X, R, N, freqs))
        b = _f64(np.atleast_2d(b))
        nL, nf, nb = P.size, f.size, b.shape[0]
        w = None if weights is None else _f64(weights)
        sc = None if scale is None else _f64(scale)
        Tb = np.empty((nb, nf)) if want_rays else None
        avg = np.empty(nf) if w is not None else None
        lay = np.empty((nf, nL)) if want_layers else None
        rc = self.lib.rb_forward(self._h, nL, _addr(P), _addr(T), _addr(X), _addr(R), _addr(N), nf,
                                 _addr(f), _addr(sc), float(Req), float(Rpol), float(orientation[0]),
                                 float(orientation[1]), GTYPE[gtype], LIMB[limb], nb, _addr(b),
                                 _addr(w), int(disc), _addr(Tb), _addr(avg), _addr(lay))
        _check(self.lib, rc, 'rb_forward')
        return dict(Tb=Tb, Tb_avg=avg, layers=lay)

    def forward_device(self, stream, nL, nb, P, T, X, R, N, freqs_host, b, Req, Rpol, Tb_out,
                       weights=None, Tb_avg=None, orientation=(0.0, 0.0), gtype='ellipse',
                       limb='shape', scale=None, disc=False):
        """Device-pointer variant of :meth:`forward`: P, T, X, R, N, b,
        weights, scale, Tb_out and Tb_avg are integer device addresses (for
        example ``tensor.data_ptr()``), ``stream`` an integer cudaStream_t.
        The work is enqueued on ``stream`` and the call returns at once.
        disc applies the E2 weighting to the rays given."""
        f = _f64(freqs_host)

        def vp(x):
            return None if x is None else _vp(int(x))

        rc = self.lib.rb_forward_device(
            self._h, _vp(int(stream)), int(nL), vp(P), vp(T), vp(X), vp(R), vp(N), f.size, _ptr(f),
            vp(scale), float(Req), float(Rpol), float(orientation[0]), float(orientation[1]),
            GTYPE[gtype], LIMB[limb], int(nb), vp(b), vp(weights), int(bool(disc)), vp(Tb_out),
            vp(Tb_avg))
        _check(self.lib, rc, 'rb_forward_device')

    def adjoint(self, P, T, X, R, N, freqs, b, Req, Rpol, grad, weights=None,
                orientation=(0.0, 0.0), gtype='ellipse', limb='shape', scale=None, disc=False):
        """Forward Tb and the gradient of sum(grad * Tb_avg) (weights given,
        grad [nf]) or sum(grad * Tb) (grad [nb, nf]) with respect to each
        layer's T, P and ln X of NH3, H2O, H2S.  disc: the b = 'disc' E2
        weighting on the nadir ray.  Returns dict(Tb, Tb_avg, dT, dP,
        dlnX [3, nL])."""
        P, T, X, R, N, f = (_f64(v) for v in (P, T, X, R, N, freqs))
        b = _f64(np.atleast_2d(b))
        nL, nf, nb = P.size, f.size, b.shape[0]
        w = None if weights is None else _f64(weights)
        g = _f64(grad)
        want = (nf,) if w is not None else (nb, nf)
        if g.shape != want:
            raise ValueError('grad must have shape {}'.format(want))
        sc = None if scale is None else _f64(scale)
        Tb = np.empty((nb, nf))
        avg = np.empty(nf) if w is not None else None
        dT, dP, dlnX = np.empty(nL), np.empty(nL), np.empty((3, nL))
        rc = self.lib.rb_adjoint(self._h, nL, _addr(P), _addr(T), _addr(X), _addr(R), _addr(N), nf,
                                 _addr(f), _addr(sc), float(Req), float(Rpol), float(orientation[0]),
                                 float(orientation[1]), GTYPE[gtype], LIMB[limb], nb, _addr(b),
                                 _addr(w), int(bool(disc)), _addr(g), _addr(Tb), _addr(avg),
                                 _addr(dT), _addr(dP), _addr(dlnX))
        _check(self.lib, rc, 'rb_adjoint')
        return dict(Tb=Tb, Tb_avg=avg, dT=dT, dP=dP, dlnX=dlnX)

    def adjoint_device(self, stream, nL, nb, P, T, X, R, N, freqs_host, b, Req, Rpol, grad, dT,
                       dP, dlnX, weights=None, Tb_out=None, Tb_avg=None, orientation=(0.0, 0.0),
                       gtype='ellipse', limb='shape', scale=None, disc=False):
        """Device-pointer variant of :meth:`adjoint` (integer device
        addresses, enqueued on ``stream``)."""
        f = _f64(freqs_host)

        def vp(x):
            return None if x is None else _vp(int(x))

        rc = self.lib.rb_adjoint_device(
            self._h, _vp(int(stream)), int(nL), vp(P), vp(T), vp(X), vp(R), vp(N), f.size, _ptr(f),
            vp(scale), float(Req), float(Rpol), float(orientation[0]), float(orientation[1]),
            GTYPE[gtype], LIMB[limb], int(nb), vp(b), vp(weights), int(bool(disc)), vp(grad),
            vp(Tb_out), vp(Tb_avg), vp(dT), vp(dP), vp(dlnX))
        _check(self.lib, rc, 'rb_adjoint_device')

    def forward_batch_device(self, stream, nL_list, P, T, X, R, N, freqs_host, b, weights, Tb_avg,
                             Req, Rpol, orientation=(0.0, 0.0), gtype='ellipse', limb='shape',
                             scale=None):
        """Batch of atmospheres (see rb_forward_batch_device): nL_list host
        layer counts; P, T, R, N, X, b, weights, Tb_avg (and scale
        [sum nL][RB_NGAS], optional) integer device addresses."""
        nl = np.ascontiguousarray(nL_list, dtype=np.int32)
        f = _f64(freqs_host)
        rc = self.lib.rb_forward_batch_device(
            self._h, _vp(int(stream)), nl.size, nl.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            _vp(int(P)), _vp(int(T)), _vp(int(X)), _vp(int(R)), _vp(int(N)), f.size, _ptr(f),
            None if scale is None else _vp(int(scale)), float(Req), float(Rpol), float(orientation[0]), float(orientation[1]), GTYPE[gtype],
            LIMB[limb], int(self._nb(b)), _vp(int(b.data_ptr())), _vp(int(weights)), _vp(int(Tb_avg)))
        _check(self.lib, rc, 'rb_forward_batch_device')

    def adjoint_batch_device(self, stream, nL_list, P, T, X, R, N, freqs_host, b, weights, grad,
                             Tb_avg, dT, dP, dlnX, Req, Rpol, orientation=(0.0, 0.0),
                             gtype='ellipse', limb='shape', scale=None):
        """Forward + adjoint of a batch (see rb_adjoint_batch_device)."""
        nl = np.ascontiguousarray(nL_list, dtype=np.int32)
        f = _f64(freqs_host)
        rc = self.lib.rb_adjoint_batch_device(
            self._h, _vp(int(stream)), nl.size, nl.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
            _vp(int(P)), _vp(int(T)), _vp(int(X)), _vp(int(R)), _vp(int(N)), f.size, _ptr(f),
            None if scale is None else _vp(int(scale)), float(Req), float(Rpol), float(orientation[0]), float(orientation[1]), GTYPE[gtype],
            LIMB[limb], int(self._nb(b)), _vp(int(b.data_ptr())), _vp(int(weights)), _vp(int(grad)),
            _vp(int(Tb_avg)), _vp(int(dT)), _vp(int(dP)), _vp(int(dlnX)))
        _check(self.lib, rc, 'rb_adjoint_batch_device')

    @staticmethod
    def _nb(b):
        """Rays of a [nb, 2] device tensor of impact parameters."""
        return int(b.shape[0])

    def last_launch_count(self):
        return int(self.lib.rb_last_launch_count(self._h))

    def set_alpha_tiling(self, M=0, W=0, item_lines=0):
        """Line-sum tiling: M slots per thread, W warps per CTA, lines per work
        item (zeros: automatic)."""
        _check(self.lib, self.lib.rb_set_alpha_tiling(self._h, int(M), int(W), int(item_lines)),
               'rb_set_alpha_tiling')

    TUNING = dict(jvp_freqs=1, jvp_ctas=2, scan_lanes=3, jvp_threads=4, adj_mode=5)   # RB_TUNE_*

    def set_tuning(self, **kw):
        """Launch shapes (rb_set_tuning): jvp_freqs (32/64/128), jvp_ctas (3/4),
        jvp_threads (128/256), scan_lanes (power of two in 4..128); 0 = automatic."""
        for k, v in kw.items():
            _check(self.lib, self.lib.rb_set_tuning(self._h, self.TUNING[k], int(v)), 'rb_set_tuning')

    def set_profiling(self, on=True):
        _check(self.lib, self.lib.rb_set_profiling(self._h, int(on)), 'rb_set_profiling')

    PHASES = ('prep', 'alpha', 'raypath', 'brightness', 'disc_avg', 'assembly')

    def phase_times(self):
        """Milliseconds of each phase of the last forward call."""
        ms = np.zeros(len(self.PHASES))
        _check(self.lib, self.lib.rb_phase_times(self._h, _ptr(ms), ms.size), 'rb_phase_times')
        return dict(zip(self.PHASES, ms.tolist()))

    def probe_fp32_peak(self):
        out = np.zeros(1)
        _check(self.lib, self.lib.rb_probe_fp32_peak(self._h, _ptr(out)), 'rb_probe_fp32_peak')
        return float(out[0])

    def debug_e2(self, x):
        x = _f64(x)
        out = np.empty_like(x)
        _check(self.lib, self.lib.rb_debug_e2(self._h, x.size, _ptr(x), _ptr(out)), 'rb_debug_e2')
        return out

    def debug_e1(self, x):
        x = _f64(x)
        out = np.empty_like(x)
        _check(self.lib, self.lib.rb_debug_e1(self._h, x.size, _ptr(x), _ptr(out)), 'rb_debug_e1')
        return out


def x_matrix(gas, C, cloud=None, Cl=None):
    """[RB_NX, nL] composition rows from a reference gas table and index
    dict, plus the cloud table and its dict when given (missing columns are
    zero)."""
    nL = gas.shape[1]
    X = np.zeros((len(X_ROWS), nL))
    for i, k in enumerate(X_ROWS):
        if k.startswith('cl:'):
            if cloud is not None and Cl is not None and k[3:] in Cl:
                X[i] = cloud[Cl[k[3:]]]
        elif k in C:
            X[i] = gas[C[k]]
    return X
