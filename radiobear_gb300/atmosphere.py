"""Atmosphere producer on the GPU: ``computeProp`` and ``regrid``.

Mirrors ``AtmosphereBase.computeProp`` (radiobear/atm_base.py:120-194) and
``regrid.regrid`` (radiobear/regrid.py:11-176) over the C ABI
(``rb_atm_props``, ``rb_regrid`` and their ``_device`` forms for batches of
atmospheres resident on the device).  Tables are the reference's column
tables with their column dicts (``config.C`` for gas, ``config.Cl`` for
clouds); the per-column chemistry is that of
``chemistry.ConstituentProperties`` (radiobear/chemistry.py:8-48,168-200).
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native

# chemistry.py:18-19 (amu, g/mol), 29-30 (c_p / R), 43-44 (refractivity; H2O
# follows 245 + 1.28e6 / T, flagged by a negative constant)
AMU = {'H2': 2.016, 'HE': 4.003, 'H2S': 34.076, 'NH3': 17.030, 'H2O': 18.015,
       'CH4': 16.04, 'PH3': 33.997, 'NH4SH': 51.110}
CP = {'H2': 3.5, 'HE': 2.50, 'H2O': 4.00, 'NH3': 4.46, 'H2S': 4.01, 'CH4': 4.50}
REFR = {'H2': 124.43, 'HE': 35.832, 'H2O': -1.0, 'H2S': 2247.0, 'NH3': 2700.0, 'CH4': 413.0}
PROP_ROWS = ('Z', 'R', 'P', 'GM', 'AMU', 'REFR', 'N', 'H', 'LAPSE', 'LAPSEP', 'g')
ROLES = ('Z', 'T', 'P', 'DZ')


def columns(D, chemistry=True):
    """(roles int32[4], chem float64[3][ncol]) for a column dict.  Columns
    are named by D's keys at their index; unnamed rows carry no chemistry."""
    ncol = max(D.values()) + 1
    for r in ROLES:
        if r not in D:
            raise ValueError('column {} missing from the table dict'.format(r))
    roles = np.array([D[r] for r in ROLES], dtype=np.int32)
    chem = np.zeros((3, ncol))
    if chemistry:
        for k, i in D.items():
            if k in ROLES:
                continue
            key = k.upper()
            chem[0, i] = AMU.get(key, 0.0)
            chem[1, i] = CP.get(key, 0.0)
            chem[2, i] = REFR.get(key, 0.0)
    return roles, chem


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def props(engine, gas, C, Req, p_ref, GM_ref):
    """computeProp of one gas table -> property table [11, nL] (PROP_ROWS)."""
    gas = np.ascontiguousarray(gas, dtype=np.float64)
    roles, chem = columns(C)
    ncol, nL = chem.shape[1], gas.shape[1]
    if gas.shape[0] < ncol:
        raise ValueError('gas table has {} rows, the dict needs {}'.format(gas.shape[0], ncol))
    gas = np.ascontiguousarray(gas[:ncol])
    out = np.empty((len(PROP_ROWS), nL))
    rc = engine.lib.rb_atm_props(engine._h, nL, ncol, _ip(roles), _native._ptr(chem), _native._ptr(gas),
                                 float(Req), float(p_ref), float(GM_ref), _native._ptr(out))
    _native._check(engine.lib, rc, 'rb_atm_props')
    return out


def pressure_grid(P, regridType, Pmin=None, Pmax=None):
    """The grid regrid.regrid builds for an integer regridType
    (regrid.py:39-55): regridType points log-spaced over [Pmin, Pmax],
    defaults the table's extent."""
    if Pmin is None or Pmin == 'auto' or Pmin == 0:
        Pmin = float(np.min(P))
    if Pmax is None or Pmax == 'auto' or Pmax == 0:
        Pmax = float(np.max(P))
    return np.logspace(np.log10(Pmin), np.log10(Pmax), int(regridType))


def regrid(engine, gas, C, Pgrid, Req, p_ref, GM_ref, cloud=None, Cl=None):
    """regrid one gas (and cloud) table onto Pgrid -> (gas, cloud or None)."""
    gas = np.ascontiguousarray(gas, dtype=np.float64)
    roles, chem = columns(C)
    ncol, nin = chem.shape[1], gas.shape[1]
    gas = np.ascontiguousarray(gas[:ncol])
    grid = np.ascontiguousarray(Pgrid, dtype=np.float64)
    nout = grid.size
    gout = np.empty((ncol, nout))
    croles, cin, cout, ncl = None, None, None, 0
    if cloud is not None:
        croles, cchem = columns(Cl, chemistry=False)
        ncl = cchem.shape[1]
        cin = np.ascontiguousarray(np.asarray(cloud, dtype=np.float64)[:ncl])
        if cin.shape[1] != nin:
            raise ValueError('the cloud table must have the gas table layers')
        cout = np.empty((ncl, nout))
    rc = engine.lib.rb_regrid(engine._h, nin, ncol, _ip(roles), _native._ptr(chem), _native._ptr(gas),
                              ncl, None if croles is None else _ip(croles), _native._ptr(cin), nout,
                              _native._ptr(grid), float(Req), float(p_ref), float(GM_ref),
                              _native._ptr(gout), _native._ptr(cout))
    _native._check(engine.lib, rc, 'rb_regrid')
    return gout, cout


def regrid_atm(atm, regridType=None, Pmin=None, Pmax=None, engine=None):
    """regrid.regrid(atm, regridType, Pmin, Pmax) (regrid.py:11-82) on an
    object with the reference Atmosphere's ``gas``, ``cloud`` and
    ``config`` (C, Cl, Req, p_ref, GM_ref, regridType); integer (or
    integer-string) regridType only.  Replaces atm.gas / atm.cloud; returns
    0 when no regrid is asked for, else 1."""
    from .dropin import engine as shared_engine
    eng = engine or shared_engine(0)
    if regridType is None:
        regridType = atm.config.regridType
    if regridType is None or (isinstance(regridType, str) and regridType.lower() == 'none'):
        return 0
    if isinstance(regridType, str):
        regridType = int(regridType)
    C, Cl = atm.config.C, getattr(atm.config, 'Cl', None)
    grid = pressure_grid(atm.gas[C['P']], regridType, Pmin, Pmax)
    cloud = getattr(atm, 'cloud', None)
    g, c = regrid(eng, atm.gas, C, grid, atm.config.Req, atm.config.p_ref, atm.config.GM_ref,
                  cloud=cloud if Cl is not None else None, Cl=Cl)
    atm.gas = g
    if c is not None:
        atm.cloud = c
    return 1


def compute_prop(atm, engine=None):
    """AtmosphereBase.computeProp on the GPU: sets atm.property."""
    from .dropin import engine as shared_engine
    eng = engine or shared_engine(0)
    c = atm.config
    atm.property = props(eng, atm.gas, c.C, c.Req, c.p_ref, c.GM_ref)
    return atm.property
