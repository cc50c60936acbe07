"""Line catalogues in the reference's schemas, and their upload to a device.

A catalogue set is a dict with any of the keys

``ammonia``  nh3_hs schema of ``constituents/nh3/ammonia.npz``
             (fo Io Eo gammaNH3o H2HeBroad, *_rot, *_v2 columns)
``nh3``      nh3_sjs schema of ``constituents/nh3/nh3.npz`` (f0 I0 E G0)
``h2o``      h2o_bk dictionary (f_o I_o E_o w_s x_s w_h2 w_he x_h2 x_he SR)
``h2s``      ``constituents/h2s/h2s.npz`` (f0 I0 E GH2S)
``ph3``      ``constituents/ph3/ph3jh.npz`` (f0 I0 E)
``ph3wgt``   ``constituents/ph3/PH3WGT.npz`` (WgtI0 WgtFGB WgtSB)
``co``       ``constituents/co/co.npz`` (f0 I0 E)

Truncation follows the reference loaders: strength truncation keeps lines
with intensity > threshold, frequency truncation keeps f0 < threshold
(``h2s_ddb.py:23-38``, ``ph3_jh.py:28-61``, ``h2o_bk.py:51-62``).
"""
from __future__ import annotations

import os

import numpy as np

_NPZ = dict(ammonia=('nh3', 'ammonia.npz'), nh3=('nh3', 'nh3.npz'), h2s=('h2s', 'h2s.npz'),
            ph3=('ph3', 'ph3jh.npz'), ph3wgt=('ph3', 'PH3WGT.npz'), co=('co', 'co.npz'))


def load_reference_catalogues(constituents_dir, truncate_strength=None, truncate_freq=None):
    """Read the shipped ``.npz`` catalogues of a reference checkout and apply
    the loaders' truncation (dicts keyed by constituent: ``h2s``, ``ph3``...).
    The h2o_bk lines are built into the reference module, not a file; pass
    them with :func:`with_lines`."""
    ts = truncate_strength or {}
    tf = truncate_freq or {}
    out = {}
    for key, (sub, fname) in _NPZ.items():
        path = os.path.join(constituents_dir, sub, fname)
        if os.path.exists(path):
            z = np.load(path)
            out[key] = {k: np.array(z[k], dtype=np.float64) for k in z.files}
    if 'h2s' in out:
        out['h2s'] = truncate(out['h2s'], 'I0', 'f0', ts.get('h2s'), tf.get('h2s'))
    if 'ph3' in out and 'ph3wgt' in out:
        merged = dict(out['ph3'])
        merged.update(out['ph3wgt'])
        merged = truncate(merged, 'I0', 'f0', ts.get('ph3'), tf.get('ph3'))
        out['ph3'] = {k: merged[k] for k in ('f0', 'I0', 'E')}
        out['ph3wgt'] = {k: merged[k] for k in ('WgtI0', 'WgtFGB', 'WgtSB')}
    return out


def truncate(table, ikey, fkey, strength=None, freq=None):
    """Keep lines with ``table[ikey] > strength`` then ``table[fkey] < freq``."""
    t = {k: np.asarray(v, dtype=np.float64) for k, v in table.items()}
    if strength is not None:
        keep = t[ikey] > strength
        t = {k: v[keep] for k, v in t.items()}
    if freq is not None:
        keep = t[fkey] < freq
        t = {k: v[keep] for k, v in t.items()}
    return t


def family_tables(lines):
    """Split a catalogue set into the device families of the C ABI."""
    fam = {}
    a = lines.get('ammonia')
    if a is not None:
        fam['NH3_INV'] = {k: a[k] for k in ('fo', 'Io', 'Eo', 'gammaNH3o')}
        fam['NH3_ROT'] = {k: a[k] for k in ('fo_rot', 'Io_rot', 'Eo_rot', 'gNH3_rot', 'gH2_rot',
                                             'gHe_rot')}
        fam['NH3_V2'] = {k: a[k] for k in ('fo_v2', 'Io_v2', 'Eo_v2')}
    if lines.get('nh3') is not None:
        fam['NH3_SJS'] = lines['nh3']
    if lines.get('h2o') is not None:
        fam['H2O'] = lines['h2o']
    if lines.get('h2s') is not None:
        fam['H2S'] = lines['h2s']
    if lines.get('ph3') is not None:
        p = dict(lines['ph3'])
        w = lines.get('ph3wgt')
        if w is None:
            n = len(p['f0'])
            w = dict(WgtI0=np.ones(n), WgtFGB=np.ones(n), WgtSB=np.ones(n))
        p.update(w)
        fam['PH3'] = p
    if lines.get('co') is not None:
        fam['CO'] = {k: lines['co'][k] for k in ('f0', 'I0', 'E')}
    return fam


def upload(engine, lines):
    """Upload every family present in ``lines``; absent families are cleared."""
    fam = family_tables(lines)
    for name in ('NH3_INV', 'NH3_ROT', 'NH3_V2', 'NH3_SJS', 'H2O', 'H2S', 'PH3', 'CO'):
        engine.set_lines(name, fam.get(name))
