"""Seeded synthetic workloads for the radioBEAR forward model.

Every input is generated in float64 from ``numpy.random.default_rng(seed)`` so
that the GPU path, the CPU oracle and the reference harness see identical
numbers.  The layouts follow the reference's own containers:

* the gas table has the reference's default column order
  (``radiobear/default_config.json`` token ``constituents``:
  Z T P H2 HE CH4 NH3 H2O H2S SOLN OTHER PH3 CO CO13 HCN DZ), pressure
  increasing with index (``radiobear/atm_base.py:69-75``) and the deepest
  layer at z = 0 (``radiobear/atm_base.py:206-219``);
* the property table (R, N, GM, ...) is a vectorised restatement of
  ``AtmosphereBase.computeProp`` (``radiobear/atm_base.py:120-194``);
* line lists are dictionaries with the keys of the reference catalogues
  (``constituents/nh3/ammonia.npz``, ``nh3.npz``, ``h2s.npz``, the ``h2o_bk``
  built-in dictionary ``constituents/h2o/h2o_bk.py:17-62``).

Workloads (shapes of the five benchmark configurations):

=====  ==================================================================
C0     200 layers 1e-3..100 bar, 21 freqs ``'1:100:5'``, one nadir ray,
       200-line synthetic NH3 list; H2O/H2S/PH3 from the real catalogues.
C1     1000 layers 1e-3..500 bar, 256 log freqs 0.5..100 GHz, 64-point
       Gauss-Legendre disc quadrature; NH3 2000 + H2O 500 + H2S 200
       synthetic lines, PH3 the real 33 truncated lines.
C2     C1 atmosphere and lines, 8 freqs, 256x256 image grid at 0.01 rNorm.
C3     C1 atmosphere and lines, 64 log freqs 1..50 GHz, 16 disc rays.
C4     4096 variants of the C0 recipe (nL uniform 300..1200, deep NH3
       log-uniform 1e-4..1e-3, deep T offset +-10 K), 128 log freqs
       0.5..50 GHz, 32 disc rays.
=====  ==================================================================
"""
from __future__ import annotations

import numpy as np

# Column orders of the reference's default configuration
# (radiobear/default_config.json, tokens "constituents", "clouds", "other").
GAS_COLUMNS = ['Z', 'T', 'P', 'H2', 'HE', 'CH4', 'NH3', 'H2O', 'H2S', 'SOLN',
               'OTHER', 'PH3', 'CO', 'CO13', 'HCN', 'DZ']
CLOUD_COLUMNS = ['Z', 'T', 'P', 'SOLN', 'H2O', 'NH4SH', 'NH3', 'H2S', 'CH4',
                 'AR', 'PH3', 'DZ']
PROPERTY_COLUMNS = ['Z', 'R', 'P', 'GM', 'AMU', 'REFR', 'N', 'H', 'LAPSE',
                    'LAPSEP', 'g']

# Jupiter defaults (radiobear/default_config.json: req, rpol, p_ref, gm).
JUPITER = dict(Req=71492.0, Rpol=66854.0, p_ref=1.0, GM_ref=126686538.0)

# Physical constants as used by the reference's chemistry module
# (radiobear/chemistry.py:7-9,18-19,29-30,45-46).
GRAV_CONST = 6.6738e-20      # km3/kg/s2
R_GAS = 8.314462             # J/K/mol
AMU = {'H2': 2.016, 'HE': 4.003, 'H2S': 34.076, 'NH3': 17.030, 'H2O': 18.015,
       'CH4': 16.04, 'PH3': 33.997}
CP_OVER_R = {'H2': 3.5, 'HE': 2.50, 'H2O': 4.00, 'NH3': 4.46, 'H2S': 4.01,
             'CH4': 4.50}
REFRACTIVITY = {'H2': 124.43, 'HE': 35.832, 'H2S': 2247.0, 'NH3': 2700.0,
                'CH4': 413.0}   # H2O is temperature dependent, see below

# Maxima of the real catalogue intensities that "relative" synthetic
# intensities are scaled by (constituents/nh3/ammonia.npz Io, Io_rot;
# constituents/nh3/nh3.npz I0; constituents/h2s/h2s.npz I0;
# constituents/h2o/h2o_bk.py built-in I_o).
IMAX = dict(nh3_inv=6.4830489e-23, nh3_rot=4.6395867e-19, nh3_sjs=2.0686e-19,
            h2s=6.7497e-20, h2o=0.1535e-08)

MHZ_PER_TORR_TO_GHZ_PER_BAR = 0.750
HC_OVER_K = 1.4387769        # K cm, converts E'' [cm^-1] to the h2o_bk E_o

MIXING = dict(H2=0.86, HE=0.136, CH4=2.0e-3, NH3=3.0e-4, H2O=1.0e-3,
              H2S=7.0e-5, PH3=6.0e-7)


# ---------------------------------------------------------------- atmosphere
def h2o_saturation_pressure(T):
    """H2O vapour pressure [bar] over ice / water (Briggs and Sackett form,
    the same coefficients the reference uses in radiobear/chemistry.py:93-112;
    ice below the 273.16 K triple point)."""
    T = np.asarray(T, dtype=np.float64)
    ice = (-5631.1206, -22.1791, 8.2312, -3.861449e-2, 2.77494e-5)
    liq = (-2313.0338, -177.848, 38.053682, -0.13844344, 7.4465367e-5)
    out = np.empty_like(T)
    for mask, a in ((T < 273.16, ice), (T >= 273.16, liq)):
        t = T[mask]
        out[mask] = np.exp(a[0] / t + a[1] + a[2] * np.log(t) + a[3] * t + a[4] * t * t)
    return out


def temperature_profile(P, T1bar=110.0, T_cap=165.0, P_cap=0.1, dT_deep=0.0):
    """Dry adiabat through ``T1bar`` at 1 bar (R/cp of the H2/He/CH4 mix),
    isothermal ``T_cap`` at P < ``P_cap``.  ``dT_deep`` shifts the adiabat."""
    cp = (MIXING['H2'] * CP_OVER_R['H2'] + MIXING['HE'] * CP_OVER_R['HE']
          + MIXING['CH4'] * CP_OVER_R['CH4']) / (MIXING['H2'] + MIXING['HE'] + MIXING['CH4'])
    kappa = 1.0 / cp
    T = (T1bar + dT_deep) * np.power(P, kappa)
    return np.where(P < P_cap, T_cap, T)


def make_gas_table(nL, Pmin, Pmax, nh3_deep=MIXING['NH3'], dT_deep=0.0,
                   mu=2.3e-3, g=24.79):
    """Gas table [len(GAS_COLUMNS), nL] of the Jupiter-like recipe.

    z comes from hydrostatic integration (trapezoid in ln P, scale height
    R T / (mu g)), with the deepest layer at z = 0 km.
    """
    P = np.logspace(np.log10(Pmin), np.log10(Pmax), nL)
    T = temperature_profile(P, dT_deep=dT_deep)
    H = R_GAS * T / (mu * g) / 1000.0                       # km
    lnP = np.log(P)
    dz = 0.5 * (H[1:] + H[:-1]) * (lnP[1:] - lnP[:-1])      # >0 going down
    z = np.concatenate([np.cumsum(dz[::-1])[::-1], [0.0]])
    gas = np.zeros((len(GAS_COLUMNS), nL))
    C = {k: i for i, k in enumerate(GAS_COLUMNS)}
    gas[C['Z']] = z
    gas[C['T']] = T
    gas[C['P']] = P
    gas[C['H2']] = MIXING['H2']
    gas[C['HE']] = MIXING['HE']
    gas[C['CH4']] = MIXING['CH4']
    gas[C['NH3']] = np.where(P >= 1.0, nh3_deep, nh3_deep * P * P)
    gas[C['H2O']] = np.minimum(MIXING['H2O'], h2o_saturation_pressure(T) / P)
    gas[C['H2S']] = MIXING['H2S']
    gas[C['PH3']] = MIXING['PH3']
    dzcm = np.abs(np.diff(gas[C['Z']])) * 1.0e5
    gas[C['DZ']] = np.concatenate([[0.0], dzcm])
    return gas


def compute_properties(gas, Req=JUPITER['Req'], p_ref=JUPITER['p_ref'],
                       GM_ref=JUPITER['GM_ref']):
    """Property table [len(PROPERTY_COLUMNS), nL]: restates
    ``AtmosphereBase.computeProp`` (radiobear/atm_base.py:120-194)."""
    C = {k: i for i, k in enumerate(GAS_COLUMNS)}
    LP = {k: i for i, k in enumerate(PROPERTY_COLUMNS)}
    P = gas[C['P']]
    T = gas[C['T']]
    z = gas[C['Z']]
    nL = len(P)
    chem_keys = [k for k in GAS_COLUMNS if k not in ('P', 'T', 'Z', 'DZ')]
    iOffset = int(np.argmin(np.abs(P - p_ref)))
    rr = Req + z - z[iOffset]
    amu = np.zeros(nL)
    refr = np.zeros(nL)
    for k in chem_keys:
        amu = amu + AMU.get(k, 0.0) * gas[C[k]]
        if k == 'H2O':
            refr = refr + (245.0 + 1.28e6 / T) * gas[C[k]]
        else:
            refr = refr + REFRACTIVITY.get(k, 0.0) * gas[C[k]]
    refr = refr * P * (293.0 / T)
    prop = np.zeros((len(PROPERTY_COLUMNS), nL))
    prop[LP['P']] = P
    prop[LP['Z']] = z
    prop[LP['R']] = rr
    prop[LP['AMU']] = amu
    prop[LP['REFR']] = refr
    prop[LP['N']] = refr / 1.0e6 + 1.0
    gm = np.zeros(nL)
    lapse = np.zeros(nL)
    lapsep = np.zeros(nL)
    if nL > 1:
        rho = (amu[1:] * P[1:]) / (R_GAS * T[1:])
        dr = np.abs(z[1:] - z[:-1])
        dM = 1.0e11 * rho * 4.0 * np.pi * rr[1:] ** 2 * dr
        gm[1:] = np.cumsum(GRAV_CONST * dM)
        lapse[1:] = np.abs(T[1:] - T[:-1]) / dr
        lapsep[1:] = np.abs(T[1:] - T[:-1]) / np.abs(P[1:] - P[:-1])
    gm = GM_ref - (gm - gm[iOffset])
    little_g = gm / rr ** 2
    prop[LP['GM']] = gm
    prop[LP['LAPSE']] = lapse
    prop[LP['LAPSEP']] = lapsep
    prop[LP['g']] = little_g
    prop[LP['H']] = (R_GAS * T) / (little_g * amu) / 1000.0
    return prop


# ---------------------------------------------------------------- line lists
def _loguniform(rng, lo, hi, n):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def _centres_nh3_like(rng, n):
    n_lo = (3 * n) // 4
    return (rng.uniform(18.0, 26.0, n_lo), _loguniform(rng, 500.0, 1500.0, n - n_lo))


def make_nh3_lines(rng, n):
    """NH3 list in both reference schemas.

    Returns ``(ammonia, nh3)``: ``ammonia`` has the ``nh3_hs`` keys of
    ``ammonia.npz`` (inversion lines = the 18-26 GHz centres, rotational lines
    = the 500-1500 GHz centres with per-line H2/He/self widths, no nu2 lines);
    ``nh3`` is the same list in the ``nh3_sjs`` ``f0 I0 E G0`` schema.
    Per-line temperature exponents are drawn (to keep the draw sequence of
    the recipe) but no NH3 formalism of the reference has a slot for them.
    """
    f_inv, f_rot = _centres_nh3_like(rng, n)
    n_inv = len(f_inv)
    i_rel = 10.0 ** rng.uniform(-6.0, -1.0, n)
    e_low = rng.uniform(0.0, 2000.0, n)
    w = rng.uniform(1.5, 3.0, (3, n)) * MHZ_PER_TORR_TO_GHZ_PER_BAR   # H2, He, self
    rng.uniform(0.6, 0.9, (3, n))                                       # exponents (unused)
    inv, rot = slice(0, n_inv), slice(n_inv, n)
    ammonia = dict(
        fo=f_inv, Io=i_rel[inv] * IMAX['nh3_inv'], Eo=e_low[inv],
        gammaNH3o=w[2, inv], H2HeBroad=w[0, inv],
        fo_rot=f_rot, Io_rot=i_rel[rot] * IMAX['nh3_rot'], Eo_rot=e_low[rot],
        gNH3_rot=w[2, rot], gH2_rot=w[0, rot], gHe_rot=w[1, rot],
        fo_v2=np.zeros(0), Io_v2=np.zeros(0), Eo_v2=np.zeros(0))
    nh3 = dict(f0=np.concatenate([f_inv, f_rot]), I0=i_rel * IMAX['nh3_sjs'],
               E=e_low.copy(), G0=w[2].copy())
    return ammonia, nh3


def make_h2o_lines(rng, n):
    """H2O list in the ``h2o_bk`` dictionary schema (centres log-uniform
    20-1000 GHz; E_o is E''*hc/k/300 as in constituents/h2o/h2o_bk.py:31)."""
    f = _loguniform(rng, 20.0, 1000.0, n)
    i_rel = 10.0 ** rng.uniform(-6.0, -1.0, n)
    e_low = rng.uniform(0.0, 2000.0, n)
    w = rng.uniform(1.5, 3.0, (3, n)) * MHZ_PER_TORR_TO_GHZ_PER_BAR   # H2, He, self
    x = rng.uniform(0.6, 0.9, (3, n))
    return dict(f_o=f, I_o=i_rel * IMAX['h2o'], E_o=e_low * HC_OVER_K / 300.0,
                w_s=w[2], x_s=x[2], w_h2=w[0], w_he=w[1], x_h2=x[0], x_he=x[1],
                SR=np.zeros(n))


def make_h2s_lines(rng, n):
    """H2S list in the ``f0 I0 E GH2S`` schema of ``h2s.npz``."""
    f_lo, f_hi = _centres_nh3_like(rng, n)
    i_rel = 10.0 ** rng.uniform(-6.0, -1.0, n)
    e_low = rng.uniform(0.0, 2000.0, n)
    w = rng.uniform(1.5, 3.0, n) * MHZ_PER_TORR_TO_GHZ_PER_BAR
    return dict(f0=np.concatenate([f_lo, f_hi]), I0=i_rel * IMAX['h2s'], E=e_low, GH2S=w)


# ---------------------------------------------------------------- rays
def gauss_legendre_disc(n):
    """Equatorial impact parameters and weights of an n-point Gauss-Legendre
    disc average: Tb_disc = sum_k w_k Tb(b_k), b_k = sqrt(1 - mu_k^2),
    w_k = 2 mu_k x (GL weight on mu in [0, 1]); sum_k w_k = 1."""
    x, w = np.polynomial.legendre.leggauss(n)
    mu = 0.5 * (x + 1.0)
    wk = 0.5 * w * 2.0 * mu
    b = np.stack([np.sqrt(1.0 - mu * mu), np.zeros(n)], axis=1)
    return b, wk


def image_grid(n=256, spacing=0.01):
    """n x n grid of impact parameters, spacing in units of rNorm, centred."""
    v = (np.arange(n) - n // 2) * spacing
    bx, by = np.meshgrid(v, v, indexing='xy')
    return np.stack([bx.ravel(), by.ravel()], axis=1)


def freq_string(srq):
    """'start:stop:step' with the stop-inclusive rule of
    radiobear/set_utils.py:132-138."""
    start, stop, step = [float(x) for x in srq.split(':')]
    return np.arange(start, stop + step / 2.0, step)


# ---------------------------------------------------------------- workloads
class Workload(dict):
    """Attribute-access dict holding one synthetic workload."""

    __getattr__ = dict.__getitem__


def make_workload(config, real=None):
    """Build configuration ``config`` (0..3) of the benchmark suite.

    ``real`` is the dictionary of real catalogue extracts (``ph3``, ``ph3wgt``,
    ``h2s``, ``h2o``) used where the recipe calls for the shipped catalogue.
    """
    rng = np.random.default_rng(config)
    if config == 0:
        gas = make_gas_table(200, 1.0e-3, 100.0)
        ammonia, nh3 = make_nh3_lines(rng, 200)
        lines = dict(ammonia=ammonia, nh3=nh3)
        if real is not None:
            lines.update(h2o=real['h2o'], h2s=real['h2s'], ph3=real['ph3'])
        freqs = freq_string('1:100:5')
        b = np.array([[0.0, 0.0]])
        w = np.ones(1)
    else:
        gas = make_gas_table(1000, 1.0e-3, 500.0)
        ammonia, nh3 = make_nh3_lines(rng, 2000)
        h2o = make_h2o_lines(rng, 500)
        h2s = make_h2s_lines(rng, 200)
        lines = dict(ammonia=ammonia, nh3=nh3, h2o=h2o, h2s=h2s)
        if real is not None:
            lines.update(ph3=real['ph3'])
        if config == 1:
            freqs = np.logspace(np.log10(0.5), np.log10(100.0), 256)
            b, w = gauss_legendre_disc(64)
        elif config == 2:
            freqs = np.array([1.4, 3.0, 6.0, 10.0, 15.0, 22.0, 33.0, 44.0])
            b = image_grid(256, 0.01)
            w = np.full(len(b), 1.0 / len(b))
        elif config == 3:
            freqs = np.logspace(0.0, np.log10(50.0), 64)
            b, w = gauss_legendre_disc(16)
        else:
            raise ValueError('config must be 0..3 (use make_variants for 4)')
    prop = compute_properties(gas)
    return Workload(config=config, gas=gas, prop=prop, lines=lines, freqs=freqs,
                    b=b, weights=w, planet=dict(JUPITER))


def make_variants(n_variants=4096, seed=4, nL_range=(300, 1200)):
    """Configuration 4: per-variant (nL, deep NH3, deep dT) draws."""
    rng = np.random.default_rng(seed)
    nL = rng.integers(nL_range[0], nL_range[1] + 1, n_variants)
    nh3 = np.exp(rng.uniform(np.log(1.0e-4), np.log(1.0e-3), n_variants))
    dT = rng.uniform(-10.0, 10.0, n_variants)
    return nL, nh3, dT
