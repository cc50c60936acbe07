"""CPU oracle: float64 numpy restatement of radioBEAR's forward-model path.

TEST INFRASTRUCTURE ONLY.  This module is the checker for the GPU path.  Only
``tests/``, ``__graft_entry__.smoke()`` and the ``cpu_baseline`` /
``--impl reference`` legs of ``bench.py`` may import it; the
``radiobear_gb300`` package never does, and it is never the thing measured
as the GPU result.

Pinning: this restatement is checked against (1) the expected brightness
table hard-coded in the reference's ``scripts/benchmark.py:20-24`` (the one
golden vector the reference ships) and (2) fixtures produced by running the
unmodified reference on the same inputs (``tests/golden/make_golden.py``):
per-gas alpha, ray paths (including tangent/egress limb rays) and Tb.

Each function cites the reference lines it restates (paths relative to the
reference project root).  Arrays are vectorised over layers and frequencies;
the arithmetic follows the reference expression by expression so the
results agree to ~1e-12 relative.
"""
from __future__ import annotations

import math

import numpy as np

T_CMB = 2.725                       # radiobear/utils.py:77
F_SPLIT = 30.0                      # constituents/nh3/nh3_hs.py:58
GHZ_TO_INV_CM = 1.0 / 29.9792458    # constituents/nh3/nh3_hs.py:44
DB_PER_INVCM = 434294.5

# nh3_hs constants, constituents/nh3/nh3_hs.py:44-56
_HS_HC = 19.858252418E-24
_HS_KB = 1.38E-23
_HS_NO = 6.02297E23
_HS_R = 8.31432E7
_HS_TO = 300.0
_HS_COEF = 1.0E6 * _HS_NO / _HS_R

# Inversion coefficient sets, f <= 30 GHz and f > 30 GHz
# (constituents/nh3/nh3_hs.py:139-168): gnu_H2, gnu_He, gnu_NH3, GAMMA_H2,
# GAMMA_He, GAMMA_NH3, zeta_H2, zeta_He, zeta_NH3, Z_H2, Z_He, Z_NH3, d, Con
HS_INV_LO = (1.640, 0.75, 0.852, 0.7756, 0.666, 1.0, 1.262, 0.3, 0.5296, 0.7964,
             0.667, 1.554, -0.0498, 0.9301)
HS_INV_HI = (1.7465, 0.9779, 0.7298, 0.8202, 1.0, 1.0, 1.2163, 0.0291, 0.5152,
             0.8873, 0.8994, 2.0 / 3.0, -0.0627, 0.9862)
# nh3_dbs inversion coefficients (constituents/nh3/nh3_dbs.py:133-162): its
# own f <= 30 GHz set, the f > 30 GHz set equal to nh3_hs's
DBS_INV_LO = (1.6937, 0.6997, 0.7523, 0.8085, 1.0, 1.0, 1.3263, 0.1607, 0.6162, 0.8199,
              0.0, 1.3832, -0.0139, 0.9619)
DBS_INV_HI = HS_INV_HI
# Rotational / nu2 (Gross) constants, constituents/nh3/nh3_hs.py:234-243,272-280
HS_ROT = dict(eta=(0.8730, 2.0 / 3.0, 1.0), gnu=(0.2984, 0.75, 3.1789), con=2.4268)
HS_V2 = dict(eta=(0.73, 0.5716, 1.0), width=(1.4, 0.68, 9.5), con=1.1206)

# BR formalisms sharing the GEISA constants (nh3_sjs.py:6-12, h2s_ddb.py:6-9,
# ph3_jh.py:7-10)
GEISA_COEF = 7.244E+21
HCK = 1.438396
GHZ = 29.9792458


def _pow(a, b):
    return np.power(a, b)


# ---------------------------------------------------------------- nh3_hs
def _ben_reuven_hs(f, fo, gamma, zeta, delt):
    """Ben-Reuven shape of nh3_hs.py:193-226 (in GHz, before the /GHztoinv_cm).

    Shapes: f [..., 1, nf]; line arrays [..., nlines, 1]."""
    f2 = np.square(f)
    Aa = (2.0 / np.pi) * np.square(f / fo)
    Bb = (gamma - zeta) * f2
    Cc = gamma + zeta
    Dd = np.square(fo + delt) + np.square(gamma) - np.square(zeta)
    Ee = f2
    Jj = np.square(fo + delt)
    Gg = np.square(gamma)
    Hh = np.square(zeta)
    Ii = 4.0 * f2 * np.square(gamma)
    return Aa * (Bb + Cc * Dd) / (np.square(Ee - Jj - Gg + Hh) + Ii)


def _gross(f, fo, gamma):
    """Gross shape of nh3_hs.py:259-263 / 296-300."""
    f2 = np.square(f)
    Aa = (4.0 / np.pi) * f2 * gamma
    Bb = np.square(np.square(fo) - f2)
    Cc = 4.0 * f2 * np.square(gamma)
    return Aa / (Bb + Cc)


def _nh3_hs_block(freq, T, P, Ph2, Phe, Pnh3, cat, coefs):
    """One homogeneous frequency block of nh3_hs.__alpha__ (nh3_hs.py:91-314),
    vectorised over layers.  T, P, ... are [nL]; freq [nf].  Returns [nL, nf]."""
    (gnu_H2, gnu_He, gnu_NH3, G_H2, G_He, G_NH3, z_H2, z_He, z_NH3, Z_H2, Z_He, Z_NH3,
     d, Con) = coefs
    T = T[:, None, None]
    Ph2 = Ph2[:, None, None]
    Phe = Phe[:, None, None]
    Pnh3 = Pnh3[:, None, None]
    f = np.asarray(freq, dtype=np.float64)[None, None, :]
    Tdiv = _HS_TO / T
    eta = 1.5
    # inversion lines (nh3_hs.py:172-229)
    fo = cat['fo'][None, :, None]
    gNo = cat['gammaNH3o'][None, :, None]
    gamma = (gnu_H2 * Ph2) * Tdiv ** G_H2 + (gnu_He * Phe) * Tdiv ** G_He \
        + (gnu_NH3 * Pnh3 * gNo) * (295.0 / T) ** G_NH3
    delt = d * gamma
    zeta = (z_H2 * Ph2) * Tdiv ** Z_H2 + (z_He * Phe) * Tdiv ** Z_He \
        + (z_NH3 * Pnh3 * gNo) * (295.0 / T) ** Z_NH3
    expo = -(1.0 / T - 1.0 / _HS_TO) * cat['Eo'][None, :, None] * _HS_HC / _HS_KB
    ST = cat['Io'][None, :, None] * np.exp(expo)
    noshape = Con * _HS_COEF * (Pnh3 / _HS_TO) * np.power(_HS_TO / T, eta + 2.0) * ST
    Ff = _ben_reuven_hs(f, fo, gamma, zeta, delt)
    a_inv = np.sum(noshape * ((1.0 / GHZ_TO_INV_CM) * Ff), axis=1)
    # rotational lines (nh3_hs.py:232-265)
    a_rot = 0.0
    if cat['fo_rot'].size:
        fo = cat['fo_rot'][None, :, None]
        ST = cat['Io_rot'][None, :, None] * np.exp((1.0 / _HS_TO - 1.0 / T) * cat['Eo_rot'][None, :, None] * _HS_HC / _HS_KB)
        eH2, eHe, eNH3 = HS_ROT['eta']
        nH2, nHe, nNH3 = HS_ROT['gnu']
        gamma = (nH2 * Ph2 * cat['gH2_rot'][None, :, None]) * Tdiv ** eH2 \
            + (nHe * Phe * cat['gHe_rot'][None, :, None]) * Tdiv ** eHe \
            + (nNH3 * Pnh3 * cat['gNH3_rot'][None, :, None]) * Tdiv ** eNH3
        F = _gross(f, fo, gamma)
        a_rot = np.sum(HS_ROT['con'] * _HS_COEF * (Pnh3 / _HS_TO) * ((_HS_TO / T) ** (eta + 2.0)) * ST
                       * ((1.0 / GHZ_TO_INV_CM) * F), axis=1)
    # nu2 roto-vibrational lines (nh3_hs.py:269-302)
    a_v2 = 0.0
    if cat['fo_v2'].size:
        fo = cat['fo_v2'][None, :, None]
        ST = cat['Io_v2'][None, :, None] * np.exp((1.0 / _HS_TO - 1.0 / T) * cat['Eo_v2'][None, :, None] * _HS_HC / _HS_KB)
        eH2, eHe, eNH3 = HS_V2['eta']
        wH2, wHe, wNH3 = HS_V2['width']
        gamma = (Ph2 * wH2) * Tdiv ** eH2 + (Phe * wHe) * Tdiv ** eHe + (Pnh3 * wNH3) * Tdiv ** eNH3
        F = _gross(f, fo, gamma)
        a_v2 = np.sum(HS_V2['con'] * _HS_COEF * (Pnh3 / _HS_TO) * ((_HS_TO / T) ** (eta + 2.0)) * ST
                      * ((1.0 / GHZ_TO_INV_CM) * F), axis=1)
    a = a_inv + a_rot + a_v2
    return np.where(a < 0.0, 1.0e-8, a)       # nh3_hs.py:311-312


def alpha_nh3_hs(freq, T, P, Xh2, Xhe, Xnh3, cat, tables=(HS_INV_LO, HS_INV_HI)):
    """nh3_hs.alpha (nh3_hs.py:70-88): the <=30 GHz block then the >30 GHz
    block, concatenated in that order (output slot k holds the k-th value of
    that concatenation, whatever the input order).  Returns [nL, nf].
    nh3_dbs (nh3_dbs.py:26-313) is the same computation with the
    DBS_INV_* tables (its H2HeBroad column is not read by either)."""
    freq = np.asarray(freq, dtype=np.float64)
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    P = np.atleast_1d(np.asarray(P, dtype=np.float64))
    Ph2, Phe, Pnh3 = P * Xh2, P * Xhe, P * Xnh3
    parts = []
    lo = freq[freq <= F_SPLIT]
    hi = freq[freq > F_SPLIT]
    if lo.size:
        parts.append(_nh3_hs_block(lo, T, P, Ph2, Phe, Pnh3, cat, tables[0]))
    if hi.size:
        parts.append(_nh3_hs_block(hi, T, P, Ph2, Phe, Pnh3, cat, tables[1]))
    return np.concatenate(parts, axis=1)


def alpha_nh3_dbs(freq, T, P, Xh2, Xhe, Xnh3, cat):
    """nh3_dbs.alpha (nh3_dbs.py:26-44, __alpha__ 47-313)."""
    return alpha_nh3_hs(freq, T, P, Xh2, Xhe, Xnh3, cat, tables=(DBS_INV_LO, DBS_INV_HI))


# ---------------------------------------------------------------- nh3_sjs
def _sjs_coefficients(T, P, Ph2):
    """Joiner / Spilker coefficient sets of nh3_sjs.py:42-77 for each layer.
    Returns dict name -> (joiner [nL], spilker [nL])."""
    rexp = 8.79 * np.exp(-T / 83.0)
    base = np.exp(9.024 - T / 20.3) - 0.9918 + Ph2
    with np.errstate(invalid='ignore'):
        GH2a = np.power(base, rexp)
    joiner_always = GH2a < 1e-12          # NaN compares False, like the reference
    GH2s = 2.122 * np.exp(-T / 116.8) / GH2a
    GH2s = 2.34 * (1.0 - GH2s)
    one = np.ones_like(T)
    spil = dict(GH2=GH2s, GHe=0.46 + T / 3000.0, GNH3=0.74 * one,
                ZH2=5.7465 - 7.7644 * GH2s + 9.1931 * GH2s ** 2 - 5.6816 * GH2s ** 3 + 1.2307 * GH2s ** 4,
                ZHe=0.28 - T / 1750.0, ZNH3=0.50 * one, D=-0.45 * one)
    join = dict(GH2=1.690 * one, GHe=0.750 * one, GNH3=0.6 * one, ZH2=1.350 * one,
                ZHe=0.300 * one, ZNH3=0.200 * one, D=-0.45 * one)
    for k in spil:
        spil[k] = np.where(joiner_always, join[k], spil[k])
    return join, spil


def alpha_nh3_sjs(freq, T, P, Xh2, Xhe, Xnh3, cat):
    """nh3_sjs.alpha (nh3_sjs.py:26-128), vectorised over layers.  [nL, nf]"""
    freq = np.asarray(freq, dtype=np.float64)
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    P = np.atleast_1d(np.asarray(P, dtype=np.float64))
    Ph2, Phe, Pnh3 = P * Xh2, P * Xhe, P * Xnh3
    Pscale = 1.0 + P / 1.0E5
    join, spil = _sjs_coefficients(T, P, Ph2)
    T0 = 296.0
    fLower, fHigher = 26.0, 34.0
    f0 = cat['f0'][None, :]
    G0 = cat['G0'][None, :]
    ITG = cat['I0'][None, :] * np.exp(-((1.0 / T[:, None]) - (1.0 / T0)) * cat['E'][None, :] * HCK)
    out = np.empty((T.size, freq.size))
    tt = np.power(T0 / T, 2.0 / 3.0)[:, None]
    for j, f in enumerate(freq):
        f2 = f ** 2
        if f <= fLower:
            c = spil
        elif f >= fHigher:
            c = join
        else:
            flfh = (fLower - fHigher) / (f - fLower)
            c = {k: spil[k] + (spil[k] - join[k]) / flfh for k in spil}
        delta = (c['D'] * Pnh3)[:, None]
        gamma = tt * ((c['GH2'] * Ph2)[:, None] + (c['GHe'] * Phe)[:, None] + G0 * (c['GNH3'] * Pnh3)[:, None])
        zeta = tt * ((c['ZH2'] * Ph2)[:, None] + (c['ZHe'] * Phe)[:, None] + G0 * (c['ZNH3'] * Pnh3)[:, None])
        g2, z2 = gamma ** 2, zeta ** 2
        num = (gamma - zeta) * f2 + (gamma + zeta) * (np.power(f0 + delta, 2.0) + g2 - z2)
        den = np.power((f2 - np.power(f0 + delta, 2.0) - g2 + z2), 2.0) + 4.0 * f2 * g2
        shape = GHZ * 2.0 * np.power(f / f0, 2.0) * num / (np.pi * den)
        out[:, j] = np.sum(shape * ITG, axis=1)
    return GEISA_COEF * (Pnh3 / T0)[:, None] * np.power(T0 / T, 1.5 + 2)[:, None] * out * Pscale[:, None]


def alpha_nh3_hs_sjs(freq, T, P, Xh2, Xhe, Xnh3, cat_hs, cat_sjs, hs=None):
    """nh3_hs_sjs.alpha (nh3_hs_sjs.py:6-26): hs below 400 bar, sjs above
    2000 bar, linear blend W=(P-400)/1600 in between.  nh3_dbs_sjs
    (nh3_dbs_sjs.py:6-26) is the same blend of nh3_dbs (``hs``)."""
    hs = hs or alpha_nh3_hs
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    P = np.atleast_1d(np.asarray(P, dtype=np.float64))
    Xh2, Xhe, Xnh3 = (np.broadcast_to(np.asarray(x, dtype=np.float64), P.shape) for x in (Xh2, Xhe, Xnh3))
    out = np.empty((P.size, len(freq)))
    lo = P < 400.0
    hi = P > 2000.0
    mid = ~(lo | hi)
    if lo.any():
        out[lo] = hs(freq, T[lo], P[lo], Xh2[lo], Xhe[lo], Xnh3[lo], cat_hs)
    if hi.any():
        out[hi] = alpha_nh3_sjs(freq, T[hi], P[hi], Xh2[hi], Xhe[hi], Xnh3[hi], cat_sjs)
    if mid.any():
        a2 = alpha_nh3_sjs(freq, T[mid], P[mid], Xh2[mid], Xhe[mid], Xnh3[mid], cat_sjs)
        a1 = hs(freq, T[mid], P[mid], Xh2[mid], Xhe[mid], Xnh3[mid], cat_hs)
        W = ((P[mid] - 400.0) / (2000.0 - 400.0))[:, None]
        out[mid] = W * a2 + (1.0 - W) * a1
    return out


def alpha_nh3_dbs_sjs(freq, T, P, Xh2, Xhe, Xnh3, cat_hs, cat_sjs):
    """nh3_dbs_sjs.alpha (nh3_dbs_sjs.py:6-26)."""
    return alpha_nh3_hs_sjs(freq, T, P, Xh2, Xhe, Xnh3, cat_hs, cat_sjs, hs=alpha_nh3_dbs)


# ---------------------------------------------------------------- co_ddb
# Hui, Armstrong & Wray (1978) rational approximation of the complex
# probability function, coefficients of co_ddb.py:25-28
VOIGT_A = (122.60793178, 214.38238869, 181.92853309, 93.15558046, 30.18014220,
           5.91262621, 0.56418958, 0.0)
VOIGT_B = (122.60793178, 352.73062511, 457.33447878, 348.70391772, 170.35400182,
           53.99290691, 10.47985711, 1.0)


def alpha_co_ddb(freq, T, P, Xh2, Xhe, Xco, cat, coshape='voigt'):
    """co_ddb.alpha (co_ddb.py:22-99) for each layer.  ``coshape`` is
    other_dict['coshape'] ('voigt' when absent); 'voigt', 'vvw' and 'diff'
    sum unweighted shapes, anything else the pressure blend times the line
    strengths.  Returns [nL, nf] cm^-1."""
    freq = np.asarray(freq, dtype=np.float64)
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    P = np.atleast_1d(np.asarray(P, dtype=np.float64))
    Xh2, Xhe, Xco = (np.broadcast_to(np.asarray(x, dtype=np.float64), P.shape) for x in (Xh2, Xhe, Xco))
    f0, I0, E = (np.asarray(cat[k], dtype=np.float64) for k in ('f0', 'I0', 'E'))
    T0, hck = 296.0, HCK
    out = np.empty((P.size, freq.size))
    for i in range(P.size):
        Ph2, Phe, Pco = P[i] * Xh2[i], P[i] * Xhe[i], P[i] * Xco[i]
        gamma = pow(T0 / T[i], 0.7) * (1.960 * Ph2 + 1.200 * Phe + 6.000 * Pco)
        g2 = gamma ** 2
        ITG = I0 * np.exp(-((1.0 / T[i]) - (1.0 / T0)) * E * hck)
        w = min(max((P[i] - 0.001) / (0.1 - 0.001), 0.0), 1.0)
        for j, f in enumerate(freq):
            f2 = f ** 2
            sV = np.zeros(f0.size)
            if P[i] <= 0.1 or coshape in ('voigt', 'diff'):
                betaD = 4.3e-7 * np.sqrt(T[i] / 28.0) * f
                xi = gamma / betaD + 1j * (f - f0) / betaD
                num = np.zeros(f0.size, dtype=np.complex128)
                den = np.zeros(f0.size, dtype=np.complex128)
                for k in range(8):
                    num += VOIGT_A[k] * xi ** k
                    den += VOIGT_B[k] * xi ** k
                sV = GHZ * (1.0 / (np.sqrt(np.pi) * betaD)) * (num / den).real
            sW = np.zeros(f0.size)
            if P[i] >= 0.001 or coshape in ('vvw', 'diff'):
                num = gamma * f2 + gamma * (f0 ** 2 + g2)
                den = (f2 - f0 ** 2 - g2) ** 2 + 4.0 * f2 * g2
                sW = GHZ * 2.0 * (f / f0) ** 2 * num / (np.pi * den)
            if coshape == 'voigt':
                out[i, j] = np.sum(sV)
            elif coshape == 'vvw':
                out[i, j] = np.sum(sW)
            elif coshape == 'diff':
                out[i, j] = np.sum(sV - sW)
            else:
                out[i, j] = np.sum((w * sW + (1.0 - w) * sV) * ITG)
        out[i] *= GEISA_COEF * (Pco / T0) * pow(T0 / T[i], 3.5)
    return out


# ---------------------------------------------------------------- clouds_idp
_ICE_FR = (1.0E8, 3.0E8, 1.0E9, 2.0E9, 3.0E9, 5.0E9, 1.0E10, 3.0E10, 1.0E11)
_ICE_EIMAG = (8.0E-3, 1.5E-3, 8.0E-4, 1.0E-3, 1.2E-3, 1.5E-3, 3.0E-3, 8.0E-3, 2.0E-2)


def water_dielectric(f, T):
    """clouds_idp.water (clouds_idp.py:75-101): complex e of water above
    0 C (Debye), ice below (log-log table of Im e)."""
    Tc = T - 273.0
    fHz = f * 1.0E9
    if Tc >= 0.0:
        RelT = 1.1109E-10 - Tc * 3.824E-12 + Tc ** 2 * 6.938E-14 - Tc ** 3 * 5.096E-16
        E0 = max(88.045 - 0.4147 * Tc + Tc ** 2 * 6.295E-4 + Tc ** 3 * 1.075E-5, 0.0)
        EINF = 4.9
        E1 = EINF + (E0 - EINF) / (1.0 + (fHz * RelT) ** 2)
        E2 = max(fHz * RelT * (E0 - EINF) / (1.0 + (fHz * RelT) ** 2), 0.0)
    else:
        E1 = 3.17
        LF = math.log10(fHz)
        for j in range(len(_ICE_FR) - 1):
            if _ICE_FR[j + 1] >= fHz:
                break
        LF0, LF1 = math.log10(_ICE_FR[j]), math.log10(_ICE_FR[j + 1])
        DLF = (LF - LF0) / (LF1 - LF0)
        X0, X1 = math.log10(_ICE_EIMAG[j]), math.log10(_ICE_EIMAG[j + 1])
        E2 = 10.0 ** (X0 + DLF * (X1 - X0))
    return E1 - E2 * 1j


def _acloud(k, fraction, e):
    K = (e - 1.0) / (e + 2.0)                  # clouds_idp.py:64-68
    return 3.0 * k * fraction * (-K.imag)


# (other_dict key, cloud column, density divisor, refractive index or None
# for the water dielectric), in the order of clouds_idp.py:16-49
CLOUD_KINDS = (('ice_p', 'H2O', 0.9, None), ('water_p', 'SOLN', 1.0, None),
               ('nh4sh_p', 'NH4SH', 1.2, 1.7 - 0.005j), ('nh3ice_p', 'NH3', 1.6, 1.3 - 0.0001j),
               ('h2sice_p', 'H2S', 1.5, 1.15 - 0.0001j), ('ch4', 'CH4', 1.0, 1.3 - 0.00001j))


def alpha_clouds_idp(freq, T, cloud, Cl, other_dict):
    """clouds_idp.alpha (clouds_idp.py:6-61) for each layer: T [nL], cloud
    table [ncol, nL] indexed by Cl.  Returns [nL, nf] cm^-1."""
    freq = np.asarray(freq, dtype=np.float64)
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    out = np.zeros((T.size, freq.size))
    for i in range(T.size):
        for j, f in enumerate(freq):
            a = 0.0
            k = 2.0 * np.pi * f / GHZ
            for key, col, div, n in CLOUD_KINDS:
                if key in other_dict and other_dict[key] > 0.0:
                    e = water_dielectric(f, T[i]) if n is None else n ** 2
                    a += _acloud(k, cloud[Cl[col]][i] / div, e)
            out[i, j] = max(a, 0.0)
    return out


# ---------------------------------------------------------------- h2o_bk
def alpha_h2o_bk(freq, T, P, Xh2, Xhe, Xh2o, cat):
    """h2o_bk.alpha + vvwlinecontribution_modified (h2o_bk.py:65-189), in
    cm^-1.  [nL, nf]"""
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))[:, None, None]
    P = np.atleast_1d(np.asarray(P, dtype=np.float64))[:, None, None]
    Ph2 = P * np.asarray(Xh2, dtype=np.float64).reshape(-1, 1, 1)
    Phe = P * np.asarray(Xhe, dtype=np.float64).reshape(-1, 1, 1)
    Ph2o = P * np.asarray(Xh2o, dtype=np.float64).reshape(-1, 1, 1)
    f = np.asarray(freq, dtype=np.float64)[None, None, :]
    Theta = 300.0 / T
    M_amu = 8.314472 / 0.46151805
    density = (M_amu * Ph2o) / (8.314472e-5 * T)
    density = 0.997317 * (density / M_amu) * 6.0221415e23 * (1.0 / 1e6)
    L = {k: np.asarray(v, dtype=np.float64)[None, :, None] for k, v in cat.items()}
    S = L['I_o'] * (Theta ** 2.5) * np.exp(L['E_o'] * (1.0 - Theta))
    df = L['w_s'] * Ph2o * np.power(Theta, L['x_s']) + L['w_h2'] * Ph2 * np.power(Theta, L['x_h2']) \
        + L['w_he'] * Phe * np.power(Theta, L['x_he'])
    base = df / (562500.0 + df ** 2)
    A = np.square(f / L['f_o']) / np.pi
    B = df / (np.square(f - L['f_o'] - L['SR']) + np.square(df))
    Cc = df / (np.square(f + L['f_o'] + L['SR']) + np.square(df))
    FSsum = np.sum(S * (A * (B - base + Cc - base)), axis=1)
    line = 4.342945 * 1e-4 * density[:, :, 0] * FSsum
    Cf_he = (1.0 / 0.001) ** 2 * 1.03562010226e-10
    Cf_h2 = (1.0 / 0.001) ** 2 * 5.07722009423e-11
    Th = Theta[:, :, 0]
    Cs1 = 3.1e-07 * np.power(Th, 12.0)
    f1 = f[:, 0, :]
    Ph2o1, Phe1, Ph21 = Ph2o[:, :, 0], Phe[:, :, 0], Ph2[:, :, 0]
    foreign = Cf_he * Phe1 * Ph2o1 * f1 ** 2 * np.power(Th, 3.0) + Cf_h2 * Ph21 * Ph2o1 * f1 ** 2 * np.power(Th, 3.0)
    selfc = Cs1 * ((Ph2o1 / 0.001) ** 2) * (f1 ** 2.0)
    a = line + 4.342945 * foreign + 4.342945 * selfc
    return a / DB_PER_INVCM


# ---------------------------------------------------------------- h2s / ph3
def _br_geisa(freq, f0, gamma, zeta, delta, ITG):
    """The Ben-Reuven line sum shared by nh3_sjs / h2s_ddb / ph3_jh
    (h2s_ddb.py:74-80, ph3_jh.py:95-101).  gamma etc. [nL, nlines]."""
    out = np.empty((gamma.shape[0], len(freq)))
    g2 = gamma ** 2
    z2 = zeta ** 2
    for j, f in enumerate(freq):
        f2 = f ** 2
        num = (gamma - zeta) * f2 + (gamma + zeta) * ((f0 + delta) ** 2 + g2 - z2)
        den = ((f2 - (f0 + delta) ** 2 - g2 + z2)) ** 2 + 4.0 * f2 * g2
        shape = GHZ * 2.0 * ((f / f0) ** 2) * num / (np.pi * den)
        out[:, j] = np.sum(shape * ITG, axis=1)
    return out


def alpha_h2s_ddb(freq, T, P, Xh2, Xhe, Xh2s, cat):
    """h2s_ddb.alpha (h2s_ddb.py:42-87).  [nL, nf]"""
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    P = np.atleast_1d(np.asarray(P, dtype=np.float64))
    Ph2, Phe, Ph2s = P * Xh2, P * Xhe, P * Xh2s
    T0 = 296.0
    delta = (1.28 * Ph2s)[:, None]
    gamma = np.power(T0 / T, 0.7)[:, None] * (1.960 * Ph2[:, None] + 1.200 * Phe[:, None]
                                              + cat['GH2S'][None, :] * Ph2s[:, None])
    ITG = cat['I0'][None, :] * np.exp(-((1.0 / T[:, None]) - (1.0 / T0)) * cat['E'][None, :] * HCK)
    s = _br_geisa(freq, cat['f0'][None, :], gamma, gamma, delta, ITG)
    return GEISA_COEF * (Ph2s / T0)[:, None] * np.power(T0 / T, 1.5 + 2)[:, None] * s


def alpha_ph3_jh(freq, T, P, Xh2, Xhe, Xph3, cat, wgt):
    """ph3_jh.alpha (ph3_jh.py:64-108).  [nL, nf]"""
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    P = np.atleast_1d(np.asarray(P, dtype=np.float64))
    Ph2, Phe, Pph3 = P * Xh2, P * Xhe, P * Xph3
    T0 = 300.0
    gamma = np.power(T0 / T, 2.0 / 3.0)[:, None] * (3.2930 * Ph2 + 1.6803 * Phe)[:, None] * wgt['WgtFGB'][None, :] \
        + np.power(T0 / T, 1.0)[:, None] * (4.2157 * Pph3)[:, None] * wgt['WgtSB'][None, :]
    ITG = cat['I0'][None, :] * wgt['WgtI0'][None, :] * np.exp(-((1.0 / T[:, None]) - (1.0 / T0)) * cat['E'][None, :] * HCK)
    zero = np.zeros((T.size, 1))
    s = _br_geisa(freq, cat['f0'][None, :], gamma, zero, zero, ITG)
    return GEISA_COEF * (Pph3 / T0)[:, None] * np.power(T0 / T, 1.5 + 2)[:, None] * s


# ---------------------------------------------------------------- h2 CIA
def alpha_h2_jj_ddb(freq, T, P, Xh2, Xhe, Xch4, h2state='e'):
    """h2_jj_ddb.alpha (h2_jj_ddb.py:7-38).  [nL, nf]"""
    T = np.atleast_1d(np.asarray(T, dtype=np.float64))
    P = np.atleast_1d(np.asarray(P, dtype=np.float64))
    Ph2, Phe, Pch4 = P * Xh2, P * Xhe, P * Xch4
    th = 273.0 / T
    if h2state == 'e':
        pre = np.minimum((T / 55.0) ** 2.7, 1.0)
        pre = np.minimum(pre * (T / 120.0) ** 0.55, 1.0)
    elif h2state == 'n':
        pre = np.minimum((T / 40.0) ** 2.5, 1.0)
    else:
        raise ValueError('invalid h2state')
    f2 = np.square(np.asarray(freq, dtype=np.float64))[None, :]
    cf = 3.9522E-14 * f2 * (Ph2 * pre)[:, None]
    return cf * (Ph2 * np.power(th, 3.12) + 1.382 * Phe * np.power(th, 2.24)
                 + 9.322 * Pch4 * np.power(th, 3.34))[:, None]


# ---------------------------------------------------------------- Alpha
GAS_FORMALISMS = ('h2', 'h2o', 'h2s', 'nh3', 'ph3')   # sorted, alpha.py:80


def alpha_per_gas(freq, gas, C, lines, constituents=GAS_FORMALISMS, h2state='e',
                  nh3='nh3_hs_sjs', chunk=16, cloud=None, Cl=None, other=None):
    """Per-gas absorption [nL, nf, nC] in cm^-1 (alpha.py:194-216
    get_alpha_from_calc, per layer; ``constituents`` in sorted order).

    ``gas`` is the reference gas table [ncol, nL] indexed by the dict ``C``;
    ``cloud`` / ``Cl`` the cloud table and its dict (clouds); ``other`` the
    other_dict per constituent (co: 'coshape', clouds: particle switches).
    """
    other = other or {}
    P = gas[C['P']]
    T = gas[C['T']]
    X = {k: (gas[C[k]] if k in C else np.zeros_like(P))
         for k in ('H2', 'HE', 'CH4', 'NH3', 'H2O', 'H2S', 'PH3', 'CO')}
    nL = P.size
    out = np.zeros((nL, len(freq), len(constituents)))
    for s in range(0, nL, chunk):
        sl = slice(s, min(nL, s + chunk))
        args = (T[sl], P[sl], X['H2'][sl], X['HE'][sl])
        for ci, c in enumerate(constituents):
            if c == 'h2':
                a = alpha_h2_jj_ddb(freq, *args, X['CH4'][sl], h2state=h2state)
            elif c == 'h2o':
                a = alpha_h2o_bk(freq, *args, X['H2O'][sl], lines['h2o'])
            elif c == 'h2s':
                a = alpha_h2s_ddb(freq, *args, X['H2S'][sl], lines['h2s'])
            elif c == 'ph3':
                a = alpha_ph3_jh(freq, *args, X['PH3'][sl], lines['ph3'], lines['ph3wgt'])
            elif c == 'nh3':
                if nh3 == 'nh3_hs_sjs':
                    a = alpha_nh3_hs_sjs(freq, *args, X['NH3'][sl], lines['ammonia'], lines['nh3'])
                elif nh3 == 'nh3_hs':
                    a = alpha_nh3_hs(freq, *args, X['NH3'][sl], lines['ammonia'])
                elif nh3 == 'nh3_sjs':
                    a = alpha_nh3_sjs(freq, *args, X['NH3'][sl], lines['nh3'])
                elif nh3 == 'nh3_dbs':
                    a = alpha_nh3_dbs(freq, *args, X['NH3'][sl], lines['ammonia'])
                elif nh3 == 'nh3_dbs_sjs':
                    a = alpha_nh3_dbs_sjs(freq, *args, X['NH3'][sl], lines['ammonia'], lines['nh3'])
                else:
                    raise ValueError(nh3)
            elif c == 'co':
                a = alpha_co_ddb(freq, *args, X['CO'][sl], lines['co'],
                                 coshape=other.get('co', {}).get('coshape', 'voigt'))
            elif c == 'clouds':
                a = alpha_clouds_idp(freq, T[sl], cloud[:, sl], Cl, other.get('clouds', {}))
            else:
                raise ValueError(c)
            out[sl, :, ci] = a
    return out


def layer_scale(scale, nL, constituents=GAS_FORMALISMS):
    """Alpha.get_layer_scale (alpha.py:235-259) as an [nL, nC] multiplier,
    plus a flag telling whether scale applies to the total (number/list)."""
    if isinstance(scale, dict):
        m = np.ones((nL, len(constituents)))
        for k, v in scale.items():
            if k not in constituents:
                raise ValueError('{} not found as constituent for alpha'.format(k))
            if len(v) != nL:
                raise ValueError('Incorrect scale for {}:  N {} vs {}'.format(k, len(v), nL))
            m[:, constituents.index(k)] = np.asarray(v, dtype=np.float64)
        return m
    if isinstance(scale, (list, np.ndarray)):
        if len(scale) != nL:
            raise ValueError('Incorrect number of scale layers.')
        return np.repeat(np.asarray(scale, dtype=np.float64)[:, None], len(constituents), axis=1)
    try:
        v = float(scale) if not isinstance(scale, (bool, dict, list)) else 1.0
    except (TypeError, ValueError):
        v = 1.0
    return np.full((nL, len(constituents)), v)


def total_alpha(per_gas, scale_matrix):
    """Alpha.total_layer_alpha (alpha.py:151-192) for every layer:
    returns (layers [nf, nL], scaled cube [nL, nf, nC])."""
    cube = per_gas * scale_matrix[:, None, :]
    tot = np.zeros(cube.shape[:2])
    for c in range(cube.shape[2]):          # sequential add, gas order
        tot = tot + cube[:, :, c]
    return tot.T.copy(), cube


# ---------------------------------------------------------------- geometry
def _r2d(a):
    return a * 180.0 / math.pi          # utils.py:90-92


def _d2r(a):
    return a * math.pi / 180.0          # utils.py:95-97


def _rot_x(x, v):
    c, s = math.cos(x), math.sin(x)
    return np.array([v[0], c * v[1] - s * v[2], s * v[1] + c * v[2]])


def _rot_y(y, v):
    c, s = math.cos(y), math.sin(y)
    return np.array([c * v[0] + s * v[2], v[1], -s * v[0] + c * v[2]])


def _rot_z(z, v):
    c, s = math.cos(z), math.sin(z)
    return np.array([c * v[0] - s * v[1], s * v[0] + c * v[1], v[2]])


def _rotate2planet(rotate, tip, v):
    return _rot_x(rotate, _rot_z(tip, v))   # raypath.py:47-51


class Ellipse:
    """Shape._calcEllipse state (shape.py:223-274): r, n, rmag."""

    def __init__(self, ab_ratio):
        self.k = ab_ratio
        self.r = np.zeros(3)
        self.n = np.zeros(3)
        self.rmag = 0.0

    def calc(self, a, pclat, delta_lng):
        b = self.k * a
        lat = _d2r(pclat)
        lng = _d2r(delta_lng)
        if lat == 0.0:
            lat = 1.0E-6
        norm = np.array([0.0, a * math.sin(lat), b * math.cos(lat)])
        norm = norm / math.sqrt(norm[1] ** 2 + norm[2] ** 2)
        self.n = _rot_y(lng, norm)
        r_vec = _rot_y(lng, np.array([0.0, b * math.sin(lat), a * math.cos(lat)]))
        self.r = r_vec
        self.rmag = math.sqrt(r_vec[0] ** 2 + r_vec[1] ** 2 + r_vec[2] ** 2)
        return self.rmag


def _latlng(v):
    nv = math.sqrt(v[0] ** 2 + v[1] ** 2 + v[2] ** 2)
    return _r2d(math.asin(v[1] / nv)), _r2d(math.atan2(v[0], v[2]))


def aspect(orientation, flattening):
    """computeAspect (raypath.py:39-44)."""
    tip = -orientation[0] * math.pi / 180.0
    rotate = -math.atan(math.tan(orientation[1] * math.pi / 180.0) * (1.0 - flattening) ** 2)
    return tip, rotate


def find_edge(b, rNorm, tip, rotate, k):
    """findEdge (raypath.py:60-105) for the ellipse geoid."""
    tmp = b[0] ** 2 + b[1] ** 2
    if tmp > 1.0:
        return None, None
    zq = np.arange(math.sqrt(1.0 - tmp) * 1.01, 0.0, -0.005)
    geo = Ellipse(k)
    r1s, r2s = [], []
    hit = False
    for z in zq:
        bv = _rotate2planet(rotate, tip, np.array([b[0], b[1], z]))
        r1 = math.sqrt(bv[0] ** 2 + bv[1] ** 2 + bv[2] ** 2) * rNorm
        lat, lng = _latlng(bv)
        r2 = geo.calc(rNorm, lat, lng)
        r1s.append(r1)
        r2s.append(r2)
        if r1 < r2:
            hit = True
            break
    if not hit:
        return None, None
    xx = np.flipud(np.array(r1s) - np.array(r2s))
    yy = np.flipud(zq[:len(r1s)])
    z = np.interp(0.0, xx, yy)
    bq = np.array([b[0], b[1], z])
    return rNorm * _rotate2planet(rotate, tip, bq), bq


def compute_ds(R, N, b, Req, Rpol, orientation=(0.0, 0.0), gtype='ellipse', limb='shape'):
    """compute_ds (raypath.py:108-273) with the tangent branch reachable
    (a negative discriminant takes the ``except ValueError`` path, as the
    reference intends; stock numpy returns NaN there instead).

    Returns (ds [km], layer4ds) as arrays, or (None, None) off the planet.
    """
    req = np.asarray(R, dtype=np.float64)
    nr = np.asarray(N, dtype=np.float64)
    nL = len(req)
    rNorm = req[0]
    if b[0] ** 2 + b[1] ** 2 >= 1.0:
        return None, None
    mu = math.sqrt(1.0 - b[0] ** 2 - b[1] ** 2)
    f = 1.0 - Rpol / Req
    k = (Rpol / Req) if gtype == 'ellipse' else 1.0
    tip, rotate = aspect(orientation, f)
    edge, _ = find_edge(b, rNorm, tip, rotate, k)
    if edge is None:
        return None, None
    pclat, dlng = _latlng(edge)
    geo = Ellipse(k)
    geo.calc(rNorm, pclat, dlng)
    s = _rotate2planet(rotate, tip, np.array([0.0, 0.0, -1.0]))
    n = geo.n
    r = geo.r
    c0 = -float(np.dot(s, n))
    t_inc = math.acos(c0) if -1.0 <= c0 <= 1.0 else float('nan')
    nratio = nr[0] / nr[1]
    t_tran = math.asin(nratio * math.sin(t_inc)) if not math.isnan(t_inc) else float('nan')
    ds_out, lay_out = [], []
    layer = 0
    direction = 1                 # ingress +1, tangent 0, egress -1
    while True:
        dvec = 1 if direction == 1 else (-1 if direction == -1 else 0)
        s = nratio * s + dvec * (nratio * math.cos(t_inc) * n - math.cos(t_tran) * n)
        rNow = geo.rmag
        rNext = geo.calc(req[layer + dvec], pclat, dlng)
        rdots = float(np.dot(r, s))
        disc = rdots ** 2.0 + rNext ** 2.0 - rNow ** 2.0
        if disc < 0.0:
            if direction == 1:
                direction = 0
                ds_step = -2.0 * rdots
                if ds_step > rNorm:
                    break
                rNext = rNow
            else:
                break
        else:
            sq = math.sqrt(disc)
            ds_step = (-rdots - sq) if direction == 1 else (-rdots + sq)
        if ds_step < 0.0:
            break
        if limb == 'sec':
            ds_step = abs(rNext - rNow) / mu
        ds_out.append(ds_step)
        lay_out.append(layer)
        rnext = r + ds_step * s
        pclat, dlng = _latlng(rnext)
        dv = 0 if direction == 0 else direction
        geo.calc(req[layer + dv], pclat, dlng)
        r = rnext
        n = geo.n
        layer += dv
        if direction == 0:
            direction = -1
            t_inc = math.pi / 2.0
        else:
            c = -direction * float(np.dot(s, n))
            t_inc = math.acos(c) if -1.0 <= c <= 1.0 else float('nan')
        # index check of raypath.py:253-264 (python negative indices wrap)
        nxt = layer + (-1 if direction == -1 else 1)
        if not (-nL <= nxt < nL) or not (-nL <= layer < nL):
            break
        nratio = 1.0
        t_tran = math.asin(nratio * math.sin(t_inc)) if not math.isnan(t_inc) else float('nan')
    return np.array(ds_out), np.array(lay_out, dtype=np.int64)


# ---------------------------------------------------------------- brightness
def expn2(x):
    from scipy.special import expn
    return expn(2, x)


def brightness(ds, layer4ds, alpha_layers, T_layers, disc=False):
    """Brightness.single core (brightness.py:53-126) for one ray.

    alpha_layers [nf, nL] cm^-1, ds in km.  Returns (Tb [nf], tau, W,
    integrated_W) with tau/W shaped [nf, nseg].
    """
    nf = alpha_layers.shape[0]
    if ds is None:
        return np.full(nf, T_CMB), None, None, None
    nseg = len(ds) - 1
    if nseg < 1:
        return np.full(nf, T_CMB), np.zeros((nf, 1)), np.zeros((nf, 1)), np.zeros(nf)
    d = np.asarray(ds[:-1], dtype=np.float64) * 1.0e3 / 1.0e-2    # km -> cm (brightness.py:66)
    ii = np.asarray(layer4ds[:-1])
    ii1 = np.asarray(layer4ds[1:])
    a0 = alpha_layers[:, ii]
    a1 = alpha_layers[:, ii1]
    dtau = (a0 + a1) * d / 2.0
    tau = np.concatenate([np.zeros((nf, 1)), np.cumsum(dtau, axis=1)], axis=1)
    if disc:
        W1 = 2.0 * a1 * expn2(tau[:, 1:])
    else:
        W1 = a1 * np.exp(-tau[:, 1:])
    W = np.concatenate([np.zeros((nf, 1)), W1], axis=1)
    iw = np.cumsum((W[:, 1:] + W[:, :-1]) * d / 2.0, axis=1)[:, -1]
    T0 = T_layers[ii]
    T1 = T_layers[ii1]
    tbl = np.cumsum((T1 * W[:, 1:] + T0 * W[:, :-1]) * d / 2.0, axis=1)[:, -1]
    Tb = np.where(tbl < T_CMB, T_CMB, tbl / np.where(tbl < T_CMB, 1.0, iw))
    return Tb, tau, W, iw


def forward(gas, C, R, N, freqs, rays, lines, Req, Rpol, orientation=(0.0, 0.0),
            disc=False, h2state='e', scale=False, weights=None, **alpha_kw):
    """alpha for every layer, then one Brightness.single per ray.
    Returns (Tb [nb, nf], layers [nf, nL], disc average or None).
    ``alpha_kw`` goes to alpha_per_gas (constituents, nh3, cloud, Cl, other)."""
    per = alpha_per_gas(freqs, gas, C, lines, h2state=h2state, **alpha_kw)
    cons = alpha_kw.get('constituents', GAS_FORMALISMS)
    layers, _ = total_alpha(per, layer_scale(scale, gas.shape[1], cons))
    T = gas[C['T']]
    tbs = []
    for b in rays:
        bb = [0.0, 0.0] if disc else b
        ds, lay = compute_ds(R, N, bb, Req, Rpol, orientation)
        tb, _, _, _ = brightness(ds, lay, layers, T, disc=disc)
        tbs.append(tb)
    tbs = np.array(tbs)
    avg = None if weights is None else np.tensordot(np.asarray(weights), tbs, axes=1)
    return tbs, layers, avg
