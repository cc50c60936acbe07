"""CPU oracle of the atmosphere producer: regrid and computeProp.

TEST INFRASTRUCTURE ONLY (see oracle/oracle.py): the checker for the GPU
atmosphere kernels; the package never imports it.

Restates, in float64 numpy with the reference's loop order:
  * ``AtmosphereBase.computeProp`` (radiobear/atm_base.py:120-194);
  * ``regrid.regrid`` (radiobear/regrid.py:11-82) with ``interpolate``
    (103-124), ``extrapolate`` (127-164), ``_extrapolate_outward``
    (167-176) and ``AtmosphereBase._renorm_z`` (atm_base.py:206-219);
  * the constituent properties of ``chemistry.ConstituentProperties``
    (radiobear/chemistry.py:8-48,168-200): amu, c_p / R and the microwave
    refractivity (H2O: 245 + 1.28e6 / T).

Pinned against the reference run on the same inputs
(tests/golden/make_golden.py f3).
"""
from __future__ import annotations

import numpy as np

GRAV_CONST = 6.6738e-20     # km3/kg/s2, chemistry.py:7
R_GAS = 8.314462            # J/K/mol, chemistry.py:8
AMU = {'H2': 2.016, 'HE': 4.003, 'H2S': 34.076, 'NH3': 17.030, 'H2O': 18.015,
       'CH4': 16.04, 'PH3': 33.997, 'NH4SH': 51.110}
CP = {'H2': 3.5, 'HE': 2.50, 'H2O': 4.00, 'NH3': 4.46, 'H2S': 4.01, 'CH4': 4.50}
REFR = {'H2': 124.43, 'HE': 35.832, 'H2S': 2247.0, 'NH3': 2700.0, 'CH4': 413.0}
PROP_ROWS = ('Z', 'R', 'P', 'GM', 'AMU', 'REFR', 'N', 'H', 'LAPSE', 'LAPSEP', 'g')


def refractivity(key, T):
    if key == 'H2O':
        return 245.0 + 1.28E6 / T
    return REFR.get(key, 0.0)


def chem_keys(C):
    return [k for k in C if k not in ('P', 'T', 'Z', 'DZ')]


def compute_prop(gas, C, Req, p_ref, GM_ref):
    """computeProp: property table [len(PROP_ROWS), nL] (rows PROP_ROWS)."""
    LP = {k: i for i, k in enumerate(PROP_ROWS)}
    keys = chem_keys(C)
    P, T, Z = gas[C['P']], gas[C['T']], gas[C['Z']]
    nL = P.size
    psep, iOffset = 1.0E6, 0
    for i in range(nL):
        if abs(P[i] - p_ref) < psep:
            psep = abs(P[i] - p_ref)
            iOffset = i
    zOffset = Z[iOffset]
    prop = np.zeros((len(PROP_ROWS), nL))
    for i in range(nL):
        prop[LP['P'], i] = P[i]
        prop[LP['Z'], i] = Z[i]
        rr = Req + Z[i] - zOffset
        prop[LP['R'], i] = rr
        amulyr = 0.0
        for k in keys:
            amulyr += AMU.get(k, 0.0) * gas[C[k], i]
        prop[LP['AMU'], i] = amulyr
        if i:
            rho = (amulyr * P[i]) / (R_GAS * T[i])
            dr = abs(Z[i] - Z[i - 1])
            dM = 1.0e11 * rho * 4.0 * np.pi * (rr ** 2) * dr
            prop[LP['GM'], i] = prop[LP['GM'], i - 1] + GRAV_CONST * dM
            dT = abs(T[i] - T[i - 1])
            prop[LP['LAPSE'], i] = dT / dr
            prop[LP['LAPSEP'], i] = dT / abs(P[i] - P[i - 1])
        refr = 0.0
        for k in keys:
            refr += refractivity(k, T[i]) * gas[C[k], i]
        refr = refr * P[i] * (293.0 / T[i])
        prop[LP['REFR'], i] = refr
        prop[LP['N'], i] = refr / 1.0E6 + 1.0
    GMnorm = prop[LP['GM'], iOffset]
    for i in range(nL):
        gm = GM_ref - (prop[LP['GM'], i] - GMnorm)
        prop[LP['GM'], i] = gm
        g = gm / prop[LP['R'], i] ** 2
        prop[LP['H'], i] = (R_GAS * T[i]) / (g * prop[LP['AMU'], i]) / 1000.0
        prop[LP['g'], i] = g
    return prop


def _interpolate(tab, ind, Pgrid, fillval):
    out = np.zeros((tab.shape[0], Pgrid.size))
    Pin = tab[ind['P']]
    out[ind['P']] = Pgrid
    inside = (Pgrid >= Pin[0]) & (Pgrid <= Pin[-1])
    for k, i in ind.items():
        if k in ('P', 'DZ'):
            continue
        out[i] = np.where(inside, np.interp(Pgrid, Pin, tab[i]), fillval)
    return out


def _renorm_z(tab, ind):
    tab[ind['Z']] = tab[ind['Z']] - tab[ind['Z']][-1]
    tab[ind['DZ']] = np.append(0.0, np.abs(np.diff(tab[ind['Z']])) * 1.0E5)


def regrid(gas, cloud, C, Cl, Pgrid, Req, p_ref, GM_ref):
    """regrid onto the pressure grid Pgrid (increasing): returns (gas, cloud)."""
    fillval = -999.9
    Pgrid = np.asarray(Pgrid, dtype=np.float64)
    new = _interpolate(gas, C, Pgrid, fillval)
    if np.any(new == fillval):
        prop = compute_prop(gas, C, Req, p_ref, GM_ref)
        LP = {k: i for i, k in enumerate(PROP_ROWS)}
        keys = chem_keys(C)
        for k, ci in C.items():                       # constituents: deepest value
            if k in ('Z', 'P', 'T', 'DZ'):
                continue
            new[ci] = np.where(new[ci] == fillval, gas[ci][-1], new[ci])
        pDeep = gas[C['P']][-1]
        g = prop[LP['g']][-1]
        r = prop[LP['R']][-1]
        n = Pgrid.size
        for i in range(n):                            # dry adiabat inward
            p = new[C['P'], i]
            if p < pDeep:
                continue
            prev = new[C['P'], (i - 1) % n]
            dP = p - prev
            T = new[C['T'], (i - 1) % n]
            z = new[C['Z'], (i - 1) % n]
            amu = 0.0
            cp = 0.0
            for k in keys:
                cp += CP.get(k, 0.0) * new[C[k], i]
                amu += AMU.get(k, 0.0) * new[C[k], i]
            new[C['T'], i] = T + T / (cp * p) * dP
            g = g + 2.0 * R_GAS * T * np.log(p / prev) / (r * amu) / 1000.0
            H = R_GAS * T / (amu * g) / 1000.0
            dz = H * dP / p
            r = r - dz
            new[C['Z'], i] = z - dz
        if np.any(new == fillval):                    # outward along the last slope
            x = new[C['P']]
            for k, ci in C.items():
                if k in ('P', 'DZ'):
                    continue
                y = new[ci]
                i0 = 0
                while i0 < y.size and y[i0] == fillval:
                    i0 += 1
                slope = (y[i0 + 1] - y[i0]) / (x[i0 + 1] - x[i0])
                for j in range(i0 - 1, -1, -1):
                    y[j] = y[j + 1] + slope * (x[j + 1] - x[j])
                    if y[j] <= 0.0:
                        y[j] = 1e-20
    if np.any(new == fillval):
        raise ValueError('fillval still in gas!')
    newc = _interpolate(cloud, Cl, Pgrid, 0.0)
    _renorm_z(new, C)
    _renorm_z(newc, Cl)
    return new, newc
