"""CPU: the absorption JVP's line-shape tangents (br_eval2 and the Gross and
VVW branches of jv_family in radiobear_gb300/csrc/rb_adjoint.cu) restated
in numpy float32 and checked against complex-step derivatives of the
oracle's float64 line shapes (oracle._ben_reuven_hs, nh3_hs.py:193-226;
oracle._gross, nh3_hs.py:259-263; the VVW terms of h2o_bk.py:177-187).

Per line t = S n / den with n = (g - z) F + (g + z) K, den = e^2 + 4 g^2 F,
e = F - K from float pairs; along a tangent (dg, dz, dK, dlnS)
dt = Ag dg + Az dz + AK dK + t dlnS with
    Ag = S/den (F + K - 8 F g n/den), Az = S/den (K - F),
    AK = S/den (g + z + 2 e n/den).
The kernel sums these in plain float32 per lane (line pairs in the two
halves of an f32x2), the value in blocks into a compensated sum.  A K
tangent maps onto the oracle's pressure shift: dK = 2 (fo + d) dd + 2 g dg
- 2 z dz.
"""
import numpy as np
import pytest

from oracle import oracle as O
from tests.test_line_sum_algebra import (FREQS, LAYERS, _cat, _inversion, f32, fma32, split,
                                         two_sum32)


def jvp_br_sums(fo, g, z, d, S, dlnS, dg, dz, dK, freqs, planted=False):
    """Sums over lines of t and of dt along three tangents ([3, nlines]
    each) at every frequency, as one line group of the JVP kernel sums them.
    planted: Az with its sign flipped (a mistake planted in the restatement)."""
    g, z, d, S, dlnS = (np.asarray(v).astype(f32) for v in (g, z, d, S, dlnS))
    dg, dz, dK = (np.asarray(v).astype(f32) for v in (dg, dz, dK))
    c2h, c2l = split(np.square(fo))
    KH, e0 = two_sum32(c2h, fma32(f32(2) * fo.astype(f32) + d, d, (g - z) * (g + z)))
    KL = e0 + c2l
    K = KH + KL
    gp, gm = g + z, g - z
    G4 = f32(4) * (g * g)
    F, FL = split(np.square(freqs))
    m8F = f32(-8) * F
    vp = np.zeros((2, len(freqs)), f32)             # value per lane, 8 pairs at a time
    ks = np.zeros(len(freqs), f32)                   # compensated sum (KSum)
    kc = np.zeros(len(freqs), f32)
    der = np.zeros((3, 2, len(freqs)), f32)

    def kadd(v):
        nonlocal ks, kc
        y = v - kc
        t = ks + y
        kc = (t - ks) - y
        ks = t

    for i in range(len(fo)):
        lane = i & 1
        e = (F + (-KH[i])) + (FL + (-KL[i]))
        r = f32(1) / fma32(e, e, G4[i] * F)
        nr = fma32(gm[i], F, gp[i] * K[i]) * r
        t = S[i] * nr
        Sr = S[i] * r
        Ag = Sr * fma32(m8F * g[i], nr, F + K[i])
        Az = Sr * ((F - K[i]) if planted else (K[i] - F))
        AK = Sr * fma32(e + e, nr, gp[i])
        for q in range(3):
            der[q, lane] = fma32(Ag, dg[q, i], fma32(Az, dz[q, i], fma32(AK, dK[q, i], der[q, lane])))
        der[0, lane] = fma32(t, dlnS[i], der[0, lane])
        vp[lane] = vp[lane] + t
        if lane == 1 and i % 16 == 15:
            kadd(vp[0] + vp[1])
            vp[:] = 0
    kadd(vp[0] + vp[1])
    return (ks - kc).astype(float), (der[:, 0] + der[:, 1]).astype(float)


def _oracle_tangents(fo, Io, g, z, d, dlnS, dg, dz, dK, freqs, smax):
    """Complex-step directional derivatives of sum_l I_l BR_l (tangent 0
    also along ln S), scaled like the kernel's sums, and the sums of the
    terms' magnitudes."""
    h = 1e-30
    f = freqs[None, :] + 0j
    out, mag = [], []
    for q in range(3):
        dd = (dK[q] - 2.0 * g * dg[q] + 2.0 * z * dz[q]) / (2.0 * (fo + d))
        w = Io * (1.0 + 1j * h * dlnS) if q == 0 else Io + 0j
        sh = w[:, None] * O._ben_reuven_hs(f, fo[:, None] + 0j, (g + 1j * h * dg[q])[:, None],
                                           (z + 1j * h * dz[q])[:, None], (d + 1j * h * dd)[:, None])
        scale = np.pi / (2.0 * np.square(freqs)) / smax / h
        out.append(np.imag(sh.sum(axis=0)) * scale)
        mag.append(np.abs(np.imag(sh)).sum(axis=0) * scale)
    return np.array(out), np.array(mag)


def _case(T, P, seed):
    cat = _cat()
    order = np.argsort(cat['ammonia__fo'], kind='stable')
    fo, Io = cat['ammonia__fo'][order], cat['ammonia__Io'][order]
    cat['ammonia__gammaNH3o'] = cat['ammonia__gammaNH3o'][order]
    rng = np.random.default_rng(seed)
    n = len(fo)
    tangents = dict(dlnS=rng.normal(size=n), dg_rel=rng.normal(size=(3, n)),
                    dz_rel=rng.normal(size=(3, n)), dK=1e-3 * np.square(fo) * rng.normal(size=(3, n)))
    return cat, fo, Io, tangents


@pytest.mark.parametrize('T,P', LAYERS)
def test_br_tangents_match_complex_step(T, P):
    """Both coefficient sets (30 GHz), every layer from 0.01 to 1000 bar:
    each tangent's sum within 5e-6 of the sum of its terms' magnitudes, the
    value within 1e-6 relative.  Measured: <= 4.1e-7, except 2.9e-6 at 0.01
    bar below 30 GHz, where lines 0.03 GHz wide sit among the frequencies
    and a line's K term (g + z + 2 e n/den) dK cancels within itself near
    its centre (the same formulas in float64 agree with the complex step to
    1.5e-12 there: the float32 rounding, not the algebra)."""
    cat, fo, Io, tg = _case(T, P, int(T + 10 * P))
    S = Io / np.square(fo)
    smax = S.max()
    for lo_set in (True, False):
        freqs = FREQS[FREQS <= O.F_SPLIT] if lo_set else FREQS[FREQS > O.F_SPLIT]
        g, z, d, _ = _inversion(cat, T, P, O.HS_INV_LO if lo_set else O.HS_INV_HI)
        dg, dz = g * tg['dg_rel'], z * tg['dz_rel']
        val, der = jvp_br_sums(fo, g, z, d, S / smax, tg['dlnS'], dg, dz, tg['dK'], freqs)
        ref, mag = _oracle_tangents(fo, Io, g, z, d, tg['dlnS'], dg, dz, tg['dK'], freqs, smax)
        assert np.max(np.abs(der - ref) / mag) < 5e-6
        vref = np.sum(Io[:, None] * O._ben_reuven_hs(freqs[None, :], fo[:, None], g[:, None],
                                                      z[:, None], d[:, None]), axis=0) \
            * np.pi / (2.0 * np.square(freqs)) / smax
        np.testing.assert_allclose(val, vref, rtol=1e-6)


def test_br_tangents_catch_a_sign_error():
    """Planted in the restatement: Az = S/den (F - K).  The tangents then
    miss the complex-step derivatives by far more than the bound above."""
    T, P = 170.0, 2.0
    cat, fo, Io, tg = _case(T, P, 7)
    S = Io / np.square(fo)
    freqs = FREQS[FREQS > O.F_SPLIT]
    g, z, d, _ = _inversion(cat, T, P, O.HS_INV_HI)
    dg, dz = g * tg['dg_rel'], z * tg['dz_rel']
    _, der = jvp_br_sums(fo, g, z, d, S / S.max(), tg['dlnS'], dg, dz, tg['dK'], freqs,
                         planted=True)
    ref, mag = _oracle_tangents(fo, Io, g, z, d, tg['dlnS'], dg, dz, tg['dK'], freqs, S.max())
    assert np.max(np.abs(der - ref) / mag) > 1e-2


def jvp_gross_sums(fo, g, S, dlnS, dg, freqs):
    """The JVP's Gross lines: t = S g / den, den = e^2 + 4 g^2 F;
    dt = t dlnS (tangent 0) + S dg (1 - 8 F g^2 / den) / den."""
    g, S, dlnS, dg = (np.asarray(v).astype(f32) for v in (g, S, dlnS, dg))
    KH, KL = split(np.square(fo))
    G4 = f32(4) * (g * g)
    F, FL = split(np.square(freqs))
    m8F = f32(-8) * F
    der = np.zeros((3, 2, len(freqs)), f32)
    for i in range(len(fo)):
        lane = i & 1
        e = (F + (-KH[i])) + (FL + (-KL[i]))
        r = f32(1) / fma32(e, e, G4[i] * F)
        Sr = S[i] * r
        tv = Sr * g[i]
        k = Sr * fma32(m8F * (g[i] * g[i]), r, f32(1))
        der[0, lane] = fma32(k, dg[0, i], fma32(tv, dlnS[i], der[0, lane]))
        for q in (1, 2):
            der[q, lane] = fma32(k, dg[q, i], der[q, lane])
    return (der[:, 0] + der[:, 1]).astype(float)


def jvp_vvw_sums(centre, df, S, dlnS, ddf, freqs):
    """The JVP's VVW lines: t = h (r1 + r2), h = S df, r1 = 1/((f - fo)^2 +
    df^2), r2 = 1/((f + fo)^2 + df^2); dt = t dlnS (tangent 0) + (S u -
    2 h df (r1^2 + r2^2)) ddf, u = r1 + r2."""
    df, S, dlnS, ddf = (np.asarray(v).astype(f32) for v in (df, S, dlnS, ddf))
    ch, cl = split(centre)
    d2 = df * df
    fq, fl = split(freqs)
    der = np.zeros((3, 2, len(freqs)), f32)
    for i in range(len(centre)):
        lane = i & 1
        dm = (fq + (-ch[i])) + (fl + (-cl[i]))
        dp = fq - (-ch[i])
        r1 = f32(1) / fma32(dm, dm, d2[i])
        r2 = f32(1) / fma32(dp, dp, d2[i])
        h = S[i] * df[i]
        u = r1 + r2
        tv = h * u
        k2 = (h + h) * (df[i] * fma32(r1, r1, r2 * r2))
        c = S[i] * u - k2
        der[0, lane] = fma32(c, ddf[0, i], fma32(tv, dlnS[i], der[0, lane]))
        for q in (1, 2):
            der[q, lane] = fma32(c, ddf[q, i], der[q, lane])
    return (der[:, 0] + der[:, 1]).astype(float)


def _complex_step(shape, w, dlnS, nq=3):
    """Directional derivatives (and term magnitudes) of sum_l w_l shape_l
    by complex step: shape(q, h) evaluates with the tangent q at step i h."""
    h = 1e-30
    out, mag = [], []
    for q in range(nq):
        ww = w * (1.0 + 1j * h * dlnS) if q == 0 else w + 0j
        terms = np.imag(ww[:, None] * shape(q, h)) / h
        out.append(terms.sum(axis=0))
        mag.append(np.abs(terms).sum(axis=0))
    return np.array(out), np.array(mag)


@pytest.mark.parametrize('grid', ['radio', 'submm'])
@pytest.mark.parametrize('T,P', LAYERS)
def test_gross_tangents_match_complex_step(grid, T, P):
    """Rotational lines (per-line widths, nh3_hs.py:232-265) against
    complex-step derivatives of oracle._gross: within 1e-6 of the terms'
    magnitudes."""
    from tests.test_line_sum_algebra import GRIDS
    freqs = GRIDS[grid]
    cat = _cat()
    order = np.argsort(cat['ammonia__fo_rot'], kind='stable')
    fo, Io = cat['ammonia__fo_rot'][order], cat['ammonia__Io_rot'][order]
    Td = 300.0 / T
    (eH2, eHe, eNH3), (nH2, nHe, nNH3) = O.HS_ROT['eta'], O.HS_ROT['gnu']
    g = (nH2 * P * 0.86 * cat['ammonia__gH2_rot'][order]) * Td ** eH2 \
        + (nHe * P * 0.135 * cat['ammonia__gHe_rot'][order]) * Td ** eHe \
        + (nNH3 * P * 3e-4 * cat['ammonia__gNH3_rot'][order]) * Td ** eNH3
    rng = np.random.default_rng(int(T + P))
    dlnS, dg = rng.normal(size=fo.size), g * rng.normal(size=(3, fo.size))
    smax = Io.max()
    der = jvp_gross_sums(fo, g, Io / smax, dlnS, dg, freqs)
    scale = np.pi / (4.0 * np.square(freqs)) / smax
    ref, mag = _complex_step(lambda q, h: O._gross(freqs[None, :] + 0j, fo[:, None] + 0j,
                                                   (g + 1j * h * dg[q])[:, None]), Io, dlnS)
    assert np.max(np.abs(der - ref * scale) / (mag * scale)) < 1e-6


@pytest.mark.parametrize('grid', ['radio', 'submm'])
@pytest.mark.parametrize('T,P', LAYERS)
def test_vvw_tangents_match_complex_step(grid, T, P):
    """Water lines: the two resonant terms of h2o_bk.py:177-187 (as in
    oracle.alpha_h2o_bk) differentiated along the width df: within 3e-6
    of the terms' magnitudes (measured 1.3e-6: a Lorentzian's width
    derivative vanishes one width from its centre, where S u and
    2 h df (r1^2 + r2^2) cancel in float32)."""
    from tests.test_line_sum_algebra import GRIDS, _water
    freqs = GRIDS[grid]
    centre, df, S = _water(T, P)
    rng = np.random.default_rng(int(3 * T + P))
    dlnS, ddf = rng.normal(size=df.size), df * rng.normal(size=(3, df.size))
    smax = S.max()
    der = jvp_vvw_sums(centre, df, S / smax, dlnS, ddf, freqs)
    f = freqs[None, :] + 0j

    def shape(q, h):
        w = (df + 1j * h * ddf[q])[:, None]
        c = centre[:, None]
        return w / ((f - c) ** 2 + w * w) + w / ((f + c) ** 2 + w * w)

    ref, mag = _complex_step(shape, S / smax, dlnS)
    assert np.max(np.abs(der - ref) / mag) < 3e-6
