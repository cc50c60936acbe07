"""CPU: the float32 arithmetic of the line-sum kernel (rb_alpha_lines_kernel,
radiobear_gb300/csrc/rb_alpha.cu) restated in numpy and checked against the
oracle's float64 line shapes on the real line catalogues.

* Record fields per line as the kernel forms them: K = (fo + d)^2 + g^2 - z^2
  as a float pair, G4 - 2K, K^2, S(g - z), S(g + z)K (Ben-Reuven, nh3_hs.py:
  193-226); G4 - 2K, K^2, S g with K = fo^2 (Gross, nh3_hs.py:259-263,
  296-300);
  2(d2 - c2), C^2, 2h, 2hC (VVW, h2o_bk.py:174-187).
* The two-operation far-line denominator F (F + (G4 - 2K)) + K^2 for lines
  whose centre lies outside [0.75 fmin, 1.3 fmax] of a chain of 32
  frequencies; inside, the float-pair difference F - K.
* Two lines sharing one reciprocal, (nP dQ + nQ dP) / (dP dQ), over the two
  lanes of a quad of four lines; compensated sums flushed every 64 lines.
* Ben-Reuven layers whose width floor is at least 0.32 of the largest line
  centre ("wide") take the far-line form for every line.
* nh3_sjs: widths from per-frequency blended coefficients, every line on
  the float-pair form with its own reciprocal.
* Line strengths 2^(l2I + cE E - M2) with the exponent as a float pair.
Float32 operations are exact numpy float32 arithmetic; a fused multiply-add
is the float64 product (exact for float32 operands) plus the addend, rounded
to float32.
"""
import numpy as np
import pytest

from oracle import oracle as O

f32 = np.float32
ULP = 2.0 ** -23                        # float32 ulp of 1.0
# the 256 log-spaced frequencies from 0.5 to 100 GHz of the 1000-layer disc
# spectrum, in chains of 32
FREQS = np.logspace(np.log10(0.5), np.log10(100.0), 256)
# and 64 from 100 GHz to 2 THz, where the rotational, H2S, PH3 and water
# lines fall inside the chains' windows
GRIDS = {'radio': FREQS, 'submm': np.logspace(2.0, np.log10(2000.0), 64)}


def _cat():
    z = np.load(__file__.rsplit('/', 1)[0] + '/golden/catalogs_real.npz')
    return {k: z[k] for k in z.files}


def fma32(a, b, c):
    return (np.asarray(a, np.float64) * np.asarray(b, np.float64)
            + np.asarray(c, np.float64)).astype(f32)


def split(x):
    """float64 -> (hi, lo) float32 pair."""
    x = np.asarray(x, np.float64)
    hi = x.astype(f32)
    return hi, (x - hi).astype(f32)


def two_sum32(a, b):
    s = a + b
    bb = s - a
    return s, (a - (s - bb)) + (b - bb)


def _pad(v, fill):
    return np.concatenate([np.asarray(v, f32), np.full((-len(v)) % 4, fill, f32)])


def br_records(fo, g, z, d, S):
    """Ben-Reuven record fields (padding lines: K = 1, G4 = 1, no strength)."""
    g, z, d, S = (np.asarray(v).astype(f32) for v in (g, z, d, S))
    c2h, c2l = split(np.square(fo))
    small = fma32(f32(2) * fo.astype(f32) + d, d, (g - z) * (g + z))
    KH, e = two_sum32(c2h, small)
    kl = e + c2l
    G4 = f32(4) * g * g
    r = dict(v0=fma32(f32(-2), KH, G4) - f32(2) * kl, v1=fma32(KH, KH, f32(2) * KH * kl),
             a=S * (g - z), b=(S * (g + z)) * (KH + kl), KH=KH, kl=kl, G4=G4)
    fill = dict(v0=-1, v1=1, a=0, b=0, KH=1, kl=0, G4=1)
    return {k: _pad(v, fill[k]) for k, v in r.items()}


def gross_records(fo, g, S):
    g, S = np.asarray(g).astype(f32), np.asarray(S).astype(f32)
    KH, kl = split(np.square(fo))
    G4 = f32(4) * g * g
    r = dict(v0=fma32(f32(-2), KH, G4) - f32(2) * kl, v1=fma32(KH, KH, f32(2) * KH * kl),
             a=S * g, KH=KH, kl=kl, G4=G4)
    fill = dict(v0=-1, v1=1, a=0, KH=1, kl=0, G4=1)
    return {k: _pad(v, fill[k]) for k, v in r.items()}


def vvw_records(centre, df, S):
    df, S = np.asarray(df).astype(f32), np.asarray(S).astype(f32)
    ch, cl = split(centre)
    c2 = fma32(ch, ch, f32(2) * ch * cl)
    d2 = df * df
    h = S * df
    C = c2 + d2
    r = dict(v0=f32(2) * (d2 - c2), v1=C * C, a=f32(2) * h, b=(f32(2) * h) * C, ch=ch, cl=cl,
             d2=d2, h=h)
    fill = dict(v0=0, v1=1, a=0, b=0, ch=0, cl=0, d2=1, h=0)
    return {k: _pad(v, fill[k]) for k, v in r.items()}


def line_terms(kind, r, i, F, FL, fq, fl, precise):
    """(numerator, denominator) of line i at every frequency, float32."""
    if kind == 'vvw':
        if precise:
            dm = (fq + (-r['ch'][i])) + (fl + (-r['cl'][i]))
            den1 = fma32(dm, dm, r['d2'][i])
            dp = fma32(-r['ch'][i], f32(-1), fq)
            den2 = fma32(dp, dp, r['d2'][i])
            return r['h'][i] * (den1 + den2), den1 * den2
        return fma32(r['a'][i], F, r['b'][i]), fma32(F, F + r['v0'][i], r['v1'][i])
    if precise:
        e = (F + (-r['KH'][i])) + (FL + (-r['kl'][i]))
        den = fma32(e, e, r['G4'][i] * F)
    else:
        den = fma32(F, F + r['v0'][i], r['v1'][i])
    num = np.full_like(F, r['a'][i]) if kind == 'gross' else fma32(r['a'][i], F, r['b'][i])
    return num, den


def kernel_sum(kind, r, freqs, precise_q):
    """The kernel's compensated line sum at each frequency.  precise_q
    [nquad, nf]: the quad runs at the float-pair tier for that frequency."""
    F, FL = split(np.square(freqs))
    fq, fl = split(freqs)
    nq = len(r['a']) // 4
    s = np.zeros((2, len(freqs)), f32)
    c = np.zeros_like(s)
    p = np.zeros_like(s)
    for q in range(nq):
        nd = []
        for i in range(4 * q, 4 * q + 4):
            fast = line_terms(kind, r, i, F, FL, fq, fl, False)
            prec = line_terms(kind, r, i, F, FL, fq, fl, True)
            nd.append((np.where(precise_q[q], prec[0], fast[0]),
                       np.where(precise_q[q], prec[1], fast[1])))
        for h in range(2):            # lanes: lines (4q, 4q+2) and (4q+1, 4q+3)
            (ni, di), (nj, dj) = nd[h], nd[h + 2]
            N = fma32(ni, dj, nj * di)
            p[h] = fma32(N, f32(1) / (di * dj), p[h])
        if q % 16 == 15 or q == nq - 1:   # 64 lines
            y = p - c
            t = s + y
            c = (t - s) - y
            s = t
            p[:] = 0
    return ((s[0] - c[0]) + (s[1] - c[1])).astype(np.float64)


def window_quads(centre, freqs, force_fast=False):
    """[nquad, nf]: quads with a line centre inside [0.75 fmin, 1.3 fmax] of
    the frequency's chain of 32."""
    inwin = np.zeros((len(centre), len(freqs)), bool)
    if not force_fast:
        for c0 in range(0, len(freqs), 32):
            lo, hi = freqs[c0:c0 + 32].min(), freqs[c0:c0 + 32].max()
            inwin[:, c0:c0 + 32] = ((centre >= 0.75 * lo) & (centre <= 1.3 * hi))[:, None]
    inwin = np.concatenate([inwin, np.zeros(((-len(centre)) % 4, len(freqs)), bool)])
    return inwin.reshape(-1, 4, len(freqs)).any(axis=1)


# (T K, P bar); at 300 K the inversion layers turn wide at ~46.6 bar (both
# coefficient sets' width floors at 0.32 of the 220 GHz largest centre)
LAYERS = [(110.0, 0.01), (115.0, 0.05), (120.0, 0.5), (170.0, 2.0), (300.0, 20.0),
          (300.0, 46.7), (450.0, 150.0), (700.0, 1000.0)]
XH2, XHE, XNH3, XH2O = 0.86, 0.135, 3e-4, 5e-3


def _inversion(cat, T, P, coefs):
    """Widths of nh3_hs.py:183-205 (oracle _nh3_hs_block)."""
    (gH2, gHe, gNH3, GH2, GHe, GNH3, zH2, zHe, zNH3, ZH2, ZHe, ZNH3, d, _) = coefs
    Ph2, Phe, Pnh3 = P * XH2, P * XHE, P * XNH3
    Td = 300.0 / T
    floor = gH2 * Ph2 * Td ** GH2 + gHe * Phe * Td ** GHe
    gamma = floor + gNH3 * Pnh3 * cat['ammonia__gammaNH3o'] * (295.0 / T) ** GNH3
    zeta = zH2 * Ph2 * Td ** ZH2 + zHe * Phe * Td ** ZHe \
        + zNH3 * Pnh3 * cat['ammonia__gammaNH3o'] * (295.0 / T) ** ZNH3
    return gamma, zeta, d * gamma, floor


@pytest.mark.parametrize('grid', sorted(GRIDS))
@pytest.mark.parametrize('T,P', LAYERS)
def test_inversion_line_sum_matches_the_oracle(grid, T, P):
    freqs = GRIDS[grid]
    cat = _cat()
    order = np.argsort(cat['ammonia__fo'], kind='stable')
    fo, Io = cat['ammonia__fo'][order], cat['ammonia__Io'][order]
    cat['ammonia__gammaNH3o'] = cat['ammonia__gammaNH3o'][order]
    floors = [_inversion(cat, T, P, c)[3] for c in (O.HS_INV_LO, O.HS_INV_HI)]
    wide = all(fl >= 0.32 * fo.max() for fl in floors)
    S = Io / np.square(fo)
    smax = S.max()
    got = np.empty(len(freqs))
    ref = np.empty(len(freqs))
    for lo_set in (True, False):        # coefficient set by frequency (30 GHz)
        sel = freqs <= O.F_SPLIT if lo_set else freqs > O.F_SPLIT
        g, z, d, _ = _inversion(cat, T, P, O.HS_INV_LO if lo_set else O.HS_INV_HI)
        r = br_records(fo, g, z, d, S / smax)
        pq = window_quads(fo, freqs, force_fast=wide)[:, sel]
        got[sel] = kernel_sum('br', r, freqs[sel], pq) * smax
        f = freqs[sel]
        ref[sel] = np.sum(Io[:, None] * O._ben_reuven_hs(f[None, :], fo[:, None], g[:, None],
                                                         z[:, None], d[:, None]), axis=0) \
            * np.pi / (2.0 * np.square(f))
    np.testing.assert_allclose(got, ref, rtol=1e-6)


@pytest.mark.parametrize('grid', sorted(GRIDS))
@pytest.mark.parametrize('band', ['rot', 'v2'])
@pytest.mark.parametrize('T,P', LAYERS)
def test_gross_line_sums_match_the_oracle(grid, band, T, P):
    """The Gross families: rotational lines with per-line widths
    (nh3_hs.py:232-265) and nu2 lines with fixed widths (nh3_hs.py:269-302)."""
    freqs = GRIDS[grid]
    cat = _cat()
    Td = 300.0 / T
    if band == 'rot':
        order = np.argsort(cat['ammonia__fo_rot'], kind='stable')
        fo, Io = cat['ammonia__fo_rot'][order], cat['ammonia__Io_rot'][order]
        eH2, eHe, eNH3 = O.HS_ROT['eta']
        nH2, nHe, nNH3 = O.HS_ROT['gnu']
        g = (nH2 * P * XH2 * cat['ammonia__gH2_rot'][order]) * Td ** eH2 \
            + (nHe * P * XHE * cat['ammonia__gHe_rot'][order]) * Td ** eHe \
            + (nNH3 * P * XNH3 * cat['ammonia__gNH3_rot'][order]) * Td ** eNH3
    else:
        order = np.argsort(cat['ammonia__fo_v2'], kind='stable')
        fo, Io = cat['ammonia__fo_v2'][order], cat['ammonia__Io_v2'][order]
        eH2, eHe, eNH3 = O.HS_V2['eta']
        wH2, wHe, wNH3 = O.HS_V2['width']
        g = np.full_like(fo, (P * XH2 * wH2) * Td ** eH2 + (P * XHE * wHe) * Td ** eHe
                         + (P * XNH3 * wNH3) * Td ** eNH3)
    smax = Io.max()
    r = gross_records(fo, g, Io / smax)
    got = kernel_sum('gross', r, freqs, window_quads(fo, freqs)) * smax
    ref = np.sum(Io[:, None] * O._gross(freqs[None, :], fo[:, None], g[:, None]), axis=0) \
        * np.pi / (4.0 * np.square(freqs))
    np.testing.assert_allclose(got, ref, rtol=1e-6)


@pytest.mark.parametrize('grid', sorted(GRIDS))
@pytest.mark.parametrize('gas', ['h2s', 'ph3'])
@pytest.mark.parametrize('T,P', LAYERS)
def test_geisa_line_sums_match_the_oracle(grid, gas, T, P):
    """h2s_ddb (zeta = gamma, a constant pressure shift; h2s_ddb.py:74-80)
    and ph3_jh (zeta = delta = 0; ph3_jh.py:95-101) through the oracle's
    _br_geisa, which carries 2 GHZ f^2 / pi outside the kernel's sum."""
    freqs = GRIDS[grid]
    cat = _cat()
    if gas == 'h2s':
        fo, I0, E = cat['h2s__f0'], cat['h2s__I0'], cat['h2s__E']
        T0, Ps = 296.0, P * 1e-5
        g = (T0 / T) ** 0.7 * (1.960 * P * XH2 + 1.200 * P * XHE + cat['h2s__GH2S'] * Ps)
        z, d = g, np.full_like(g, 1.28 * Ps)
        itg = I0 * np.exp(-(1.0 / T - 1.0 / T0) * E * O.HCK)
    else:
        fo, I0, E = cat['ph3__f0'], cat['ph3__I0'], cat['ph3__E']
        T0, Ps = 300.0, P * 5e-6
        g = (T0 / T) ** (2.0 / 3.0) * (3.2930 * P * XH2 + 1.6803 * P * XHE) * cat['ph3wgt__WgtFGB'] \
            + (T0 / T) * 4.2157 * Ps * cat['ph3wgt__WgtSB']
        z = d = np.zeros_like(g)
        itg = I0 * cat['ph3wgt__WgtI0'] * np.exp(-(1.0 / T - 1.0 / T0) * E * O.HCK)
    order = np.argsort(fo, kind='stable')
    fo, g, z, d, itg = fo[order], g[order], z[order], d[order], itg[order]
    S = itg / np.square(fo)
    smax = S.max()
    r = br_records(fo, g, z, d, S / smax)
    got = kernel_sum('br', r, freqs, window_quads(fo, freqs)) * smax
    ref = O._br_geisa(freqs, fo[None, :], g[None, :], z[None, :], d[None, :], itg[None, :])[0] \
        * np.pi / (2.0 * O.GHZ * np.square(freqs))
    np.testing.assert_allclose(got, ref, rtol=1e-6)


def sjs_kernel_sum(fo, G0, S, shift, coef, freqs):
    """The nh3_sjs item (sjs_item): coefficients A..D of
    gamma = A + B G0, zeta = C + D G0 blended per frequency, every line on
    the float-pair form with its own reciprocal, lanes (4q, 4q+2) and
    (4q+1, 4q+3), flushed every 8 quads and at each 128-line chunk's end."""
    shift = f32(shift)
    c2h, c2l = split(np.square(fo))
    KH, e = two_sum32(c2h, (f32(2) * fo.astype(f32) + shift) * shift)
    KL = e + c2l
    mKH, mKL = _pad(-KH, -1e18), _pad(-KL, 0)
    w, st = _pad(np.asarray(G0).astype(f32), 0), _pad(np.asarray(S).astype(f32), 0)
    F, FL = split(np.square(freqs))
    F4 = f32(4) * F
    A, B, C, D = (np.asarray(c).astype(f32) for c in coef)          # [nf] each
    nq = len(w) // 4
    s = np.zeros((2, len(freqs)), f32)
    c = np.zeros_like(s)
    p = np.zeros_like(s)
    for q in range(nq):
        for lane in range(2):
            for i in (4 * q + lane, 4 * q + 2 + lane):
                g = fma32(B, w[i], A)
                z = fma32(D, w[i], C)
                gm = fma32(z, f32(-1), g)
                gp = g + z
                g2z2 = gm * gp
                d1 = fma32(g2z2, f32(-1), (F + mKH[i]) + (FL + mKL[i]))
                den = fma32(d1, d1, F4 * (g * g))
                num = fma32(gm, F, gp * fma32(mKH[i], f32(-1), g2z2))
                p[lane] = fma32(st[i] * num, f32(1) / den, p[lane])
        if q % 8 == 7 or q % 32 == 31 or q == nq - 1:
            y = p - c
            t = s + y
            c = (t - s) - y
            s = t
            p[:] = 0
    return ((s[0] - c[0]) + (s[1] - c[1])).astype(np.float64)


@pytest.mark.parametrize('grid', sorted(GRIDS))
@pytest.mark.parametrize('T,P', LAYERS)
def test_sjs_line_sum_matches_the_oracle(grid, T, P):
    """nh3_sjs (nh3_sjs.py:37-124) against the oracle's alpha_nh3_sjs with
    its layer prefactor and the 2 GHZ f^2 / pi of the shape taken out."""
    freqs = GRIDS[grid]
    cat = _cat()
    sc = {k.split('__')[1]: v for k, v in cat.items() if k.startswith('nh3__')}
    order = np.argsort(sc['f0'], kind='stable')
    sc = {k: v[order] for k, v in sc.items()}
    Ta = np.array([T])
    Ph2, Phe, Pnh3 = P * XH2, P * XHE, P * XNH3
    join, spil = O._sjs_coefficients(Ta, np.array([P]), np.array([Ph2]))
    wJ = np.clip((freqs - 26.0) / 8.0, 0.0, 1.0)          # Spilker <= 26 GHz, Joiner >= 34
    tt = (296.0 / T) ** (2.0 / 3.0)
    blend = {k: spil[k][0] + (join[k][0] - spil[k][0]) * wJ for k in join}
    coef = (tt * (blend['GH2'] * Ph2 + blend['GHe'] * Phe), tt * blend['GNH3'] * Pnh3,
            tt * (blend['ZH2'] * Ph2 + blend['ZHe'] * Phe), tt * blend['ZNH3'] * Pnh3)
    itg = sc['I0'] * np.exp(-(1.0 / T - 1.0 / 296.0) * sc['E'] * O.HCK)
    S = itg / np.square(sc['f0'])
    smax = S.max()
    got = sjs_kernel_sum(sc['f0'], sc['G0'], S / smax, -0.45 * Pnh3, coef, freqs) * smax
    pre = O.GEISA_COEF * (Pnh3 / 296.0) * (296.0 / T) ** 3.5 * (1.0 + P / 1.0e5)
    ref = O.alpha_nh3_sjs(freqs, Ta, np.array([P]), XH2, XHE, XNH3, sc)[0] / pre \
        * np.pi / (2.0 * O.GHZ * np.square(freqs))
    np.testing.assert_allclose(got, ref, rtol=1e-6)


def _water(T, P):
    cat = _cat()
    L = {k.split('__')[1]: v for k, v in cat.items() if k.startswith('h2o__')}
    Th = 300.0 / T
    df = L['w_s'] * P * XH2O * Th ** L['x_s'] + L['w_h2'] * P * XH2 * Th ** L['x_h2'] \
        + L['w_he'] * P * XHE * Th ** L['x_he']
    S = L['I_o'] * Th ** 2.5 * np.exp(L['E_o'] * (1.0 - Th)) / np.square(L['f_o'])
    centre = L['f_o'] + L['SR']
    order = np.argsort(centre, kind='stable')
    return centre[order], df[order], S[order]


@pytest.mark.parametrize('grid', sorted(GRIDS))
@pytest.mark.parametrize('T,P', LAYERS)
def test_water_line_sum_matches_the_oracle(grid, T, P):
    """The two resonant terms of h2o_bk.py:177-187 (oracle alpha_h2o_bk's B
    and Cc), without the 750 GHz base term the kernel adds per layer."""
    freqs = GRIDS[grid]
    centre, df, S = _water(T, P)
    smax = S.max()
    r = vvw_records(centre, df, S / smax)
    got = kernel_sum('vvw', r, freqs, window_quads(centre, freqs)) * smax
    f = freqs[None, :]
    c, w = centre[:, None], df[:, None]
    ref = np.sum(S[:, None] * (w / (np.square(f - c) + w * w) + w / (np.square(f + c) + w * w)),
                 axis=0)
    np.testing.assert_allclose(got, ref, rtol=1e-6)


def test_far_line_form_needs_the_window():
    """Planted in the restatement: every line on the two-operation form.
    Near a narrow line's centre F (F + G4 - 2K) + K^2 cancels: at 0.01 bar
    the inversion sum below 30 GHz then misses the oracle by more than 1e-3,
    where the windowed sum holds the 1e-6 of the tests above."""
    cat = _cat()
    order = np.argsort(cat['ammonia__fo'], kind='stable')
    fo, Io = cat['ammonia__fo'][order], cat['ammonia__Io'][order]
    cat['ammonia__gammaNH3o'] = cat['ammonia__gammaNH3o'][order]
    f = FREQS[FREQS <= O.F_SPLIT]
    g, z, d, _ = _inversion(cat, 110.0, 0.01, O.HS_INV_LO)
    S = Io / np.square(fo)
    r = br_records(fo, g, z, d, S / S.max())
    ref = np.sum(Io[:, None] * O._ben_reuven_hs(f[None, :], fo[:, None], g[:, None], z[:, None],
                                                 d[:, None]), axis=0) * np.pi / (2.0 * f * f)
    err = {}
    for planted in (False, True):
        got = kernel_sum('br', r, f, window_quads(fo, f, force_fast=planted)) * S.max()
        err[planted] = np.max(np.abs(got / ref - 1.0))
    assert err[False] < 1e-6 and err[True] > 1e-3, err


@pytest.mark.parametrize('edge', ['below', 'above'])
def test_far_line_denominator_error_bound(edge):
    """Lines just outside a chain's window (centre 0.75 fmin or 1.3 fmax)
    and narrow (the worst case: no 4 g^2 F term to dominate), over chains
    from 0.3 to 6000 GHz: the record fields and the two operations stay
    within 18 ulp of (F - K)^2 + G4 F evaluated in float64 from the same
    float32 inputs (the cancellation amplifies the terms' roundings by
    ((1 + r^2)/(1 - r^2))^2, r = fo/f, at most ~15 at the window's edges)."""
    rng = np.random.default_rng(11 if edge == 'below' else 12)
    worst = 0.0
    for _ in range(400):
        fmin = 10.0 ** rng.uniform(-0.5, 3.8)
        f = np.sort(fmin * rng.uniform(1.0, 2.0, 32))
        if edge == 'below':
            fo = 0.75 * f[0] * rng.uniform(0.0, 1.0, 64)
        else:
            fo = 1.3 * f[-1] * rng.uniform(1.0, 3.0, 64)
        fo = fo[fo > 0]
        g = fo * 10.0 ** rng.uniform(-7.0, -1.0, fo.size)
        z = g * rng.uniform(-1.0, 1.0, fo.size)
        d = g * rng.uniform(-0.1, 0.1, fo.size)
        r = br_records(fo, g, z, d, np.ones_like(fo))
        n = fo.size
        F, _ = split(np.square(f))
        den = fma32(F[:, None], F[:, None] + r['v0'][None, :n], r['v1'][None, :n])
        K = r['KH'][:n].astype(float) + r['kl'][:n].astype(float)
        Fx = F.astype(float)[:, None]
        exact = np.square(Fx - K[None, :]) + r['G4'][:n].astype(float)[None, :] * Fx
        worst = max(worst, float(np.max(np.abs(den - exact) / exact)))
    assert worst < 18 * ULP, worst / ULP


def test_denominator_products_stay_in_float32_range():
    """Frequencies and line centres up to 2e4 GHz (the bounds the C ABI
    accepts) with widths up to 3000 GHz: the paired product dP dQ of two
    denominators and the numerator stay finite in float32 with a margin of
    more than two decades."""
    fmax = 2.0e4
    F = f32(fmax * fmax)
    worst = 0.0
    for fo in (1e-3, 1.0, fmax):
        for g in (1e-6, 3e3):
            r = br_records(np.array([fo]), np.array([g]), np.array([g]), np.array([0.0]),
                           np.array([1.0]))
            den = float(fma32(F, F + r['v0'][0], r['v1'][0]))
            num = float(fma32(r['a'][0], F, r['b'][0]))
            worst = max(worst, den * den, num * den)
    assert worst < np.finfo(f32).max / 100.0


def test_compensated_block_sums():
    """The kernel's accumulator: a plain float32 sum per lane over a block of
    64 lines (16 two-line terms), blocks added with Kahan compensation.
    For positive terms its error stays within ~(16 + 2) units of roundoff
    of the exact sum, where one float32 running sum over 2233 lines can lose
    ~1e3 of them."""
    rng = np.random.default_rng(5)
    for trial in range(20):
        n = 2233
        terms = (10.0 ** rng.uniform(-6.0, 0.0, n) * rng.uniform(0.5, 1.5, n)).astype(f32)
        exact = np.sum(terms.astype(np.float64))
        s = np.zeros(2, f32)
        c = np.zeros(2, f32)
        p = np.zeros(2, f32)
        t2 = np.concatenate([terms, np.zeros((-n) % 4, f32)]).reshape(-1, 2, 2)
        for q in range(t2.shape[0]):
            p = p + (t2[q, :, 0] + t2[q, :, 1])
            if q % 16 == 15 or q == t2.shape[0] - 1:
                y = p - c
                t = s + y
                c = (t - s) - y
                s = t
                p[:] = 0
        got = float((s[0] - c[0]) + (s[1] - c[1]))
        assert abs(got - exact) / exact < 18 * 2.0 ** -24


def kernel_strength(l2I, E, cE, M2, single=False):
    """line_strength: S = 2^(l2I + cE E - M2) with the exponent as a float
    pair (log2 of intensity / centre^2, lower-state energy and the layer's
    cE each split hi/lo, the product's error by fma), split into integer
    and fractional parts before exp2.  single: the exponent in one float32
    (the planted variant)."""
    if single:
        s = (f32(l2I) - f32(M2)) + f32(cE) * f32(E)
        ti = np.rint(s)
        return np.ldexp(np.exp2(s - ti), ti.astype(int)).astype(f32)
    l2Ih, l2Il = split(l2I)
    Eh, El = split(E)
    cEh, cEl = split(cE)
    ph = cEh * Eh
    pl = fma32(cEh, Eh, -ph) + fma32(cEh, El, cEl * Eh)
    s, e = two_sum32(l2Ih - f32(M2), ph)
    lo = (e + pl) + l2Il
    ti = np.rint(s)
    out = np.ldexp(np.exp2((s - ti) + lo), ti.astype(int)).astype(f32)
    return np.where(ti < -140, f32(0), out)


@pytest.mark.parametrize('T', [100.0, 300.0, 1000.0])
@pytest.mark.parametrize('cols', [('ammonia__fo', 'ammonia__Io', 'ammonia__Eo'),
                                  ('ammonia__fo_rot', 'ammonia__Io_rot', 'ammonia__Eo_rot'),
                                  ('nh3__f0', 'nh3__I0', 'nh3__E'), ('h2s__f0', 'h2s__I0', 'h2s__E'),
                                  ('ph3__f0', 'ph3__I0', 'ph3__E')])
def test_line_strength_exponent_as_float_pair(cols, T):
    """Strengths relative to the layer's bound M2 = ceil(max exponent) + 1
    (scale_bound): within 2.5e-7 of float64 (measured 1.0e-7, the exp2
    rounding; CUDA's exp2f adds at most 2 ulp more), where one float32
    exponent loses 2.5e-6 to 8e-6 (exponents down to -170)."""
    cat = _cat()
    fo, I, E = (cat[c] for c in cols)
    l2I = np.log2(I) - 2.0 * np.log2(fo)
    cE = -(1.0 / T - 1.0 / 300.0) * 1.438396 / np.log(2.0)
    M2 = np.ceil(f32(l2I.max() + max(cE * E.min(), cE * E.max()))) + 1.0
    exact = np.exp2(l2I + cE * E - M2)
    ok = exact > 2.0 ** -126
    err = {single: np.max(np.abs(kernel_strength(l2I, E, cE, M2, single)[ok] / exact[ok] - 1.0))
           for single in (False, True)}
    assert err[False] < 2.5e-7 and err[True] > 2e-6, err
