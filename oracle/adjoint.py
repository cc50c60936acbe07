"""CPU checker for the adjoint: float64 reverse sweep of the brightness scan
and finite-difference gradients of the oracle forward model.

TEST INFRASTRUCTURE ONLY (same rule as ``oracle/oracle.py``): imported by
``tests/`` and the accuracy leg of ``bench.py`` as the checker, never by the
``radiobear_gb300`` package.

The reference has no derivatives, so gradients are pinned by (1) central
finite differences of the float64 oracle (``oracle.forward``), step 1e-4
relative, and (2) the reverse sweep below, itself checked against those
finite differences.  The scan it differentiates is ``oracle.brightness``
(brightness.py:53-117, exp weighting):

    tau_{i+1} = tau_i + (a_i + a_{i+1}) d_i / 2,   W_0 = 0,  W_i = a_i exp(-tau_i)
    intW = sum_i (W_i + W_{i+1}) d_i / 2,  TbL = sum_i (T_i W_i + T_{i+1} W_{i+1}) d_i / 2
    Tb = TbL / intW  (T_cmb when TbL < T_cmb)
"""
from __future__ import annotations

import numpy as np

from oracle import oracle as O


def brightness_vjp(ds, layer4ds, alpha_layers, T_layers, gTb):
    """Reverse sweep of one ray.  gTb [nf] = d loss / d Tb.  Returns
    (galpha [nf, nL] = d loss / d alpha, gT [nL] = d loss / d T through the
    source term), both accumulated over the layers the ray visits."""
    nf, nL = alpha_layers.shape
    galpha = np.zeros((nf, nL))
    gT = np.zeros(nL)
    if ds is None or len(ds) < 2:
        return galpha, gT
    d = np.asarray(ds[:-1], dtype=np.float64) * 1.0e3 / 1.0e-2
    lay = np.asarray(layer4ds) % nL
    n = len(lay)
    a = alpha_layers[:, lay]                        # [nf, n]
    Tn = T_layers[lay]
    dtau = (a[:, :-1] + a[:, 1:]) * d / 2.0
    tau = np.concatenate([np.zeros((nf, 1)), np.cumsum(dtau, axis=1)], axis=1)
    E = np.exp(-tau)
    E[:, 0] = 0.0                                   # W_0 = 0
    W = a * E
    c = np.zeros(n)
    c[:-1] += d / 2.0
    c[1:] += d / 2.0
    iw = (W * c).sum(axis=1)
    tbl = (W * Tn * c).sum(axis=1)
    live = tbl >= O.T_CMB
    Tb = np.where(live, tbl / np.where(live, iw, 1.0), O.T_CMB)
    g = np.where(live, gTb, 0.0)
    w = c[None, :] * (Tn[None, :] - Tb[:, None]) / np.where(live, iw, 1.0)[:, None]   # dTb/dW_i
    lam = -w * a * E                                # dTb/dtau_i
    Lam = np.cumsum(lam[:, ::-1], axis=1)[:, ::-1]  # sum_{i >= k}
    Lam_next = np.concatenate([Lam[:, 1:], np.zeros((nf, 1))], axis=1)
    dprev = np.concatenate([[0.0], d])
    dcur = np.concatenate([d, [0.0]])
    gA = w * E + 0.5 * dprev[None, :] * Lam * (np.arange(n) >= 1)[None, :] + 0.5 * dcur[None, :] * Lam_next
    src = W * c[None, :] / np.where(live, iw, 1.0)[:, None]
    np.add.at(galpha.T, lay, (g[:, None] * gA).T)
    np.add.at(gT, lay, (g[:, None] * src).sum(axis=0))
    return galpha, gT


def loss_forward(gas, C, R, N, freqs, rays, lines, Req, Rpol, weights, grad, h2state='e',
                 **alpha_kw):
    """sum_f grad[f] Tb_avg[f] of the oracle forward model."""
    _, _, avg = O.forward(gas, C, R, N, freqs, rays, lines, Req, Rpol, weights=weights,
                          h2state=h2state, **alpha_kw)
    return float(np.dot(grad, avg))


PARAMS = ('T', 'P', 'NH3', 'H2O', 'H2S')


def perturb(gas, C, direction, h):
    """gas with T += h dT, P *= (1 + h dP/P ...), ln X += h dlnX.
    direction: dict name -> [nL] (T in K, P in bar, abundances in ln X)."""
    g = np.array(gas, dtype=np.float64, copy=True)
    for name, v in direction.items():
        v = np.asarray(v, dtype=np.float64)
        if name in ('T', 'P'):
            g[C[name]] = g[C[name]] + h * v
        else:
            g[C[name]] = g[C[name]] * np.exp(h * v)
    return g


def directional_fd(gas, C, R, N, freqs, rays, lines, Req, Rpol, weights, grad, direction,
                   h=1e-4, h2state='e', **alpha_kw):
    """Central difference of the loss along `direction` (step h)."""
    lp = loss_forward(perturb(gas, C, direction, h), C, R, N, freqs, rays, lines, Req, Rpol,
                      weights, grad, h2state, **alpha_kw)
    lm = loss_forward(perturb(gas, C, direction, -h), C, R, N, freqs, rays, lines, Req, Rpol,
                      weights, grad, h2state, **alpha_kw)
    return (lp - lm) / (2.0 * h)


def random_direction(rng, gas, C):
    """A perturbation of the benchmark's gradient checks: T Gaussian 5 K, ln X
    of NH3 / H2O / H2S Gaussian 0.3 dex correlated over 5 layers (a 5-layer
    moving average rescaled to the same variance), P Gaussian 1 %."""
    nL = gas.shape[1]
    k = np.ones(5) / 5.0

    def corr(sigma):
        return np.convolve(rng.normal(0.0, sigma, nL + 4), k, mode='valid') * np.sqrt(5.0)

    dex = 0.3 * np.log(10.0)
    return dict(T=rng.normal(0.0, 5.0, nL), P=0.01 * gas[C['P']] * rng.normal(0.0, 1.0, nL),
                NH3=corr(dex), H2O=corr(dex), H2S=corr(dex))


def dot(grad, direction):
    """<gradient, direction> for a gradient dict (dT, dP, dlnX [3, nL])."""
    return (np.dot(grad['dT'], direction['T']) + np.dot(grad['dP'], direction['P']) +
            np.dot(grad['dlnX'][0], direction['NH3']) + np.dot(grad['dlnX'][1], direction['H2O']) +
            np.dot(grad['dlnX'][2], direction['H2S']))
