"""CPU: the float64 autograd reference (oracle/torch64.py) is pinned to the
numpy oracle before it checks the GPU's gradients.

* its absorption equals the oracle's (which the reference's own fixtures
  pin) on layers in every nh3_hs_sjs regime: nh3_hs only, the 400-2000 bar
  blend and nh3_sjs only;
* its Tb equals the oracle's scan, for the exp and the 'disc' (E2)
  weighting;
* its gradients agree with central finite differences (step 1e-4) of the
  oracle forward model along random perturbations, in both weightings.
"""
import numpy as np
import pytest

torch = pytest.importorskip('torch')

from oracle import adjoint as A        # noqa: E402
from oracle import oracle as O          # noqa: E402
from oracle import torch64 as T64       # noqa: E402
from radiobear_gb300 import synth       # noqa: E402
from tests import goldio as G           # noqa: E402
from tests.test_adjoint import random_direction   # noqa: E402

LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
C = G.C


def case(nL=36, Pmax=2600.0):
    gas = synth.make_gas_table(nL, 1.0e-2, Pmax)
    prop = synth.compute_properties(gas)
    freqs = np.array([1.4, 5.0, 12.0, 22.2, 24.0, 28.0, 33.0, 44.0, 60.0])
    return gas, prop[LP['R']], prop[LP['N']], freqs, G.c0_lines()


def params(gas):
    lnX = np.log(np.stack([gas[C['NH3']], gas[C['H2O']], gas[C['H2S']]]))
    return gas[C['T']].copy(), gas[C['P']].copy(), lnX


def test_absorption_matches_the_oracle_in_every_nh3_regime():
    gas, R, N, freqs, lines = case()
    P = gas[C['P']]
    assert (P < 400).any() and ((P >= 400) & (P <= 2000)).any() and (P > 2000).any()
    per = O.alpha_per_gas(freqs, gas, C, lines)
    ref, _ = O.total_alpha(per, O.layer_scale(False, gas.shape[1]))
    m = T64.Model(gas, C, lines, freqs)
    T, P, lnX = params(gas)
    got = m.layers(*(torch.as_tensor(v, dtype=torch.float64) for v in (T, P, lnX))).numpy()
    assert np.max(np.abs(got - ref) / np.abs(ref)) < 1e-11


@pytest.mark.parametrize('disc', [False, True])
def test_scan_matches_the_oracle(disc):
    gas, R, N, freqs, lines = case()
    per = O.alpha_per_gas(freqs, gas, C, lines)
    layers, _ = O.total_alpha(per, O.layer_scale(False, gas.shape[1]))
    T = gas[C['T']]
    for b in ([0.0, 0.0], [0.6, 0.2], [0.95, 0.0]):
        ds, lay = O.compute_ds(R, N, b, G.REQ, G.RPOL)
        ref, _, _, _ = O.brightness(ds, lay, layers, T, disc=disc)
        got = T64.scan(torch.as_tensor(layers), torch.as_tensor(T), (ds, lay), disc=disc).numpy()
        assert np.max(np.abs(got - ref)) < 1e-9


@pytest.mark.parametrize('disc', [False, True])
def test_gradients_match_finite_differences(disc):
    gas, R, N, freqs, lines = case(nL=30)
    nb = 1 if disc else 3
    b, w = synth.gauss_legendre_disc(nb)
    if disc:
        b, w = np.zeros((1, 2)), np.ones(1)
    rng = np.random.default_rng(11)
    g = rng.normal(size=freqs.size)
    paths = [O.compute_ds(R, N, bb, G.REQ, G.RPOL) for bb in b]
    m = T64.Model(gas, C, lines, freqs)
    T, P, lnX = params(gas)
    _, _, dT, dP, dX = T64.gradients(m, T, P, lnX, paths, w, g, disc=disc)

    def loss(gg):
        tb, _, _ = O.forward(gg, C, R, N, freqs, b, lines, G.REQ, G.RPOL, disc=disc)
        return float(np.dot(g, np.tensordot(w, tb, axes=1)))

    for _ in range(3):
        d = random_direction(rng, gas)
        h = 1e-4
        fd = (loss(A.perturb(gas, C, d, h)) - loss(A.perturb(gas, C, d, -h))) / (2 * h)
        ad = (np.dot(dT, d['T']) + np.dot(dP, d['P']) + np.dot(dX[0], d['NH3'])
              + np.dot(dX[1], d['H2O']) + np.dot(dX[2], d['H2S']))
        assert abs(ad - fd) <= 2e-6 * abs(fd) + 1e-9, (ad, fd)
