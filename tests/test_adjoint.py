"""Adjoint: dTb/dT, dTb/dP and dTb/dln X per layer.

The reference has no derivatives ("parity unpinned" for gradients); the
gradient of loss = sum_f g_f Tb_avg(f) is pinned by central finite
differences (step 1e-4) of the float64 oracle forward model, along random
perturbations of the layer parameters (T Gaussian 5 K, ln X Gaussian 0.3
dex correlated over 5 layers, P Gaussian 1 %) and along single layer
parameters.  The scan's reverse sweep is checked on CPU against finite
differences of the oracle's brightness scan.
"""
import numpy as np
import pytest

from oracle import adjoint as A
from oracle import oracle as O
from radiobear_gb300 import synth
from tests import goldio as G

LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
C = G.C

# Directional derivatives: float32 absorption and float32 tangent sums
# against float64 finite differences.
DIR_RTOL = 3e-3
LAYER_RTOL = 1e-2


def small_case(nL=40, Pmax=700.0, nrays=3):
    gas = synth.make_gas_table(nL, 1.0e-2, Pmax)
    prop = synth.compute_properties(gas)
    freqs = np.array([1.4, 5.0, 12.0, 22.2, 24.0, 33.0, 44.0, 60.0])
    b, w = synth.gauss_legendre_disc(nrays)
    return gas, prop[LP['R']], prop[LP['N']], freqs, b, w, G.c0_lines()


def random_direction(rng, gas):
    return A.random_direction(rng, gas, C)


def dot(grad, direction):
    return A.dot(grad, direction)


def test_brightness_vjp_matches_finite_differences():
    """CPU: the reverse sweep of the scan against central differences."""
    z = G.load('c0')
    g = G.gas_table(z)
    nL = g.shape[1]
    rng = np.random.default_rng(7)
    alpha = z['alpha_layers']
    T = g[C['T']]
    ds = z['ray0_ds']
    lay = z['ray0_layer']
    nf = alpha.shape[0]
    gTb = rng.normal(size=nf)
    ga, gT = A.brightness_vjp(ds, lay, alpha, T, gTb)

    def loss(al, TT):
        tb, _, _, _ = O.brightness(ds, lay, al, TT)
        return float(np.dot(gTb, tb))

    for (f, L) in [(0, 10), (3, 60), (7, 120), (12, 180), (20, nL - 1)]:
        h = 1e-5 * np.max(alpha[f])
        ap, am = alpha.copy(), alpha.copy()
        ap[f, L] += h
        am[f, L] -= h
        fd = (loss(ap, T) - loss(am, T)) / (2 * h)
        assert abs(ga[f, L] - fd) <= 2e-6 * abs(fd) + 1e-7 * np.max(np.abs(ga[f])), (f, L, ga[f, L], fd)
    # source term: T enters only through the weighting of the emission
    for L in (5, 50, 150):
        Tp, Tm = T.copy(), T.copy()
        Tp[L] += 1e-3
        Tm[L] -= 1e-3
        fd = (loss(alpha, Tp) - loss(alpha, Tm)) / 2e-3
        assert abs(gT[L] - fd) <= 1e-6 * abs(fd) + 1e-7 * np.max(np.abs(gT)), (L, gT[L], fd)


@pytest.fixture(scope='module')
def engine():
    from radiobear_gb300 import _native
    e = _native.Engine(0)
    yield e
    e.close()


@pytest.fixture(scope='module')
def case():
    return small_case()


def _run(engine, case, grad):
    from radiobear_gb300 import catalog
    from radiobear_gb300._native import x_matrix
    gas, R, N, freqs, b, w, lines = case
    catalog.upload(engine, lines)
    engine.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    return engine.adjoint(gas[C['P']], gas[C['T']], x_matrix(gas, C), R, N, freqs, b, G.REQ,
                          G.RPOL, grad, weights=w)


@pytest.mark.gpu
def test_adjoint_forward_matches_oracle(engine, case):
    gas, R, N, freqs, b, w, lines = case
    grad = np.ones(freqs.size)
    out = _run(engine, case, grad)
    tbs, _, avg = O.forward(gas, C, R, N, freqs, b, lines, G.REQ, G.RPOL, weights=w)
    assert np.max(np.abs(out['Tb'] - tbs)) < 1e-3
    assert np.max(np.abs(out['Tb_avg'] - avg)) < 1e-3


@pytest.mark.gpu
def test_adjoint_directional_derivatives(engine, case):
    """32 random perturbations: <gradient, direction> against central
    differences of the float64 oracle."""
    gas, R, N, freqs, b, w, lines = case
    rng = np.random.default_rng(3)
    grad = rng.normal(size=freqs.size)
    out = _run(engine, case, grad)
    errs = []
    for k in range(32):
        d = random_direction(rng, gas)
        fd = A.directional_fd(gas, C, R, N, freqs, b, lines, G.REQ, G.RPOL, w, grad, d, h=1e-4)
        ad = dot(out, d)
        errs.append(abs(ad - fd) / max(abs(fd), 1e-9))
        assert abs(ad - fd) <= DIR_RTOL * abs(fd) + 1e-7, (k, ad, fd)
    print('directional rel err max', max(errs))


@pytest.mark.gpu
@pytest.mark.parametrize('param', ['T', 'P', 'NH3', 'H2O', 'H2S'])
def test_adjoint_single_layers(engine, case, param):
    gas, R, N, freqs, b, w, lines = case
    nL = gas.shape[1]
    rng = np.random.default_rng(11)
    grad = rng.normal(size=freqs.size)
    out = _run(engine, case, grad)
    key = {'T': out['dT'], 'P': out['dP'], 'NH3': out['dlnX'][0], 'H2O': out['dlnX'][1],
           'H2S': out['dlnX'][2]}[param]
    scale = np.max(np.abs(key)) + 1e-30
    for L in (3, 15, 27, nL - 3, nL - 1):
        v = np.zeros(nL)
        v[L] = 1.0 if param != 'P' else gas[C['P'], L] * 1e-2
        fd = A.directional_fd(gas, C, R, N, freqs, b, lines, G.REQ, G.RPOL, w, grad, {param: v},
                              h=1e-4 if param != 'T' else 1e-3)
        ad = key[L] * v[L]
        assert abs(ad - fd) <= LAYER_RTOL * abs(fd) + 1e-4 * scale * abs(v[L]), (param, L, ad, fd)


@pytest.mark.gpu
def test_adjoint_modes_agree(engine, case):
    """The stored-tangent adjoint (the JVP before the scan gives alpha and
    stores d alpha / d theta) against the recomputing one (forward line
    sums, JVP contracted after the reverse sweep): the same JVP arithmetic,
    alpha from two float32 kernels."""
    gas, R, N, freqs, b, w, lines = case
    grad = np.random.default_rng(5).normal(size=freqs.size)
    try:
        engine.set_tuning(adj_mode=1)
        st = _run(engine, case, grad)
        engine.set_tuning(adj_mode=2)
        rc = _run(engine, case, grad)
    finally:
        engine.set_tuning(adj_mode=0)
    assert np.max(np.abs(st['Tb'] - rc['Tb'])) < 2e-4
    assert np.max(np.abs(st['Tb_avg'] - rc['Tb_avg'])) < 2e-4
    for k in ('dT', 'dP', 'dlnX'):
        scale = np.max(np.abs(rc[k]))
        assert np.max(np.abs(st[k] - rc[k])) <= 1e-4 * scale, (k, np.max(np.abs(st[k] - rc[k])), scale)


@pytest.mark.gpu
def test_autograd_function(engine, case):
    """torch.autograd through TbFunction: forward equals rb_forward, the
    gradient equals rb_adjoint and a finite difference of the oracle."""
    import torch
    from radiobear_gb300 import catalog
    from radiobear_gb300._native import x_matrix
    from radiobear_gb300.autograd import TbModel
    gas, R, N, freqs, b, w, lines = case
    catalog.upload(engine, lines)
    engine.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    X = x_matrix(gas, C)
    model = TbModel(engine, R, N, freqs, b, w, X, G.REQ, G.RPOL)
    dev = torch.device('cuda')
    T = torch.tensor(gas[C['T']], dtype=torch.float64, device=dev, requires_grad=True)
    P = torch.tensor(gas[C['P']], dtype=torch.float64, device=dev, requires_grad=True)
    lnX = torch.tensor(np.log(np.stack([gas[C['NH3']], gas[C['H2O']], gas[C['H2S']]])),
                       dtype=torch.float64, device=dev, requires_grad=True)
    rng = np.random.default_rng(5)
    gw = rng.normal(size=freqs.size)
    avg = model(T, P, lnX)
    loss = (avg * torch.tensor(gw, dtype=torch.float64, device=dev)).sum()
    loss.backward()
    ref = _run(engine, case, gw)
    fwd = engine.forward(gas[C['P']], gas[C['T']], X, R, N, freqs, b, G.REQ, G.RPOL, weights=w)
    np.testing.assert_allclose(avg.detach().cpu().numpy(), fwd['Tb_avg'], rtol=0, atol=1e-9)
    # the stored-tangent adjoint's own forward takes alpha from the JVP
    # kernel (float32 sums in another order): within rounding of rb_forward
    np.testing.assert_allclose(avg.detach().cpu().numpy(), ref['Tb_avg'], rtol=0, atol=2e-4)
    # the adjoint's layer sums are float32 atomics: run-to-run rounding ~1e-7
    for got, want in ((T.grad, ref['dT']), (P.grad, ref['dP']), (lnX.grad, ref['dlnX'])):
        np.testing.assert_allclose(got.cpu().numpy(), want, rtol=1e-5, atol=1e-6 * np.max(np.abs(want)))
    d = random_direction(rng, gas)
    fd = A.directional_fd(gas, C, R, N, freqs, b, lines, G.REQ, G.RPOL, w, gw, d, h=1e-4)
    ad = dot(dict(dT=T.grad.cpu().numpy(), dP=P.grad.cpu().numpy(), dlnX=lnX.grad.cpu().numpy()), d)
    assert abs(ad - fd) <= DIR_RTOL * abs(fd) + 1e-7


def _torch64_grad(case, grad, disc=False, device='cpu'):
    from oracle import torch64 as T64
    gas, R, N, freqs, b, w, lines = case
    if disc:
        b, w = np.zeros((1, 2)), np.ones(1)
    paths = [O.compute_ds(R, N, bb, G.REQ, G.RPOL) for bb in b]
    m = T64.Model(gas, C, lines, freqs, device=device)
    lnX = np.log(np.stack([gas[C['NH3']], gas[C['H2O']], gas[C['H2S']]]))
    tb, loss, dT, dP, dX = T64.gradients(m, gas[C['T']], gas[C['P']], lnX, paths, w, grad, disc=disc)
    return dict(Tb=tb, dT=dT, dP=dP, dlnX=dX)


def _vec_err(got, ref):
    """max |got - ref| over the layers, relative to max |ref|, per parameter."""
    out = {}
    for k, (a, r) in dict(T=(got['dT'], ref['dT']), P=(got['dP'], ref['dP']),
                          NH3=(got['dlnX'][0], ref['dlnX'][0]), H2O=(got['dlnX'][1], ref['dlnX'][1]),
                          H2S=(got['dlnX'][2], ref['dlnX'][2])).items():
        out[k] = float(np.max(np.abs(a - r)) / max(np.max(np.abs(r)), 1e-300))
    return out


# Per-layer gradient vectors against the float64 autograd reference: the
# device's float32 line sums and tangents give ~1e-4 of the largest entry.
VEC_RTOL = 2e-3


@pytest.mark.gpu
def test_adjoint_against_fp64_autograd(engine, case):
    """Every layer's dTb/dT, dTb/dP, dTb/dlnX against torch autograd of the
    float64 restatement (oracle/torch64.py), and 32 directional derivatives."""
    gas, R, N, freqs, b, w, lines = case
    rng = np.random.default_rng(21)
    grad = rng.normal(size=freqs.size)
    out = _run(engine, case, grad)
    ref = _torch64_grad(case, grad)
    errs = _vec_err(out, ref)
    print('per-parameter max err / max |grad|', errs)
    assert max(errs.values()) < VEC_RTOL, errs
    for _ in range(32):
        d = random_direction(rng, gas)
        ad, rd = dot(out, d), dot(ref, d)
        assert abs(ad - rd) <= DIR_RTOL * abs(rd) + 1e-7, (ad, rd)


@pytest.mark.gpu
def test_disc_mode_adjoint(engine, case):
    """b = 'disc' (nadir ray, 2 E2(tau) weighting, brightness.py:96): the
    gradient against the float64 autograd reference (dE2/dx = -E1 from
    scipy) and against central differences of the oracle's disc forward."""
    from radiobear_gb300 import catalog
    from radiobear_gb300._native import x_matrix
    gas, R, N, freqs, b, w, lines = case
    catalog.upload(engine, lines)
    engine.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    rng = np.random.default_rng(8)
    grad = rng.normal(size=freqs.size)
    out = engine.adjoint(gas[C['P']], gas[C['T']], x_matrix(gas, C), R, N, freqs, np.zeros((1, 2)),
                         G.REQ, G.RPOL, grad, weights=np.ones(1), disc=True)
    tb_ref, _, _ = O.forward(gas, C, R, N, freqs, np.zeros((1, 2)), lines, G.REQ, G.RPOL, disc=True)
    assert np.max(np.abs(out['Tb'] - tb_ref)) < 1e-3
    ref = _torch64_grad(case, grad, disc=True)
    errs = _vec_err(out, ref)
    print('disc: per-parameter max err / max |grad|', errs)
    assert max(errs.values()) < VEC_RTOL, errs

    def loss(gg):
        tb, _, _ = O.forward(gg, C, R, N, freqs, np.zeros((1, 2)), lines, G.REQ, G.RPOL, disc=True)
        return float(np.dot(grad, tb[0]))

    for _ in range(4):
        d = random_direction(rng, gas)
        fd = (loss(A.perturb(gas, C, d, 1e-4)) - loss(A.perturb(gas, C, d, -1e-4))) / 2e-4
        ad = dot(out, d)
        assert abs(ad - fd) <= DIR_RTOL * abs(fd) + 1e-7, (ad, fd)


@pytest.mark.gpu
def test_autograd_function_disc(engine, case):
    """TbFunction with disc=True equals rb_adjoint with disc = 1."""
    import torch
    from radiobear_gb300 import catalog
    from radiobear_gb300._native import x_matrix
    from radiobear_gb300.autograd import TbModel
    gas, R, N, freqs, b, w, lines = case
    catalog.upload(engine, lines)
    engine.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    X = x_matrix(gas, C)
    model = TbModel(engine, R, N, freqs, np.zeros((1, 2)), np.ones(1), X, G.REQ, G.RPOL, disc=True)
    dev = torch.device('cuda')
    T = torch.tensor(gas[C['T']], dtype=torch.float64, device=dev, requires_grad=True)
    P = torch.tensor(gas[C['P']], dtype=torch.float64, device=dev, requires_grad=True)
    lnX = torch.tensor(np.log(np.stack([gas[C['NH3']], gas[C['H2O']], gas[C['H2S']]])),
                       dtype=torch.float64, device=dev, requires_grad=True)
    gw = np.random.default_rng(2).normal(size=freqs.size)
    avg = model(T, P, lnX)
    (avg * torch.tensor(gw, dtype=torch.float64, device=dev)).sum().backward()
    ref = engine.adjoint(gas[C['P']], gas[C['T']], X, R, N, freqs, np.zeros((1, 2)), G.REQ, G.RPOL,
                         gw, weights=np.ones(1), disc=True)
    fwd = engine.forward(gas[C['P']], gas[C['T']], X, R, N, freqs, np.zeros((1, 2)), G.REQ, G.RPOL,
                         weights=np.ones(1), disc=True)
    np.testing.assert_allclose(avg.detach().cpu().numpy(), fwd['Tb_avg'], rtol=0, atol=1e-9)
    # the stored-tangent adjoint's alpha comes from the JVP kernel
    np.testing.assert_allclose(avg.detach().cpu().numpy(), ref['Tb_avg'], rtol=0, atol=2e-4)
    for got, want in ((T.grad, ref['dT']), (P.grad, ref['dP']), (lnX.grad, ref['dlnX'])):
        np.testing.assert_allclose(got.cpu().numpy(), want, rtol=1e-5, atol=1e-6 * np.max(np.abs(want)))
