"""Batches of atmospheres: one call over variants with different layer
counts equals one call per variant (same kernels, same arithmetic; the
adjoint's sums over rays and frequencies are float32 atomics, so gradients
agree to float32 rounding of those sums, ~1e-6 relative)."""
import numpy as np
import pytest

from radiobear_gb300 import synth
from tests import goldio as G

pytestmark = pytest.mark.gpu

LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
C = G.C


def variants():
    out = []
    for nL, Pmax, nh3, dT in ((40, 700.0, 3e-4, 0.0), (23, 90.0, 8e-4, 6.0), (31, 450.0, 1.5e-4, -8.0)):
        gas = synth.make_gas_table(nL, 1.0e-2, Pmax, nh3_deep=nh3, dT_deep=dT)
        prop = synth.compute_properties(gas)
        out.append((gas, prop[LP['R']], prop[LP['N']]))
    return out


@pytest.fixture(scope='module')
def setup():
    import torch
    from radiobear_gb300 import _native, catalog
    from radiobear_gb300._native import x_matrix
    e = _native.Engine(0)
    catalog.upload(e, G.c0_lines())
    e.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    vs = variants()
    freqs = np.array([1.4, 5.0, 12.0, 22.2, 24.0, 33.0, 44.0, 60.0])
    b, w = synth.gauss_legendre_disc(4)
    dev = torch.device('cuda')

    def cat(k):
        return np.concatenate([g[C[k]] for g, _, _ in vs])

    arrays = dict(P=cat('P'), T=cat('T'), X=np.concatenate([x_matrix(g, C) for g, _, _ in vs], axis=1),
                  R=np.concatenate([r for _, r, _ in vs]), N=np.concatenate([n for _, _, n in vs]))
    t = {k: torch.tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev) for k, v in arrays.items()}
    t['b'] = torch.tensor(b, dtype=torch.float64, device=dev)
    t['w'] = torch.tensor(w, dtype=torch.float64, device=dev)
    yield e, vs, freqs, b, w, t, [g.shape[1] for g, _, _ in vs]
    e.close()


def test_forward_batch_equals_single(setup):
    import torch
    from radiobear_gb300._native import x_matrix
    e, vs, freqs, b, w, t, nl = setup
    avg = torch.empty((len(vs), freqs.size), dtype=torch.float64, device='cuda')
    s = torch.cuda.current_stream().cuda_stream
    e.forward_batch_device(s, nl, t['P'].data_ptr(), t['T'].data_ptr(), t['X'].data_ptr(),
                           t['R'].data_ptr(), t['N'].data_ptr(), freqs, t['b'], t['w'].data_ptr(),
                           avg.data_ptr(), G.REQ, G.RPOL)
    torch.cuda.synchronize()
    got = avg.cpu().numpy()
    for v, (gas, R, N) in enumerate(vs):
        ref = e.forward(gas[C['P']], gas[C['T']], x_matrix(gas, C), R, N, freqs, b, G.REQ, G.RPOL,
                        weights=w, want_rays=False)['Tb_avg']
        assert np.max(np.abs(got[v] - ref)) <= 1e-9, (v, got[v], ref)


def test_adjoint_batch_equals_single(setup):
    import torch
    from radiobear_gb300._native import x_matrix
    e, vs, freqs, b, w, t, nl = setup
    NLT = sum(nl)
    rng = np.random.default_rng(2)
    grad = rng.normal(size=(len(vs), freqs.size))
    g = torch.tensor(grad, dtype=torch.float64, device='cuda')
    avg = torch.empty((len(vs), freqs.size), dtype=torch.float64, device='cuda')
    dT, dP = (torch.empty(NLT, dtype=torch.float64, device='cuda') for _ in range(2))
    dX = torch.empty((3, NLT), dtype=torch.float64, device='cuda')
    s = torch.cuda.current_stream().cuda_stream
    e.adjoint_batch_device(s, nl, t['P'].data_ptr(), t['T'].data_ptr(), t['X'].data_ptr(),
                           t['R'].data_ptr(), t['N'].data_ptr(), freqs, t['b'], t['w'].data_ptr(),
                           g.data_ptr(), avg.data_ptr(), dT.data_ptr(), dP.data_ptr(), dX.data_ptr(),
                           G.REQ, G.RPOL)
    torch.cuda.synchronize()
    dT, dP, dX = dT.cpu().numpy(), dP.cpu().numpy(), dX.cpu().numpy()
    o = 0
    for v, (gas, R, N) in enumerate(vs):
        n = gas.shape[1]
        ref = e.adjoint(gas[C['P']], gas[C['T']], x_matrix(gas, C), R, N, freqs, b, G.REQ, G.RPOL,
                        grad[v], weights=w)
        for got, want in ((dT[o:o + n], ref['dT']), (dP[o:o + n], ref['dP']), (dX[:, o:o + n], ref['dlnX'])):
            scale = np.max(np.abs(want)) + 1e-300
            assert np.max(np.abs(got - want)) <= 1e-6 * scale, (v, np.max(np.abs(got - want)), scale)
        assert np.max(np.abs(avg.cpu().numpy()[v] - ref['Tb_avg'])) <= 1e-9
        o += n


def _variant_scales(nl):
    """Per-variant scale tables [sum nL][RB_NGAS]: variant 0 unscaled, 1 a
    per-gas dict (nh3 ramp, h2o x2), 2 a per-layer list (the reference's
    scale forms, alpha.py:235-259, one walker each)."""
    from radiobear_gb300 import _native
    ng = len(_native.GASES)
    out = []
    for v, n in enumerate(nl):
        s = np.ones((n, ng))
        if v == 1:
            s[:, _native.GASES.index('nh3')] = np.linspace(0.5, 1.5, n)
            s[:, _native.GASES.index('h2o')] = 2.0
        elif v == 2:
            s *= np.linspace(0.8, 1.3, n)[:, None]
        out.append(s)
    return out


def test_batches_with_per_variant_scale(setup):
    """scripts/demo_batch.py:24-41 reruns one atmosphere with different scale
    dicts; here every variant of a batch carries its own scale table, and
    the batch equals one scaled call per variant (forward and adjoint)."""
    import torch
    from radiobear_gb300._native import x_matrix
    e, vs, freqs, b, w, t, nl = setup
    NLT = sum(nl)
    scales = _variant_scales(nl)
    sc = torch.tensor(np.ascontiguousarray(np.concatenate(scales)), dtype=torch.float64, device='cuda')
    s = torch.cuda.current_stream().cuda_stream
    avg = torch.empty((len(vs), freqs.size), dtype=torch.float64, device='cuda')
    e.forward_batch_device(s, nl, t['P'].data_ptr(), t['T'].data_ptr(), t['X'].data_ptr(),
                           t['R'].data_ptr(), t['N'].data_ptr(), freqs, t['b'], t['w'].data_ptr(),
                           avg.data_ptr(), G.REQ, G.RPOL, scale=sc.data_ptr())
    grad = np.random.default_rng(9).normal(size=(len(vs), freqs.size))
    g = torch.tensor(grad, dtype=torch.float64, device='cuda')
    avg2 = torch.empty_like(avg)
    dT, dP = (torch.empty(NLT, dtype=torch.float64, device='cuda') for _ in range(2))
    dX = torch.empty((3, NLT), dtype=torch.float64, device='cuda')
    e.adjoint_batch_device(s, nl, t['P'].data_ptr(), t['T'].data_ptr(), t['X'].data_ptr(),
                           t['R'].data_ptr(), t['N'].data_ptr(), freqs, t['b'], t['w'].data_ptr(),
                           g.data_ptr(), avg2.data_ptr(), dT.data_ptr(), dP.data_ptr(), dX.data_ptr(),
                           G.REQ, G.RPOL, scale=sc.data_ptr())
    torch.cuda.synchronize()
    got, got2 = avg.cpu().numpy(), avg2.cpu().numpy()
    dT, dP, dX = dT.cpu().numpy(), dP.cpu().numpy(), dX.cpu().numpy()
    o = 0
    unscaled = e.forward(vs[1][0][C['P']], vs[1][0][C['T']], x_matrix(vs[1][0], C), vs[1][1], vs[1][2],
                         freqs, b, G.REQ, G.RPOL, weights=w, want_rays=False)['Tb_avg']
    assert np.max(np.abs(got[1] - unscaled)) > 1e-3          # the scale does act
    for v, (gas, R, N) in enumerate(vs):
        n = gas.shape[1]
        X = x_matrix(gas, C)
        ref = e.forward(gas[C['P']], gas[C['T']], X, R, N, freqs, b, G.REQ, G.RPOL, weights=w,
                        scale=scales[v], want_rays=False)['Tb_avg']
        assert np.max(np.abs(got[v] - ref)) <= 1e-9, v
        # the adjoint's forward (stored-tangent mode) takes alpha from the JVP
        # kernel: within float32 rounding of the forward's line sums
        assert np.max(np.abs(got2[v] - ref)) <= 2e-4, v
        ra = e.adjoint(gas[C['P']], gas[C['T']], X, R, N, freqs, b, G.REQ, G.RPOL, grad[v], weights=w,
                       scale=scales[v])
        assert np.max(np.abs(got2[v] - ra['Tb_avg'])) <= 1e-9, v
        for gg, want in ((dT[o:o + n], ra['dT']), (dP[o:o + n], ra['dP']), (dX[:, o:o + n], ra['dlnX'])):
            assert np.max(np.abs(gg - want)) <= 1e-6 * (np.max(np.abs(want)) + 1e-300), v
        o += n
