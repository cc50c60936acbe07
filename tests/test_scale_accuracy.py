"""Accuracy at the benchmarked sizes against the float64 oracle
(``oracle/accuracy.py``), the bar of the metric: <= 1 mK in Tb and 1e-5
relative in alpha, gradients against a float64 autograd reference and
central differences.

* C1: every one of the 64 disc rays at all 256 frequencies, the disc
  average, and the whole 1000 x 256 absorption table;
* C2: 256 rays of the 256 x 256 image at 8 frequencies through the
  1000-layer atmosphere, including the 16 longest (limb) paths and the 16
  outermost rays that reach the planet;
* C3: the gradient of a disc-averaged spectrum (1000 layers x 64 freqs x 16
  rays) along 32 random perturbations against torch autograd in float64,
  8 of them against central differences, and the b = 'disc' (E2) gradient;
* C4: 8 sampled variants of the retrieval batch (300..1200 layers, 128
  freqs, 32 rays) in one batched launch: Tb_avg and gradient directions.
"""
import numpy as np
import pytest

from oracle import accuracy as ACC
from oracle import adjoint as A
from oracle import parallel as OP
from radiobear_gb300 import synth
from tests import goldio as G

pytestmark = pytest.mark.gpu

LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
C = G.C
TB_ATOL = 1e-3          # 1 mK, the metric's bar
ALPHA_RTOL = 1e-5
DIR_RTOL = 3e-3         # float32 line sums and tangents against float64
VEC_RTOL = 5e-3


@pytest.fixture(scope='module')
def pool():
    p, _ = OP.make_pool()
    yield p
    p.close()
    p.join()


@pytest.fixture(scope='module')
def engine():
    from radiobear_gb300 import _native
    e = _native.Engine(0)
    yield e
    e.close()


def workload(cfg, engine):
    from radiobear_gb300 import catalog
    from radiobear_gb300._native import x_matrix
    cats = G.real_catalogues()
    wl = synth.make_workload(cfg, real=cats)
    wl['lines']['ph3wgt'] = cats['ph3wgt']
    catalog.upload(engine, wl.lines)
    engine.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    g = wl.gas
    return wl, dict(P=g[C['P']], T=g[C['T']], X=x_matrix(g, C), R=wl.prop[LP['R']], N=wl.prop[LP['N']])


def test_c1_every_ray_and_the_absorption_table(pool, engine):
    wl, a = workload(1, engine)
    out = engine.forward(a['P'], a['T'], a['X'], a['R'], a['N'], wl.freqs, wl.b, G.REQ, G.RPOL,
                         weights=wl.weights, want_layers=True)
    acc = ACC.spectra(pool, wl.freqs, wl.gas, C, a['R'], a['N'], wl.b, wl.weights, wl.lines, G.REQ,
                      G.RPOL, out['Tb'], out['Tb_avg'], out['layers'])
    print('C1 accuracy', acc)
    assert acc['rays'] == 64
    assert acc['max_abs_dTb_K'] < TB_ATOL
    assert acc['max_abs_dTb_avg_K'] < TB_ATOL
    assert acc['alpha_max_rel_err'] < ALPHA_RTOL


def test_c2_image_limb_rays(pool, engine):
    wl, a = workload(2, engine)
    b = np.ascontiguousarray(wl.b)
    r = np.hypot(b[:, 0], b[:, 1])
    on = np.nonzero(r < 1.0)[0]
    rng = np.random.default_rng(5)
    cand = np.union1d(on[r[on] > 0.985], rng.choice(on, 1024, replace=False))
    paths = engine.raypath(a['R'], a['N'], b[cand], G.REQ, G.RPOL)
    sel, longest, outer = ACC.image_sample(b[cand], paths['nseg'])
    idx = cand[sel]
    out = engine.forward(a['P'], a['T'], a['X'], a['R'], a['N'], wl.freqs, b, G.REQ, G.RPOL)
    acc, _, nseg = ACC.image(pool, wl.freqs, wl.gas, C, a['R'], a['N'], b[idx], wl.lines, G.REQ,
                             G.RPOL, out['Tb'][idx])
    print('C2 accuracy', acc)
    assert len(idx) >= 256
    assert np.array_equal(nseg, paths['nseg'][sel])        # same path lengths as the oracle
    assert acc['max_path_segments'] > 1800                  # limb rays are in the sample
    assert acc['max_abs_dTb_K'] < TB_ATOL
    off = r >= 1.0
    assert np.all(out['Tb'][off] == 2.725)


@pytest.mark.parametrize('disc', [False, True])
def test_c3_gradients_at_full_size(pool, engine, disc):
    wl, a = workload(3, engine)
    g = np.random.default_rng(3).normal(size=wl.freqs.size)
    b, w = (np.zeros((1, 2)), np.ones(1)) if disc else (wl.b, wl.weights)
    out = engine.adjoint(a['P'], a['T'], a['X'], a['R'], a['N'], wl.freqs, b, G.REQ, G.RPOL, g,
                         weights=w, disc=disc)
    acc = ACC.gradients(pool, wl.freqs, wl.gas, C, a['R'], a['N'], wl.b, wl.weights, wl.lines,
                        G.REQ, G.RPOL, out, g, n_dir=32, n_fd=8 if not disc else 4, device='cuda',
                        disc=disc)
    print('C3 gradient accuracy (disc={})'.format(disc), acc)
    assert acc['fp64_autograd_vs_central_differences'] < 1e-5      # the two references agree
    assert acc['dir_rel_err_vs_fp64_autograd'] < DIR_RTOL
    assert acc['dir_rel_err_vs_central_differences'] < DIR_RTOL
    assert max(acc['layer_grad_max_err_rel'].values()) < VEC_RTOL


def test_c4_sampled_variants_in_one_batch(pool, engine):
    """8 variants spread over the 300..1200-layer range, batched exactly as
    the C4 step (one rb_adjoint_batch_device), each against the oracle."""
    import torch
    from radiobear_gb300 import catalog
    from radiobear_gb300._native import x_matrix
    cats = G.real_catalogues()
    lines = dict(synth.make_workload(0, real=cats).lines)
    lines['ph3wgt'] = cats['ph3wgt']
    catalog.upload(engine, lines)
    engine.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    nLs, nh3, dT = synth.make_variants(4096)
    pick = np.argsort(nLs)[np.linspace(0, 4095, 8).astype(int)]
    freqs = np.logspace(np.log10(0.5), np.log10(50.0), 128)
    b, w = synth.gauss_legendre_disc(32)
    vs = []
    for i in pick:
        gas = synth.make_gas_table(int(nLs[i]), 1.0e-3, 100.0, nh3_deep=nh3[i], dT_deep=dT[i])
        pr = synth.compute_properties(gas)
        vs.append((gas, pr[LP['R']], pr[LP['N']]))
    dev = torch.device('cuda')
    f64 = dict(dtype=torch.float64, device=dev)

    def cat(f):
        return torch.tensor(np.ascontiguousarray(np.concatenate([f(v) for v in vs], axis=-1)), **f64)

    t = dict(P=cat(lambda v: v[0][C['P']]), T=cat(lambda v: v[0][C['T']]),
             X=cat(lambda v: x_matrix(v[0], C)), R=cat(lambda v: v[1]), N=cat(lambda v: v[2]))
    nl = [v[0].shape[1] for v in vs]
    NLT = sum(nl)
    grad = np.random.default_rng(4).normal(size=(len(vs), freqs.size))
    tg = torch.tensor(grad, **f64)
    avg = torch.empty((len(vs), freqs.size), **f64)
    gT, gP, gX = torch.empty(NLT, **f64), torch.empty(NLT, **f64), torch.empty((3, NLT), **f64)
    engine.adjoint_batch_device(torch.cuda.current_stream().cuda_stream, nl, t['P'].data_ptr(),
                                t['T'].data_ptr(), t['X'].data_ptr(), t['R'].data_ptr(),
                                t['N'].data_ptr(), freqs, torch.tensor(b, **f64),
                                torch.tensor(w, **f64).data_ptr(), tg.data_ptr(), avg.data_ptr(),
                                gT.data_ptr(), gP.data_ptr(), gX.data_ptr(), G.REQ, G.RPOL)
    torch.cuda.synchronize()
    avg, gT, gP, gX = avg.cpu().numpy(), gT.cpu().numpy(), gP.cpu().numpy(), gX.cpu().numpy()
    o = 0
    worst_tb, worst_dir = 0.0, 0.0
    for v, (gas, R, N) in enumerate(vs):
        n = gas.shape[1]
        layers = OP.layers(pool, freqs, gas, C, lines)
        tb, _ = OP.rays(pool, R, N, b, G.REQ, G.RPOL, layers, gas[C['T']])
        worst_tb = max(worst_tb, float(np.max(np.abs(avg[v] - np.tensordot(w, tb, axes=1)))))
        got = dict(dT=gT[o:o + n], dP=gP[o:o + n], dlnX=gX[:, o:o + n])
        rng = np.random.default_rng(100 + v)
        dirs = [A.random_direction(rng, gas, C)]
        fd = OP.directional_fd(pool, gas, C, R, N, freqs, b, lines, G.REQ, G.RPOL, w, grad[v], dirs)
        worst_dir = max(worst_dir, float(abs(A.dot(got, dirs[0]) - fd[0]) / abs(fd[0])))
        o += n
    print('C4 sampled variants: max |dTb_avg| {:.2e} K, max directional rel err {:.2e}'.format(
        worst_tb, worst_dir))
    assert worst_tb < TB_ATOL
    assert worst_dir < DIR_RTOL
