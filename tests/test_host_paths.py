"""Host-side execution paths on the GPU:

* the ray set-up one ray per thread (rb_ray_setup_kernel, from 2048 rays
  in a call) against the set-up inside each ray's warp (fewer rays): the
  same float64 arithmetic, so paths must be identical, and the reference's
  fixture rays inside a large batch still match the reference;
* rb_forward / rb_adjoint with host buffers, which replay a captured CUDA
  graph from the second call of a shape on: repeated calls with new inputs
  and a configuration change in between must equal the device-pointer
  entry points (same kernels, no graph) exactly;
* a _device call returns before its kernels run: a host call, or a _device
  call on another stream, made right after it on the same handle waits for
  that work instead of overwriting the workspaces it still uses.
"""
import numpy as np
import pytest

from tests import goldio as G

pytestmark = pytest.mark.gpu

DS_RTOL = 5e-7
SETUP_KERNEL_MIN = 2048   # rays per call from which the set-up kernel runs


@pytest.fixture(scope='module')
def engine():
    from radiobear_gb300 import _native
    e = _native.Engine(0)
    yield e
    e.close()


def _X(g):
    from radiobear_gb300._native import x_matrix
    return x_matrix(g, G.C)


def _load(engine, lines, h2o=True):
    from radiobear_gb300 import catalog
    catalog.upload(engine, lines)
    engine.set_formalisms('nh3_hs_sjs', True, h2o, True, True, 'e')
    engine.set_co_clouds(co=False)


def _ray_batch(z, n):
    """The fixture rays first, then a seeded spread over and around the disc
    (polar limb, misses, off-planet), n rays in all."""
    rng = np.random.default_rng(11)
    fx = np.asarray(z['rays_b'], dtype=float)
    r = np.sqrt(rng.uniform(0.0, 1.1, n - len(fx)))
    t = rng.uniform(0.0, 2 * np.pi, n - len(fx))
    return np.concatenate([fx, np.stack([r * np.cos(t), r * np.sin(t)], axis=1)])


@pytest.mark.parametrize('orientation', [(0.0, 0.0), (10.0, 25.0)])
def test_ray_setup_kernel_equals_warp_setup(engine, orientation):
    z = G.load('c0')
    b = _ray_batch(z, SETUP_KERNEL_MIN + 101)
    big = engine.raypath(z['prop_R'], z['prop_N'], b, G.REQ, G.RPOL, orientation=orientation,
                         extras=True)
    parts = [engine.raypath(z['prop_R'], z['prop_N'], b[i:i + 700], G.REQ, G.RPOL,
                            orientation=orientation, extras=True) for i in range(0, len(b), 700)]
    P = {k: np.concatenate([q[k] for q in parts], axis=0)
         for k in ('nseg', 'end', 'layer', 'ds', 'r4ds', 'latlng')}
    assert np.array_equal(big['nseg'], P['nseg'])
    assert np.array_equal(big['end'], P['end'])
    # entries past a ray's nseg are unspecified; the two kernels compile the
    # same float64 set-up in different contexts (contractions may differ in
    # the last bit) and the walk's float32 steps round from there, so
    # segment lengths agree to the reference tolerance
    for i, n in enumerate(big['nseg']):
        assert np.array_equal(big['layer'][i, :n], P['layer'][i, :n]), i
        for key, m, floor in (('ds', n, 1e-30), ('r4ds', n, 1e-30), ('latlng', n + 1 if n else 0, 1.0)):
            a, p = big[key][i, :m], P[key][i, :m]
            if m:
                err = float(np.max(np.abs(a - p) / np.maximum(np.abs(p), floor)))
                assert err < DS_RTOL, (i, key, err)
    assert (big['nseg'] > 0).sum() > 1000 and (big['nseg'] == 0).sum() > 50


def test_ray_setup_kernel_fixture_rays(engine):
    z = G.load('c0')
    b = _ray_batch(z, SETUP_KERNEL_MIN + 7)
    out = engine.raypath(z['prop_R'], z['prop_N'], b, G.REQ, G.RPOL)
    for i in range(len(z['rays_b'])):
        ref = z['ray{}_ds'.format(i)]
        n = out['nseg'][i]
        assert n == ref.size, (i, n, ref.size)
        if n:
            assert np.array_equal(out['layer'][i, :n], z['ray{}_layer'.format(i)])
            assert np.max(np.abs(out['ds'][i, :n] - ref) / np.abs(ref)) < DS_RTOL


def _device_forward(engine, g, z, freqs, b, w):
    import torch
    dev = torch.device('cuda')
    t = {k: torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev)
         for k, v in dict(P=g[G.C['P']], T=g[G.C['T']], X=_X(g), R=z['prop_R'], N=z['prop_N'],
                          b=b, w=w).items()}
    nL, nb, nf = g.shape[1], len(b), len(freqs)
    Tb = torch.empty((nb, nf), dtype=torch.float64, device=dev)
    avg = torch.empty(nf, dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream()
    engine.forward_device(s.cuda_stream, nL, nb, t['P'].data_ptr(), t['T'].data_ptr(),
                          t['X'].data_ptr(), t['R'].data_ptr(), t['N'].data_ptr(), freqs,
                          t['b'].data_ptr(), G.REQ, G.RPOL, Tb.data_ptr(),
                          weights=t['w'].data_ptr(), Tb_avg=avg.data_ptr())
    s.synchronize()
    return Tb.cpu().numpy(), avg.cpu().numpy()


def test_forward_graph_replay_matches_device_path(engine):
    z, g0 = G.load('c0'), G.gas_table(G.load('c0'))
    lines = G.c0_lines()
    freqs = z['freqs']
    b = np.array([[0.0, 0.0], [0.3, 0.1], [0.0, 0.7], [0.55, -0.4]])
    w = np.array([0.4, 0.3, 0.2, 0.1])
    _load(engine, lines)
    # calls 0-2: direct, captured, replayed; h2o_bk switched off (new
    # configuration): 3-5 the same again; back on: 6 runs directly
    for step, h2o in enumerate([True, True, True, False, False, False, True]):
        if step in (3, 6):
            engine.set_formalisms('nh3_hs_sjs', True, h2o, True, True, 'e')
        g = g0.copy()
        g[G.C['T']] = g0[G.C['T']] * (1.0 + 0.01 * step)
        out = engine.forward(g[G.C['P']], g[G.C['T']], _X(g), z['prop_R'], z['prop_N'], freqs, b,
                             G.REQ, G.RPOL, weights=w)
        Tb, avg = _device_forward(engine, g, z, freqs, b, w)
        assert np.array_equal(out['Tb'], Tb), step
        assert np.array_equal(out['Tb_avg'], avg), step


def test_adjoint_graph_replay_matches_device_path(engine):
    import torch
    z, g = G.load('c0'), G.gas_table(G.load('c0'))
    _load(engine, G.c0_lines())
    freqs = z['freqs']
    b = np.array([[0.0, 0.0], [0.3, 0.1], [0.5, 0.5]])
    w = np.array([0.5, 0.3, 0.2])
    nL, nb, nf = g.shape[1], len(b), len(freqs)
    dev = torch.device('cuda')
    dt = lambda v: torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev)
    tP, tT, tX, tR, tN, tb, tw = (dt(v) for v in (g[G.C['P']], g[G.C['T']], _X(g), z['prop_R'],
                                                   z['prop_N'], b, w))
    rng = np.random.default_rng(3)
    for step in range(4):
        grad = rng.normal(size=nf)
        out = engine.adjoint(g[G.C['P']], g[G.C['T']], _X(g), z['prop_R'], z['prop_N'], freqs, b,
                             G.REQ, G.RPOL, grad, weights=w)
        dT, dP = torch.empty(nL, dtype=torch.float64, device=dev), torch.empty(nL, dtype=torch.float64, device=dev)
        dX = torch.empty((3, nL), dtype=torch.float64, device=dev)
        avg = torch.empty(nf, dtype=torch.float64, device=dev)
        s = torch.cuda.current_stream()
        engine.adjoint_device(s.cuda_stream, nL, nb, tP.data_ptr(), tT.data_ptr(), tX.data_ptr(),
                              tR.data_ptr(), tN.data_ptr(), freqs, tb.data_ptr(), G.REQ, G.RPOL,
                              dt(grad).data_ptr(), dT.data_ptr(), dP.data_ptr(), dX.data_ptr(),
                              weights=tw.data_ptr(), Tb_avg=avg.data_ptr())
        s.synchronize()
        assert np.array_equal(out['Tb_avg'], avg.cpu().numpy()), step
        # d loss / d alpha is accumulated with float atomics over rays, so the
        # gradients agree to float32 rounding, not bit for bit
        for a, d in ((out['dT'], dT), (out['dP'], dP), (out['dlnX'], dX)):
            d = d.cpu().numpy()
            assert np.max(np.abs(a - d)) <= 1e-6 * np.max(np.abs(d)), step


def test_calls_after_an_unfinished_device_call_are_ordered(engine):
    """C3-sized adjoint (1000 layers, 64 freqs, 16 rays) enqueued on a side
    stream, then at once the same adjoint from host buffers and a second
    _device call on another stream, with no synchronisation in between:
    both equal a clean host call (float atomics: ~1e-6 relative)."""
    import torch
    from radiobear_gb300 import catalog, synth
    cats = G.real_catalogues()
    wl = synth.make_workload(3, real=cats)
    wl['lines']['ph3wgt'] = cats['ph3wgt']
    catalog.upload(engine, wl.lines)
    engine.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
    g = wl.gas
    P, T, X = g[G.C['P']], g[G.C['T']], _X(g)
    R, N = wl.prop[LP['R']], wl.prop[LP['N']]
    nL, nb, nf = P.size, len(wl.b), wl.freqs.size
    grad = np.random.default_rng(6).normal(size=nf)
    ref = engine.adjoint(P, T, X, R, N, wl.freqs, wl.b, G.REQ, G.RPOL, grad, weights=wl.weights)
    dev = torch.device('cuda')
    dt = lambda v: torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64, device=dev)
    tP, tT, tX, tR, tN, tb, tw, tg = (dt(v) for v in (P, T, X, R, N, wl.b, wl.weights, grad))
    outs = []
    streams = (torch.cuda.Stream(), torch.cuda.Stream())
    for s in streams:
        dT, dP = torch.empty(nL, dtype=torch.float64, device=dev), torch.empty(nL, dtype=torch.float64, device=dev)
        dX = torch.empty((3, nL), dtype=torch.float64, device=dev)
        engine.adjoint_device(s.cuda_stream, nL, nb, tP.data_ptr(), tT.data_ptr(), tX.data_ptr(),
                              tR.data_ptr(), tN.data_ptr(), wl.freqs, tb.data_ptr(), G.REQ, G.RPOL,
                              tg.data_ptr(), dT.data_ptr(), dP.data_ptr(), dX.data_ptr(),
                              weights=tw.data_ptr())
        outs.append((dT, dP, dX))
    host = engine.adjoint(P, T, X, R, N, wl.freqs, wl.b, G.REQ, G.RPOL, grad, weights=wl.weights)
    torch.cuda.synchronize()
    for got in [(host['dT'], host['dP'], host['dlnX'])] + [tuple(v.cpu().numpy() for v in o) for o in outs]:
        for a, want in zip(got, (ref['dT'], ref['dP'], ref['dlnX'])):
            assert np.max(np.abs(a - want)) <= 1e-6 * np.max(np.abs(want))


def test_launch_shape_knobs_keep_the_results(engine):
    """rb_set_tuning: every JVP launch shape (frequencies per CTA, CTAs per
    SM) gives the same gradient (the per-tile partial sums change their
    float64 summation order only), and every scan lane count the same Tb
    bit for bit (each (ray, chunk, frequency) runs the same arithmetic)."""
    from radiobear_gb300 import synth
    z, g = G.load('c0'), G.gas_table(G.load('c0'))
    _load(engine, G.c0_lines())
    freqs = np.logspace(0.0, np.log10(50.0), 64)
    b, w = synth.gauss_legendre_disc(6)
    args = (g[G.C['P']], g[G.C['T']], _X(g), z['prop_R'], z['prop_N'], freqs, b, G.REQ, G.RPOL)
    grad = np.random.default_rng(2).normal(size=freqs.size)
    try:
        ref = engine.adjoint(*args, grad, weights=w)
        for ft, ctas, nt in ((32, 3, 256), (64, 4, 256), (64, 4, 128), (64, 6, 128), (128, 3, 256), (128, 4, 256),
                             (128, 4, 128)):
            engine.set_tuning(jvp_freqs=ft, jvp_ctas=ctas, jvp_threads=nt)
            out = engine.adjoint(*args, grad, weights=w)
            for k in ('dT', 'dP', 'dlnX'):
                assert np.max(np.abs(out[k] - ref[k])) <= 1e-6 * np.max(np.abs(ref[k])), (ft, ctas, nt, k)
        engine.set_tuning(jvp_freqs=0, jvp_ctas=0, jvp_threads=0)
        tb0 = engine.forward(*args, weights=w)['Tb']
        for lanes in (4, 8, 16, 32, 64, 128):
            engine.set_tuning(scan_lanes=lanes)
            assert np.array_equal(engine.forward(*args, weights=w)['Tb'], tb0), lanes
    finally:
        engine.set_tuning(jvp_freqs=0, jvp_ctas=0, jvp_threads=0, scan_lanes=0)
    from radiobear_gb300._native import RBError
    with pytest.raises((RBError, ValueError)):
        engine.set_tuning(scan_lanes=6)
    with pytest.raises((RBError, ValueError)):
        engine.set_tuning(adj_mode=3)
