"""Benchmark: disc-averaged Tb spectra per second on GB300.

Workload (one "step" = one disc-averaged spectrum of one atmosphere): the
1000-layer Jupiter-like atmosphere (1e-3..500 bar), 256 frequencies log-spaced
0.5..100 GHz, 64-point Gauss-Legendre disc quadrature, line lists NH3 2000 +
H2O 500 + H2S 200 (synthetic, seeded) + PH3 33 (real catalogue).  A step runs
the whole hot path: per-layer absorption, 64 ray paths, 64 x 256 Tb scans and
the disc average.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

``value``: spectra/s with inputs resident in HBM (rb_forward_device on
device tensors), per-step CUDA events, L2 flushed between steps.
``e2e``:  spectra/s through the C ABI (rb_forward) with pinned host buffers,
host->device copies of the atmosphere and the device->host read of the
disc-averaged spectrum inside each timed step.
For N > 1 (torchrun) every rank runs an independent replica ("replicas
only": the forward model has no exchange step).
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = 'disc-avg Tb spectra/s and dTb/dX gradients/s on 1 GB300 at ≤1 mK vs FP64'
UNIT = 'spectra/s'
WORKLOAD = ('C1 plain drop-in disc average: 1000 layers (1e-3..500 bar) x 256 freqs '
            '(0.5..100 GHz log) x 64 Gauss-Legendre disc rays, 2233 lines')


def parse():
    p = argparse.ArgumentParser()
    p.add_argument('--gpus', type=int, default=1)
    p.add_argument('--steps', type=int, default=200)
    p.add_argument('--warmup', type=int, default=5)
    p.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    p.add_argument('--no-cpu-baseline', action='store_true')
    p.add_argument('--no-image', action='store_true', help='skip the C2 image measurement')
    p.add_argument('--batch-variants', type=int, default=4096,
                   help='atmospheres in the batched forward+adjoint measurement (0: skip)')
    p.add_argument('--alpha-tiling', default='',
                   help='line-sum tiling M,W,item_lines (default: automatic)')
    p.add_argument('--no-accuracy', action='store_true',
                   help='skip the per-workload accuracy checks against the float64 oracle')
    p.add_argument('--no-stock-reference', action='store_true',
                   help='reference arm: skip the stock-reference sample')
    return p.parse_args()


def load_workload():
    from radiobear_gb300 import synth
    from tests import goldio
    cats = goldio.real_catalogues()
    wl = synth.make_workload(1, real=cats)
    wl['lines']['ph3wgt'] = cats['ph3wgt']
    return wl


def workload_arrays(wl):
    from radiobear_gb300 import synth, _native
    C = {k: i for i, k in enumerate(synth.GAS_COLUMNS)}
    LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
    g = wl.gas
    return dict(P=g[C['P']].copy(), T=g[C['T']].copy(), X=_native.x_matrix(g, C),
                R=wl.prop[LP['R']].copy(), N=wl.prop[LP['N']].copy(), freqs=wl.freqs.copy(),
                b=np.ascontiguousarray(wl.b), w=np.ascontiguousarray(wl.weights), C=C)


GRAD_WORKLOAD = ('C3 differentiable forward model: 1000 layers (1e-3..500 bar) x 64 freqs '
                 '(1..50 GHz log) x 16 Gauss-Legendre disc rays; forward Tb_avg + adjoint '
                 'dTb/dT, dTb/dP, dTb/dlnX(NH3, H2O, H2S) per layer')


def adjoint_mode(dev, nL, nf):
    """How the adjoint entry points get d alpha / d theta at this size
    (RB_TUNE_ADJ_MODE automatic: stored when nL x nf x 5 floats take at most
    an eighth of the device memory)."""
    import torch
    nbytes = 4 * 5 * int(nL) * int(nf)
    stored = nbytes <= torch.cuda.get_device_properties(dev).total_memory // 8
    return dict(mode='stored d alpha/d theta' if stored else 'recomputed after the reverse sweep',
                stored_bytes=nbytes if stored else 0)


def measure_gradients(args, dev, stream, flush, pool=None):
    """Spectra + gradients per second on the C3 workload: each step runs
    rb_adjoint_device (forward, then the adjoint with alpha recomputed)
    on device-resident inputs; e2e through rb_adjoint with host buffers.
    With a pool, the last timed step's gradient is checked against the
    float64 autograd reference (32 perturbations) and central differences
    of the oracle (8 of them)."""
    import torch
    from radiobear_gb300 import _native, catalog, synth
    from tests import goldio
    cats = goldio.real_catalogues()
    wl = synth.make_workload(3, real=cats)
    wl['lines']['ph3wgt'] = cats['ph3wgt']
    a = workload_arrays(wl)
    nL, nf, nb = a['P'].size, a['freqs'].size, a['b'].shape[0]
    eng = _native.Engine(dev.index or 0)
    catalog.upload(eng, wl.lines)
    eng.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')

    def dt(x):
        return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)

    dP, dT, dX, dR, dN, db, dw = (dt(a[k]) for k in ('P', 'T', 'X', 'R', 'N', 'b', 'w'))
    g = dt(np.random.default_rng(3).normal(size=nf))
    gT, gP, gX = (torch.empty(n, dtype=torch.float64, device=dev) for n in (nL, nL, 3 * nL))
    avg = torch.empty(nf, dtype=torch.float64, device=dev)
    sp = stream.cuda_stream

    def step():
        eng.adjoint_device(sp, nL, nb, dP.data_ptr(), dT.data_ptr(), dX.data_ptr(), dR.data_ptr(),
                           dN.data_ptr(), a['freqs'], db.data_ptr(), 71492.0, 66854.0,
                           g.data_ptr(), gT.data_ptr(), gP.data_ptr(), gX.data_ptr(),
                           weights=dw.data_ptr(), Tb_avg=avg.data_ptr())

    from radiobear_gb300 import tune
    jbest, jt = tune.tune_adjoint(eng, step, key=tune.workload_key('gradients', wl, nb), reps=5,
                                  candidates=[c for c in tune.JVP_CANDIDATES if c[0] <= nf],
                                  stream=stream)
    step()
    torch.cuda.synchronize()
    launches = eng.last_launch_count()
    for _ in range(args.warmup):
        flush.zero_()
        step()
    n = max(10, min(args.steps, 50))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    torch.cuda.synchronize()
    for i in range(n):
        flush.zero_()
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([s.elapsed_time(e) for s, e in ev]))
    grad_gpu = dict(dT=gT.cpu().numpy(), dP=gP.cpu().numpy(), dlnX=gX.cpu().numpy().reshape(3, nL))
    tb_avg_gpu = avg.cpu().numpy()
    host = {k: np.ascontiguousarray(a[k]) for k in ('P', 'T', 'X', 'R', 'N', 'b', 'w')}
    gh = g.cpu().numpy()
    e2e = []
    for i in range(args.warmup + 10):
        t0 = time.perf_counter()
        out = eng.adjoint(host['P'], host['T'], host['X'], host['R'], host['N'], a['freqs'], host['b'],
                          71492.0, 66854.0, gh, weights=host['w'])
        if i >= args.warmup:
            e2e.append(time.perf_counter() - t0)
    h2d = sum(v.nbytes for v in host.values()) + gh.nbytes + a['freqs'].nbytes
    d2h = out['dT'].nbytes + out['dP'].nbytes + out['dlnX'].nbytes + out['Tb'].nbytes + out['Tb_avg'].nbytes
    eng.close()
    out = dict(metric='disc-avg Tb spectra + dTb/dT, dTb/dP, dTb/dlnX gradients per second',
               value=1e3 / ms, unit='spectra+gradients/s', ms_per_step=ms, steps=n,
               config=dict(workload=GRAD_WORKLOAD, layers=nL, freqs=nf, rays=nb,
                           adjoint=adjoint_mode(dev, nL, nf),
                           jvp=dict(freqs_per_cta=jbest[0], ctas_per_sm=jbest[1], threads=jbest[2]),
                           jvp_tuning_ms={','.join(map(str, k)): v for k, v in jt.items()}),
               gpu_launches_per_step=int(launches),
               e2e=dict(value=1.0 / float(np.mean(e2e)), unit='spectra+gradients/s',
                        h2d_bytes_per_step=int(h2d), d2h_bytes_per_step=int(d2h),
                        api='rb_adjoint (C ABI, host buffers)'))
    if pool is not None:
        from oracle import accuracy as ACC
        from oracle import parallel as OP
        acc = ACC.gradients(pool, wl.freqs, wl.gas, a['C'], a['R'], a['N'], a['b'], a['w'], wl.lines,
                            71492.0, 66854.0, grad_gpu, gh, n_dir=32, n_fd=8, device=str(dev))
        layers = OP.layers(pool, wl.freqs, wl.gas, a['C'], wl.lines)
        tb, _ = OP.rays(pool, a['R'], a['N'], a['b'], 71492.0, 66854.0, layers, a['T'])
        acc['max_abs_dTb_avg_K'] = float(np.max(np.abs(tb_avg_gpu - np.tensordot(a['w'], tb, axes=1))))
        out['accuracy'] = acc
    return out


BATCH_WORKLOAD = ('C4 batched retrieval sweep: {n} variants of the 1e-3..100 bar recipe (deep NH3 '
                  'log-U 1e-4..1e-3, deep T offset U(-10, 10) K, 300..1200 layers), 128 freqs '
                  '(0.5..50 GHz log), 32-ray disc quadrature, configuration-0 line lists; forward '
                  'Tb_avg + adjoint dTb/dT, dTb/dP, dTb/dlnX for every variant per step, replayed '
                  'from one captured CUDA graph; alpha and d alpha/d theta from one JVP pass before '
                  'the scan (d alpha/d theta stored, contracted after the reverse sweep), JVP '
                  'launch shape from the autotuner')


def measure_batch(args, dev, n_var, pool=None):
    """Spectra + gradients per second for a batch of n_var atmospheres
    (rb_adjoint_batch_device captured in a CUDA graph and replayed), beside
    the same variants run one call per atmosphere (rb_adjoint_device).  With
    a pool, 8 variants spread over the layer range are checked against the
    float64 oracle (Tb_avg, and a gradient direction by central
    differences)."""
    import torch
    from radiobear_gb300 import _native, catalog, synth, tune
    from tests import goldio
    cats = goldio.real_catalogues()
    wl0 = synth.make_workload(0, real=cats)
    lines = dict(wl0.lines)
    lines['ph3wgt'] = cats['ph3wgt']
    nLs, nh3, dT = synth.make_variants(n_var)
    C = {k: i for i, k in enumerate(synth.GAS_COLUMNS)}
    LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
    P, T, X, R, N = [], [], [], [], []
    for i in range(n_var):
        g = synth.make_gas_table(int(nLs[i]), 1.0e-3, 100.0, nh3_deep=nh3[i], dT_deep=dT[i])
        pr = synth.compute_properties(g)
        P.append(g[C['P']])
        T.append(g[C['T']])
        X.append(_native.x_matrix(g, C))
        R.append(pr[LP['R']])
        N.append(pr[LP['N']])
    freqs = np.logspace(np.log10(0.5), np.log10(50.0), 128)
    b, w = synth.gauss_legendre_disc(32)
    nf, nb, NLT = freqs.size, b.shape[0], int(np.sum(nLs))
    f64 = dict(dtype=torch.float64, device=dev)
    t = dict(P=torch.tensor(np.concatenate(P), **f64), T=torch.tensor(np.concatenate(T), **f64),
             X=torch.tensor(np.ascontiguousarray(np.concatenate(X, axis=1)), **f64),
             R=torch.tensor(np.concatenate(R), **f64), N=torch.tensor(np.concatenate(N), **f64),
             b=torch.tensor(b, **f64), w=torch.tensor(w, **f64))
    grad = torch.tensor(np.random.default_rng(4).normal(size=(n_var, nf)), **f64)
    avg = torch.empty((n_var, nf), **f64)
    gT, gP = torch.empty(NLT, **f64), torch.empty(NLT, **f64)
    gX = torch.empty((3, NLT), **f64)
    eng = _native.Engine(dev.index or 0)
    catalog.upload(eng, lines)
    eng.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    stream = torch.cuda.current_stream(dev)

    def step():
        eng.adjoint_batch_device(torch.cuda.current_stream(dev).cuda_stream, nLs, t['P'].data_ptr(),
                                 t['T'].data_ptr(), t['X'].data_ptr(), t['R'].data_ptr(),
                                 t['N'].data_ptr(), freqs, t['b'], t['w'].data_ptr(), grad.data_ptr(),
                                 avg.data_ptr(), gT.data_ptr(), gP.data_ptr(), gX.data_ptr(),
                                 71492.0, 66854.0)

    jbest, jt = tune.tune_adjoint(eng, step, key=tune.workload_key('batch', dict(freqs=freqs, lines=lines),
                                                                  nb, layers=(300, 1200)),
                                  reps=1, stream=stream)
    step()                                   # plan and buffers for the chosen tiling
    torch.cuda.synchronize()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step()
    graph.replay()
    torch.cuda.synchronize()
    n = max(3, min(args.steps, 5))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    for s, e in ev:
        s.record(stream)
        graph.replay()
        e.record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([s.elapsed_time(e) for s, e in ev]))
    ok = bool(torch.isfinite(avg).all().item() and torch.isfinite(gT).all().item())
    res = dict(avg=avg.cpu().numpy(), dT=gT.cpu().numpy(), dP=gP.cpu().numpy(), dX=gX.cpu().numpy(),
               grad=grad.cpu().numpy())
    # the same variants one atmosphere per call (plain path), a sample of 16
    one = _native.Engine(dev.index or 0)
    catalog.upload(one, lines)
    one.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    o = np.concatenate([[0], np.cumsum(nLs)])
    single = []
    for i in range(min(16, n_var)):
        sl = slice(int(o[i]), int(o[i + 1]))
        args1 = (t['P'][sl].contiguous(), t['T'][sl].contiguous(), t['X'][:, sl].contiguous(),
                 t['R'][sl].contiguous(), t['N'][sl].contiguous())
        g1 = grad[i].contiguous()
        d1 = [torch.empty(int(nLs[i]), **f64) for _ in range(2)] + [torch.empty((3, int(nLs[i])), **f64)]

        def one_step():
            one.adjoint_device(stream.cuda_stream, int(nLs[i]), nb, args1[0].data_ptr(), args1[1].data_ptr(),
                               args1[2].data_ptr(), args1[3].data_ptr(), args1[4].data_ptr(), freqs,
                               t['b'].data_ptr(), 71492.0, 66854.0, g1.data_ptr(), d1[0].data_ptr(),
                               d1[1].data_ptr(), d1[2].data_ptr(), weights=t['w'].data_ptr())
        tb1 = torch.empty((nb, nf), **f64)
        av1 = torch.empty(nf, **f64)

        def one_fwd():
            one.forward_device(stream.cuda_stream, int(nLs[i]), nb, args1[0].data_ptr(), args1[1].data_ptr(),
                               args1[2].data_ptr(), args1[3].data_ptr(), args1[4].data_ptr(), freqs,
                               t['b'].data_ptr(), 71492.0, 66854.0, tb1.data_ptr(),
                               weights=t['w'].data_ptr(), Tb_avg=av1.data_ptr())
        row = []
        for fn in (one_step, one_fwd):
            fn()
            torch.cuda.synchronize()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record(stream)
            fn()
            s1.record(stream)
            torch.cuda.synchronize()
            row.append(s0.elapsed_time(s1) * 1e3 / int(nLs[i]))   # us per layer
        single.append(row)
    per_layer = np.mean(np.array(single), axis=0)
    per_var_ms = float(per_layer[0]) * float(np.mean(nLs)) * 1e-3
    fwd_ms = float(per_layer[1]) * float(np.mean(nLs)) * 1e-3
    eng.close()
    one.close()
    value = n_var / (ms * 1e-3)
    plain = 1e3 / per_var_ms
    fd_rate = 1e3 / (fwd_ms * (1 + 2 * 5 * float(np.mean(nLs))))
    return dict(metric='disc-avg Tb spectra + dTb/dT, dTb/dP, dTb/dlnX gradients per second (batched)',
                value=value, unit='spectra+gradients/s', ms_per_step=ms, steps=n, finite=ok,
                config=dict(workload=BATCH_WORKLOAD.format(n=n_var), variants=n_var,
                            layers_total=NLT, freqs=nf, rays_per_variant=nb,
                            adjoint=adjoint_mode(dev, NLT, nf),
                            jvp=dict(freqs_per_cta=jbest[0], ctas_per_sm=jbest[1], threads=jbest[2]),
                            jvp_tuning_ms={','.join(map(str, k)): v for k, v in jt.items()},
                            l2='working set of tens of GB, larger than L2'),
                per_atmosphere_adjoint=dict(value=plain, unit='spectra+gradients/s',
                                            api='rb_adjoint_device, one atmosphere per call, '
                                                '16-variant sample scaled by layer count'),
                plain_dropin_finite_differences=dict(
                    value=fd_rate, unit='spectra+gradients/s',
                    how='plain drop-in forward (rb_forward_device, one atmosphere per call) '
                        'times 1 + 2 x 5 x nL central differences per gradient set'),
                speedup_vs_per_atmosphere_adjoint=value / plain,
                speedup_vs_plain_dropin=value / fd_rate,
                accuracy=None if pool is None else batch_accuracy(pool, nLs, nh3, dT, freqs, b, w, lines,
                                                                  C, LP, res))


def batch_accuracy(pool, nLs, nh3, dT, freqs, b, w, lines, C, LP, res, n_sample=8):
    """8 variants spread over the layer range: Tb_avg against the float64
    oracle and one random perturbation's directional derivative against
    central differences of the oracle."""
    from oracle import adjoint as A
    from oracle import parallel as OP
    from radiobear_gb300 import synth
    off = np.concatenate([[0], np.cumsum(nLs)])
    pick = np.argsort(nLs, kind='stable')[np.linspace(0, len(nLs) - 1, n_sample).astype(int)]
    worst_tb, worst_dir, layers_seen = 0.0, 0.0, []
    for v in pick:
        gas = synth.make_gas_table(int(nLs[v]), 1.0e-3, 100.0, nh3_deep=nh3[v], dT_deep=dT[v])
        pr = synth.compute_properties(gas)
        R, N = pr[LP['R']], pr[LP['N']]
        lay = OP.layers(pool, freqs, gas, C, lines)
        tb, _ = OP.rays(pool, R, N, b, 71492.0, 66854.0, lay, gas[C['T']])
        worst_tb = max(worst_tb, float(np.max(np.abs(res['avg'][v] - np.tensordot(w, tb, axes=1)))))
        sl = slice(int(off[v]), int(off[v + 1]))
        got = dict(dT=res['dT'][sl], dP=res['dP'][sl], dlnX=res['dX'][:, sl])
        d = A.random_direction(np.random.default_rng(1000 + int(v)), gas, C)
        fd = OP.directional_fd(pool, gas, C, R, N, freqs, b, lines, 71492.0, 66854.0, w, res['grad'][v], [d])
        worst_dir = max(worst_dir, float(abs(A.dot(got, d) - fd[0]) / abs(fd[0])))
        layers_seen.append(int(nLs[v]))
    return dict(variants=n_sample, layers=layers_seen, max_abs_dTb_avg_K=worst_tb,
                dir_rel_err_vs_central_differences=worst_dir,
                reference='float64 oracle; central differences step 1e-4')


IMAGE_WORKLOAD = ('C2 batched image rays: 256 x 256 impact parameters at 0.01 planet radius '
                  '(31,397 on the disc incl. limb rays of up to ~2000 segments, the rest off the '
                  'planet -> T_cmb) x 8 freqs (1.4..44 GHz), 1000 layers, C1 line lists; one step = '
                  'one image replayed from a captured CUDA graph, line-sum tiling from the '
                  'autotuner')


def measure_image(args, dev, stream, flush, pool=None):
    """Images per second (and rays/s) for the C2 grid: every ray of an image
    in one rb_forward_device, captured once into a CUDA graph and replayed;
    the line-sum tiling chosen by the autotuner for this shape.  The scan's
    HBM fraction (its segments stream from HBM here) and, with a pool, the
    accuracy of a 256-ray sample against the float64 oracle."""
    import torch
    from radiobear_gb300 import _native, catalog, synth, tune
    from tests import goldio
    cats = goldio.real_catalogues()
    wl = synth.make_workload(2, real=cats)
    wl['lines']['ph3wgt'] = cats['ph3wgt']
    a = workload_arrays(wl)
    nL, nf, nb = a['P'].size, a['freqs'].size, a['b'].shape[0]
    eng = _native.Engine(dev.index or 0)
    catalog.upload(eng, wl.lines)
    eng.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')

    def dt(x):
        return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)

    dP, dT, dX, dR, dN, db = (dt(a[k]) for k in ('P', 'T', 'X', 'R', 'N', 'b'))
    Tb = torch.empty((nb, nf), dtype=torch.float64, device=dev)

    def step():
        eng.forward_device(torch.cuda.current_stream(dev).cuda_stream, nL, nb, dP.data_ptr(),
                           dT.data_ptr(), dX.data_ptr(), dR.data_ptr(), dN.data_ptr(), a['freqs'],
                           db.data_ptr(), 71492.0, 66854.0, Tb.data_ptr())

    best, tt = tune.tune_alpha(eng, step, key=tune.workload_key('image', wl, nb),
                               candidates=((2, 1, 1024), (2, 2, 1024), (4, 1, 1024), (2, 4, 1024),
                                           (2, 1, 512)), reps=2, stream=stream)
    step()                                   # plan and buffers for the chosen tiling
    torch.cuda.synchronize()
    launches = eng.last_launch_count()
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        step()
    for _ in range(args.warmup):
        flush.zero_()
        graph.replay()
    n = max(3, min(args.steps, 20))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    torch.cuda.synchronize()
    for s, e in ev:
        flush.zero_()
        s.record(stream)
        graph.replay()
        e.record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([s.elapsed_time(e) for s, e in ev]))
    t = Tb.cpu().numpy()
    on = np.hypot(a['b'][:, 0], a['b'][:, 1]) < 1.0
    # scan phase (library events on the launching streams) and the rays' path lengths
    eng.set_profiling(True)
    phs = []
    for _ in range(5):
        flush.zero_()
        step()
        phs.append(eng.phase_times())
    eng.set_profiling(False)
    ph = {k: float(np.mean([p[k] for p in phs])) for k in phs[0]}
    nseg = np.concatenate([eng.raypath(a['R'], a['N'], a['b'][k:k + 4096], 71492.0, 66854.0)['nseg']
                           for k in range(0, nb, 4096)])
    sbytes = scan_bytes(nseg, nf, nb)
    hbm = measured_peaks().get('hbm_gbs')
    scan_gbs = sbytes / (ph['brightness'] * 1e-3) / 1e9
    out = dict(metric='brightness images per second', value=1e3 / ms, unit='images/s',
               rays_per_s=nb * 1e3 / ms, ms_per_step=ms, steps=n, gpu_launches_per_step=int(launches),
               config=dict(workload=IMAGE_WORKLOAD, layers=nL, freqs=nf, rays=nb,
                           rays_on_disc=int(on.sum()), max_path_segments=int(nseg.max()),
                           cuda_graph=True, tiling=dict(M=best[0], W=best[1], item_lines=best[2]),
                           tuning_ms={'{},{},{}'.format(*k): v for k, v in tt.items()},
                           l2='256 MiB buffer written between steps'),
               phase_ms=ph,
               roofline_scan=dict(bound='hbm', kernel='rb_tb_chunk2_kernel+rb_tb_combine_kernel',
                                  achieved=scan_gbs, peak=hbm, unit='GB/s',
                                  frac=(scan_gbs / hbm) if hbm else None,
                                  algorithmic_bytes_per_launch=sbytes,
                                  peak_source='MEASURED_PEAKS.json hbm_gbs (of measured)'),
               finite=bool(np.isfinite(t).all()),
               off_disc_is_tcmb=bool(np.all(t[~on] == 2.725)))
    if pool is not None:
        from oracle import accuracy as ACC
        rng = np.random.default_rng(5)
        onx = np.nonzero(on)[0]
        r = np.hypot(a['b'][:, 0], a['b'][:, 1])
        cand = np.union1d(onx[r[onx] > 0.985], rng.choice(onx, 1024, replace=False))
        sel, _, _ = ACC.image_sample(a['b'][cand], nseg[cand])
        idx = cand[sel]
        acc, _, _ = ACC.image(pool, wl.freqs, wl.gas, a['C'], a['R'], a['N'], a['b'][idx], wl.lines,
                              71492.0, 66854.0, t[idx])
        acc['sample'] = ('{} rays reaching the planet: the 16 longest paths (limb rays), the 16 '
                         'outermost, a seeded random fill').format(len(idx))
        out['accuracy'] = acc
    eng.close()
    return out


def replica_time(tot_ms, dist=None, device=None):
    """Replicas only: each rank times its own copy of the workload; the job
    time is the slowest rank's (MAX all-reduce), and the job's value counts
    every rank's spectra (world x steps) over it."""
    if dist is None:
        return tot_ms
    import torch
    t = torch.tensor([tot_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def alpha_flops(wl):
    """Algorithmic FLOPs of one absorption launch: per (layer, line, freq)
    Ben-Reuven 10, Gross 8, VVW 12 (FMA = 2); blend layers add the nh3_sjs
    lines at 10."""
    from radiobear_gb300 import synth
    C = {k: i for i, k in enumerate(synth.GAS_COLUMNS)}
    P = wl.gas[C['P']]
    L = wl.lines
    nL, nf = P.size, wl.freqs.size
    n_br = len(L['ammonia']['fo']) + len(L['h2s']['f0']) + len(L['ph3']['f0'])
    n_gross = len(L['ammonia']['fo_rot']) + len(L['ammonia']['fo_v2'])
    n_vvw = len(L['h2o']['f_o'])
    n_blend = int(np.sum((P >= 400.0) & (P <= 2000.0)))
    n_sjs = len(L['nh3']['f0'])
    per = 10 * n_br + 8 * n_gross + 12 * n_vvw
    return nL * nf * per + n_blend * nf * 10 * n_sjs, dict(n_br=n_br, n_gross=n_gross, n_vvw=n_vvw,
                                                            n_sjs_blend_layers=n_blend, n_sjs=n_sjs)


# Algorithmic FLOPs of the scan per (segment, frequency), exp counted as one:
# optical depth (add, multiply, add), W = a exp(-tau) (exp, multiply), intW
# (add, multiply, add), TbL (two multiplies, add, multiply, add).
SCAN_FLOPS = 13


def scan_flops(nseg, nf):
    return int(np.sum(np.maximum(np.asarray(nseg) - 1, 0)) * nf * SCAN_FLOPS)


def l2_bandwidth(dev, mib=16, reps=200):
    """Read + write GB/s of copies between two L2-resident buffers."""
    import torch
    x = torch.ones(mib << 18, dtype=torch.float32, device=dev)
    y = torch.empty_like(x)
    for _ in range(10):
        y.copy_(x)
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    for _ in range(reps):
        y.copy_(x)
    e.record()
    torch.cuda.synchronize()
    return 2.0 * x.numel() * 4 * reps / (s.elapsed_time(e) * 1e-3) / 1e9


def scan_bytes(nseg, nf, nb):
    """Algorithmic bytes of the Tb scan: per segment float32 alpha for every
    frequency + float64 ds + int32 layer, and float64 Tb out."""
    return int(np.sum(nseg) * (4 * nf + 12) + nb * nf * 8)


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples every 50 ms while the timed steps run.  Entering
    waits (at most 3 s) for the first sample so the sampler is live before
    the first timed step; `region(t0, t1)` gives the timed region's wall
    clock, and the summary keeps the samples stamped inside it (all samples
    if none is)."""
    FIELDS = ('timestamp', 'index', 'clocks.sm', 'clocks.max.sm', 'power.draw',
              'clocks_event_reasons.active', 'clocks_event_reasons.hw_slowdown',
              'clocks_event_reasons.hw_thermal_slowdown',
              'clocks_event_reasons.sw_thermal_slowdown', 'clocks_event_reasons.sw_power_cap')
    REASONS = ('hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap')

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.path = None
        self.window = None

    def _start(self, period_ms):
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index),
                                          '--query-gpu=' + ','.join(self.FIELDS),
                                          '--format=csv,noheader,nounits', '-lms', str(period_ms)],
                                         stdout=open(self.path, 'w'), stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
            return
        deadline = time.time() + 3.0
        while time.time() < deadline and self.proc.poll() is None:
            if self._rows():
                return
            time.sleep(0.01)

    def __enter__(self):
        fd, self.path = tempfile.mkstemp(suffix='.csv')
        os.close(fd)
        self._start(50)
        if self.proc is not None and self.proc.poll() is not None and not self._rows():
            self._start(200)     # the 50 ms period refused: the usual 200 ms
        return self

    def region(self, t0, t1):
        self.window = (t0, t1)

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def _rows(self):
        rows = []
        try:
            with open(self.path) as fp:
                for line in fp:
                    if not line.endswith('\n'):
                        break
                    parts = [p.strip() for p in line.split(',')]
                    if len(parts) >= len(self.FIELDS):
                        rows.append(parts)
        except OSError:
            pass
        return rows

    @staticmethod
    def _stamp(text):
        import datetime
        try:
            return datetime.datetime.strptime(text, '%Y/%m/%d %H:%M:%S.%f').timestamp()
        except ValueError:
            return None

    @staticmethod
    def _num(text):
        try:
            return float(text)
        except ValueError:
            return None

    def summary(self):
        rows = self._rows()
        if self.path and os.path.exists(self.path):
            os.unlink(self.path)
        if not rows:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        inside = []
        if self.window is not None:
            t0, t1 = self.window[0] - 0.025, self.window[1] + 0.025
            for r in rows:
                t = self._stamp(r[0])
                if t is not None and t0 <= t <= t1:
                    inside.append(r)
        in_region = bool(inside)
        use = inside if in_region else rows
        sm = [v for v in (self._num(r[2]) for r in use) if v is not None]
        mx = [v for v in (self._num(r[3]) for r in use) if v is not None]
        reasons = sorted({self.REASONS[i] for r in use for i in range(4)
                          if r[6 + i].lower() == 'active'})
        return {'sm_mhz': statistics.median(sm) if sm else None,
                'sm_max_mhz': max(mx) if mx else None, 'reasons': reasons,
                'samples': len(use), 'in_timed_region': in_region}


def profile_traffic(name='alpha_kernel_c1.md'):
    """dram bytes per launch from a committed ncu summary of the same
    workload (a capture of that kernel, not a measurement of this run)."""
    path = os.path.join(ROOT, 'profiles', name)
    try:
        with open(path) as fp:
            m = re.search(r'traffic_bytes_per_launch:\s*([0-9.eE+]+)', fp.read())
        return dict(file='profiles/' + name, dram_bytes_per_launch=float(m.group(1))) if m else None
    except OSError:
        return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as fp:
            return json.load(fp)
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------------ CPU oracle
def make_pool():
    """Spawn-context pool over the host cores (made before the first GPU call)."""
    from oracle import parallel as OP
    return OP.make_pool()


def port_spectrum(pool, wl):
    """One whole C1 disc-averaged spectrum by the float64 oracle on the pool:
    alpha of every layer (blocks of layers per worker), the 64 ray paths and
    scans (one ray per task) and the quadrature average.  Returns (seconds,
    Tb_avg)."""
    from oracle import parallel as OP
    a = workload_arrays(wl)
    t0 = time.perf_counter()
    layers = OP.layers(pool, wl.freqs, wl.gas, a['C'], wl.lines)
    tb, _ = OP.rays(pool, a['R'], a['N'], wl.b, 71492.0, 66854.0, layers, a['T'])
    avg = np.tensordot(wl.weights, tb, axes=1)
    return time.perf_counter() - t0, avg


PORT_SAMPLE = ('one whole spectrum per step: alpha of all 1000 layers x 256 freqs, 64 ray paths '
               'and scans, the disc average; float64 numpy oracle on {} worker processes')


def cpu_baseline(wl, pool, cores):
    sec, _ = port_spectrum(pool, wl)
    return dict(value=1.0 / sec, unit=UNIT, cores=cores, kind='port', sample=PORT_SAMPLE.format(cores),
                seconds_per_spectrum=sec)


def stock_reference(cores, layers_per_worker=2):
    """The unmodified reference (installed under baseline/_ref) timed on a
    sample of the same C1 workload: its own Alpha.get_alpha_from_calc for
    2 layers per worker and Brightness.single for one ray per worker, each
    worker on its own core; wall times scaled to the 1000 layers and 64
    rays of one spectrum (extrapolated)."""
    ref = os.path.join(ROOT, 'baseline', '_ref')
    if not os.path.isdir(os.path.join(ref, 'radiobear')):
        return dict(unavailable='the reference is not installed under baseline/_ref')
    import multiprocessing as mp
    sys.path.insert(0, os.path.join(ROOT, 'tests', 'golden'))
    import refharness as H
    pool = mp.get_context('spawn').Pool(cores, initializer=H.stock_init, initargs=(ref, ROOT))
    try:
        nL, nb = 1000, 64
        lay = np.linspace(0, nL - 1, cores * layers_per_worker).astype(int)
        jobs = [lay[k::cores].tolist() for k in range(cores)]
        rays = np.linspace(1, nb - 1, min(cores, nb - 1)).astype(int).tolist()
        pool.map(H.stock_ray_job, rays[:1])                  # first call warms the modules
        t0 = time.perf_counter()
        pool.map(H.stock_alpha_job, jobs, chunksize=1)
        t_alpha = time.perf_counter() - t0
        t0 = time.perf_counter()
        pool.map(H.stock_ray_job, rays, chunksize=1)
        t_rays = time.perf_counter() - t0
    finally:
        pool.close()
        pool.join()
    per = t_alpha * nL / len(lay) + t_rays * nb / len(rays)
    return dict(value=1.0 / per, unit=UNIT, cores=cores, kind='reference', extrapolated=True,
                seconds_per_spectrum=per,
                sample=('the unmodified reference (pip-installed from its source): '
                        'Alpha.get_alpha_from_calc of {} of 1000 layers and Brightness.single of {} '
                        'of 64 rays, one worker process per core, wall times scaled to one spectrum '
                        '(limb branch of compute_ds restored as in the parity harness)').format(
                            len(lay), len(rays)))


# ------------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    """Rank 0 only.  Each step is one whole C1 spectrum by the float64 port on
    every host core (nothing sampled or extrapolated); beside it, the stock
    reference on a sample (extrapolated, marked so)."""
    if rank != 0:
        return
    wl = load_workload()
    pool, cores = make_pool()
    try:
        for _ in range(args.warmup):
            port_spectrum(pool, wl)
        secs = []
        t_wall = time.perf_counter()
        for _ in range(args.steps):
            secs.append(port_spectrum(pool, wl)[0])
        t_wall = time.perf_counter() - t_wall
    finally:
        pool.close()
        pool.join()
    stock = None if args.no_stock_reference else stock_reference(cores)
    ms = 1e3 * float(np.mean(secs))
    value = 1e3 / ms
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=ms, higher_is_better=True, scaling='weak',
                vs_baseline=None, dtype='f64', data='synthetic', impl='reference',
                config=dict(workload=WORKLOAD, layers=1000, freqs=256, rays=64),
                timed_region_s=t_wall,
                cpu_baseline=dict(value=value, unit=UNIT, cores=cores, kind='port',
                                  sample=PORT_SAMPLE.format(cores), extrapolated=False),
                stock_reference=stock,
                e2e=dict(value=value, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, rank, world, local_rank):
    import torch
    from radiobear_gb300 import _native, catalog

    pool = cores = None
    if rank == 0 and not (args.no_cpu_baseline and args.no_accuracy):
        pool, cores = make_pool()          # spawn before the first GPU call
    acc_pool = None if args.no_accuracy else pool

    torch.cuda.set_device(local_rank)
    dev = torch.device('cuda', local_rank)
    wl = load_workload()
    a = workload_arrays(wl)
    nL, nf, nb = a['P'].size, a['freqs'].size, a['b'].shape[0]
    eng = _native.Engine(local_rank)
    catalog.upload(eng, wl.lines)
    eng.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    if args.alpha_tiling:
        eng.set_alpha_tiling(*[int(v) for v in args.alpha_tiling.split(',')])
    stream = torch.cuda.current_stream(dev)
    sp = stream.cuda_stream

    def dt(x):
        return torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float64, device=dev)

    dP, dT, dX, dR, dN = dt(a['P']), dt(a['T']), dt(a['X']), dt(a['R']), dt(a['N'])
    db, dw = dt(a['b']), dt(a['w'])
    dTb = torch.empty((nb, nf), dtype=torch.float64, device=dev)
    davg = torch.empty(nf, dtype=torch.float64, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        eng.forward_device(sp, nL, nb, dP.data_ptr(), dT.data_ptr(), dX.data_ptr(), dR.data_ptr(),
                           dN.data_ptr(), a['freqs'], db.data_ptr(), 71492.0, 66854.0,
                           dTb.data_ptr(), weights=dw.data_ptr(), Tb_avg=davg.data_ptr())

    from radiobear_gb300 import tune
    tuned = {}
    if not args.alpha_tiling:
        key = tune.workload_key('spectrum', wl, nb)
        ab, at = tune.tune_alpha(eng, step, key=key, candidates=((2, 4, 1024), (2, 2, 1024),
                                                                 (4, 2, 1024), (2, 4, 512)),
                                 reps=5, stream=stream)
        sb, st_ = tune.tune_scan(eng, step, key=key, candidates=((32,), (64,), (128,)), reps=5,
                                 stream=stream)
        tuned = dict(tiling=dict(M=ab[0], W=ab[1], item_lines=ab[2]),
                     tuning_ms={'{},{},{}'.format(*k): v for k, v in at.items()},
                     scan_lanes=sb[0], scan_tuning_ms={str(k[0]): v for k, v in st_.items()})
    step()
    torch.cuda.synchronize()
    launches_per_step = eng.last_launch_count()
    for _ in range(args.warmup):
        flush.zero_()
        step()
    torch.cuda.synchronize()

    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(args.steps)]
    with ClockSampler(local_rank) as clk:
        t_wall0 = time.time()
        for i in range(args.steps):
            flush.zero_()
            ev[i][0].record(stream)
            step()
            ev[i][1].record(stream)
        torch.cuda.synchronize()
        clk.region(t_wall0, time.time())
    if dist is not None:
        dist.barrier()
    step_ms = [s.elapsed_time(e) for s, e in ev]
    tot_ms = replica_time(float(sum(step_ms)), dist, dev)
    clocks = clk.summary()

    # phase timing (CUDA events recorded inside the library on the streams
    # the kernels run on), same workload, L2 flushed before each step
    eng.set_profiling(True)
    phases = {k: [] for k in eng.PHASES}
    for i in range(max(10, min(args.steps, 50))):
        flush.zero_()
        step()
        for k, v in eng.phase_times().items():
            phases[k].append(v)
    eng.set_profiling(False)
    ph = {k: float(np.mean(v)) for k, v in phases.items()}

    # e2e through the C ABI with pinned host buffers
    pin = {k: torch.from_numpy(np.ascontiguousarray(a[k])).pin_memory()
           for k in ('P', 'T', 'X', 'R', 'N', 'b', 'w')}
    host = {k: v.numpy() for k, v in pin.items()}
    e2e_times = []
    for i in range(args.warmup + max(10, min(args.steps, 100))):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        out = eng.forward(host['P'], host['T'], host['X'], host['R'], host['N'], a['freqs'],
                          host['b'], 71492.0, 66854.0, weights=host['w'], want_rays=False)
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_times.append(t1 - t0)
    h2d = sum(host[k].nbytes for k in host) + a['freqs'].nbytes
    d2h = out['Tb_avg'].nbytes

    # the last timed step's outputs, and the absorption table, for the accuracy check
    tb_gpu, avg_gpu = dTb.cpu().numpy(), davg.cpu().numpy()
    layers_gpu = eng.forward(host['P'], host['T'], host['X'], host['R'], host['N'], a['freqs'],
                             host['b'], 71492.0, 66854.0, want_rays=False, want_layers=True)['layers']

    grads = measure_gradients(args, dev, stream, flush, acc_pool if rank == 0 else None)
    image = None if args.no_image else measure_image(args, dev, stream, flush,
                                                     acc_pool if rank == 0 else None)
    batched = (measure_batch(args, dev, args.batch_variants, acc_pool if rank == 0 else None)
               if args.batch_variants > 0 else None)
    if rank != 0:
        return
    # roofline of the dominant kernel (the line sums, timed alone on their
    # stream) and of the Tb scan
    flops, counts = alpha_flops(wl)
    fp32_peak = eng.probe_fp32_peak()
    ach = flops / (ph['alpha'] * 1e-3) / 1e12
    rays = eng.raypath(a['R'], a['N'], a['b'], 71492.0, 66854.0)
    sbytes = scan_bytes(rays['nseg'], nf, nb)
    sflops = scan_flops(rays['nseg'], nf)
    l2 = l2_bandwidth(dev)
    scan_s = ph['brightness'] * 1e-3
    value = world * args.steps / (tot_ms * 1e-3)
    line = dict(
        metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
        ms_per_step=tot_ms / args.steps, higher_is_better=True, scaling='weak', vs_baseline=None,
        dtype='f32', data='synthetic',
        config=dict(workload=WORKLOAD, layers=nL, freqs=nf, rays=nb, lines=counts,
                    parallelism='replicas' if world > 1 else 'single',
                    l2='256 MiB buffer written between steps; per-step CUDA events',
                    precision='f32 compensated (Kahan) line sums; f64 ray set-up, double-float (float pair) ray walk; double-float optical depth, compensated f32 weighted sums',
                    autotuned=tuned),
        e2e=dict(value=1.0 / float(np.mean(e2e_times)), unit=UNIT, h2d_bytes_per_step=int(h2d),
                 d2h_bytes_per_step=int(d2h), api='rb_forward (C ABI, pinned host buffers)'),
        gpu_launches=int(launches_per_step * args.steps),
        roofline=dict(bound='fp32', kernel='rb_alpha_lines_kernel', achieved=ach, peak=fp32_peak,
                      unit='TFLOP/s', frac=ach / fp32_peak, traffic=None,
                      traffic_ncu_capture=profile_traffic(),
                      algorithmic_flops_per_launch=flops,
                      peak_source='in-run FFMA probe (no fp32 entry in MEASURED_PEAKS.json)'),
        # C1's scan reads the 1 MB absorption table from L2 and is bound by
        # the FMA pipe (ncu): its algorithmic flops against the FP32 peak,
        # its algorithmic bytes against the measured L2 rate
        roofline_scan=dict(bound='fp32', kernel='rb_tb_chunk2_kernel+rb_tb_combine_kernel',
                           achieved=sflops / scan_s / 1e12, peak=fp32_peak, unit='TFLOP/s',
                           frac=sflops / scan_s / 1e12 / fp32_peak,
                           algorithmic_flops_per_launch=sflops,
                           flops_per_segment_and_freq=SCAN_FLOPS,
                           l2=dict(achieved=sbytes / scan_s / 1e9, peak=l2, unit='GB/s',
                                   frac=sbytes / scan_s / 1e9 / l2,
                                   algorithmic_bytes_per_launch=sbytes,
                                   peak_source='in-run copy of an L2-resident 2 x 16 MiB buffer pair'),
                           traffic_ncu_capture=profile_traffic('tb_scan_c1.md'),
                           peak_source='in-run FFMA probe'),
        phase_ms=ph, clocks=clocks, gradients=grads, batched=batched, image=image)
    if acc_pool is not None:
        from oracle import accuracy as ACC
        acc = ACC.spectra(acc_pool, wl.freqs, wl.gas, a['C'], a['R'], a['N'], a['b'], a['w'], wl.lines,
                          71492.0, 66854.0, tb_gpu, avg_gpu, layers_gpu)
        line['accuracy'] = acc
    if pool is not None and not args.no_cpu_baseline:
        line['cpu_baseline'] = cpu_baseline(wl, pool, cores)
    if pool is not None:
        pool.close()
        pool.join()
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world = int(os.environ.get('WORLD_SIZE', '1'))
    rank = int(os.environ.get('RANK', '0'))
    local_rank = int(os.environ.get('LOCAL_RANK', '0'))
    if args.impl == 'reference':
        run_reference(args, rank, world)
        return
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local_rank)
        dist.init_process_group('nccl')
    try:
        run_gpu(args, rank, world, local_rank)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()


if __name__ == '__main__':
    main()
