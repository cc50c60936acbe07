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
    p.add_argument('--cpu-sample-s', type=float, default=20.0)
    p.add_argument('--no-image', action='store_true', help='skip the C2 image measurement')
    p.add_argument('--batch-variants', type=int, default=4096,
                   help='atmospheres in the batched forward+adjoint measurement (0: skip)')
    p.add_argument('--alpha-tiling', default='',
                   help='line-sum tiling M,W,item_lines (default: automatic)')
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


def measure_gradients(args, dev, stream, flush):
    """Spectra + gradients per second on the C3 workload: each step runs
    rb_adjoint_device (forward, then the adjoint with alpha recomputed)
    on device-resident inputs; e2e through rb_adjoint with host buffers."""
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
    return dict(metric='disc-avg Tb spectra + dTb/dT, dTb/dP, dTb/dlnX gradients per second',
                value=1e3 / ms, unit='spectra+gradients/s', ms_per_step=ms, steps=n,
                config=dict(workload=GRAD_WORKLOAD, layers=nL, freqs=nf, rays=nb),
                gpu_launches_per_step=int(launches),
                e2e=dict(value=1.0 / float(np.mean(e2e)), unit='spectra+gradients/s',
                         h2d_bytes_per_step=int(h2d), d2h_bytes_per_step=int(d2h),
                         api='rb_adjoint (C ABI, host buffers)'))


BATCH_WORKLOAD = ('C4 batched retrieval sweep: {n} variants of the 1e-3..100 bar recipe (deep NH3 '
                  'log-U 1e-4..1e-3, deep T offset U(-10, 10) K, 300..1200 layers), 128 freqs '
                  '(0.5..50 GHz log), 32-ray disc quadrature, configuration-0 line lists; forward '
                  'Tb_avg + adjoint dTb/dT, dTb/dP, dTb/dlnX for every variant per step, replayed '
                  'from one captured CUDA graph, line-sum tiling from the autotuner')


def measure_batch(args, dev, n_var):
    """Spectra + gradients per second for a batch of n_var atmospheres
    (rb_adjoint_batch_device captured in a CUDA graph and replayed), beside
    the same variants run one call per atmosphere (rb_adjoint_device)."""
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

    best, tt = tune.tune_alpha(eng, step, key=('C4', n_var, nf),
                               candidates=((2, 2, 1024), (2, 4, 1024), (4, 1, 1024), (4, 2, 1024)),
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
                            tiling=dict(M=best[0], W=best[1], item_lines=best[2]),
                            tuning_ms={'{},{},{}'.format(*k): v for k, v in tt.items()},
                            l2='working set of tens of GB, larger than L2'),
                per_atmosphere_adjoint=dict(value=plain, unit='spectra+gradients/s',
                                            api='rb_adjoint_device, one atmosphere per call, '
                                                '16-variant sample scaled by layer count'),
                plain_dropin_finite_differences=dict(
                    value=fd_rate, unit='spectra+gradients/s',
                    how='plain drop-in forward (rb_forward_device, one atmosphere per call) '
                        'times 1 + 2 x 5 x nL central differences per gradient set'),
                speedup_vs_per_atmosphere_adjoint=value / plain,
                speedup_vs_plain_dropin=value / fd_rate)


IMAGE_WORKLOAD = ('C2 batched image rays: 256 x 256 impact parameters at 0.01 planet radius '
                  '(31,397 on the disc incl. limb rays of up to ~2000 segments, the rest off the '
                  'planet -> T_cmb) x 8 freqs (1.4..44 GHz), 1000 layers, C1 line lists')


def measure_image(args, dev, stream, flush):
    """Images per second (and rays/s) for the C2 grid: one rb_forward_device
    call per image, every ray in the same launches."""
    import torch
    from radiobear_gb300 import _native, catalog, synth
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
    sp = stream.cuda_stream

    def step():
        eng.forward_device(sp, nL, nb, dP.data_ptr(), dT.data_ptr(), dX.data_ptr(), dR.data_ptr(),
                           dN.data_ptr(), a['freqs'], db.data_ptr(), 71492.0, 66854.0, Tb.data_ptr())

    step()
    torch.cuda.synchronize()
    for _ in range(args.warmup):
        flush.zero_()
        step()
    n = max(3, min(args.steps, 20))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(n)]
    torch.cuda.synchronize()
    for s, e in ev:
        flush.zero_()
        s.record(stream)
        step()
        e.record(stream)
    torch.cuda.synchronize()
    ms = float(np.mean([s.elapsed_time(e) for s, e in ev]))
    t = Tb.cpu().numpy()
    on = np.hypot(a['b'][:, 0], a['b'][:, 1]) < 1.0
    rays = eng.raypath(a['R'], a['N'], a['b'][on][::97], 71492.0, 66854.0)
    eng.close()
    return dict(metric='brightness images per second', value=1e3 / ms, unit='images/s',
                rays_per_s=nb * 1e3 / ms, ms_per_step=ms, steps=n,
                config=dict(workload=IMAGE_WORKLOAD, layers=nL, freqs=nf, rays=nb,
                            rays_on_disc=int(on.sum()),
                            max_path_segments_sampled=int(rays['nseg'].max())),
                finite=bool(np.isfinite(t).all()),
                off_disc_is_tcmb=bool(np.all(t[~on] == 2.725)))


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


def read_profile_traffic():
    """dram bytes per absorption launch from the committed ncu summary."""
    path = os.path.join(ROOT, 'profiles', 'alpha_kernel_c1.md')
    try:
        with open(path) as fp:
            m = re.search(r'traffic_bytes_per_launch:\s*([0-9.eE+]+)', fp.read())
        return float(m.group(1)) if m else None
    except OSError:
        return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, 'MEASURED_PEAKS.json')) as fp:
            return json.load(fp)
    except (OSError, ValueError):
        return {}


# ------------------------------------------------------------------ CPU oracle
def _cpu_alpha_job(args):
    layers, freqs, gas, lines = args
    os.environ.setdefault('OMP_NUM_THREADS', '1')
    from oracle import oracle as O
    from radiobear_gb300 import synth
    C = {k: i for i, k in enumerate(synth.GAS_COLUMNS)}
    O.alpha_per_gas(freqs, gas[:, layers], C, lines, chunk=4)
    return len(layers)


def _cpu_ray_job(args):
    b, R, N, layers_alpha, T, Req, Rpol = args
    from oracle import oracle as O
    ds, lay = O.compute_ds(R, N, b, Req, Rpol)
    O.brightness(ds, lay, layers_alpha, T)
    return 1


def cpu_sample(wl, pool, nL_sample, nb_sample, cores):
    """Time alpha for nL_sample layers and ray path + Tb for nb_sample rays on
    the pool; returns (seconds per full spectrum, description)."""
    a = workload_arrays(wl)
    nL = a['P'].size
    idx = np.linspace(0, nL - 1, nL_sample).astype(int)
    chunks = [idx[i::cores] for i in range(cores) if idx[i::cores].size]
    t0 = time.perf_counter()
    pool.map(_cpu_alpha_job, [(c, wl.freqs, wl.gas, wl.lines) for c in chunks])
    t_alpha = time.perf_counter() - t0
    layers_alpha = np.full((wl.freqs.size, nL), 1e-6)   # geometry + scan cost is alpha-independent
    rays = wl.b[np.linspace(0, len(wl.b) - 1, nb_sample).astype(int)]
    t0 = time.perf_counter()
    pool.map(_cpu_ray_job, [(b, a['R'], a['N'], layers_alpha, a['T'], 71492.0, 66854.0) for b in rays])
    t_rays = time.perf_counter() - t0
    per_spec = t_alpha * nL / nL_sample + t_rays * len(wl.b) / nb_sample
    desc = ('alpha of {} of {} layers + ray path and Tb scan of {} of {} rays, {} worker processes; '
            'scaled to one spectrum').format(nL_sample, nL, nb_sample, len(wl.b), cores)
    return per_spec, desc


def make_pool():
    import multiprocessing as mp
    cores = os.cpu_count() or 1
    ctx = mp.get_context('spawn')
    return ctx.Pool(cores, initializer=_pool_init), cores


def _pool_init():
    os.environ['OMP_NUM_THREADS'] = '1'
    os.environ['OPENBLAS_NUM_THREADS'] = '1'
    sys.path.insert(0, ROOT)


def cpu_baseline(wl, budget_s, pool, cores):
    # calibrate on a small sample, then scale the sample to the budget
    per, _ = cpu_sample(wl, pool, nL_sample=cores, nb_sample=min(cores, 8), cores=cores)
    frac = min(1.0, budget_s / max(per, 1e-3))
    nL_s = max(cores, int(1000 * frac))
    nb_s = max(min(cores, 8), int(64 * frac))
    per, desc = cpu_sample(wl, pool, nL_sample=min(nL_s, 1000), nb_sample=min(nb_s, 64), cores=cores)
    return dict(value=1.0 / per, unit=UNIT, cores=cores, kind='port', sample=desc)


# ------------------------------------------------------------------ reference arm
def run_reference(args, rank, world):
    if rank != 0:
        return
    wl = load_workload()
    pool, cores = make_pool()
    try:
        budget = max(1.0, min(10.0, 150.0 / max(1, args.steps + args.warmup)))
        cal, _ = cpu_sample(wl, pool, nL_sample=cores, nb_sample=min(cores, 8), cores=cores)
        frac = min(1.0, budget / max(cal, 1e-3))
        nL_s = min(1000, max(cores, int(1000 * frac)))
        nb_s = min(64, max(min(cores, 8), int(64 * frac)))
        for _ in range(args.warmup):
            cpu_sample(wl, pool, nL_s, nb_s, cores)
        pers = []
        desc = ''
        for _ in range(args.steps):
            per, desc = cpu_sample(wl, pool, nL_s, nb_s, cores)
            pers.append(per)
    finally:
        pool.close()
        pool.join()
    ms = 1e3 * float(np.mean(pers))
    value = 1e3 / ms
    line = dict(metric=METRIC, value=value, unit=UNIT, n_gpus=args.gpus, steps=args.steps,
                warmup=args.warmup, ms_per_step=ms, higher_is_better=True, scaling='weak',
                vs_baseline=None, dtype='f64', data='synthetic', impl='reference',
                config=dict(workload=WORKLOAD, layers=1000, freqs=256, rays=64),
                cpu_baseline=dict(value=value, unit=UNIT, cores=cores, kind='port', sample=desc),
                e2e=dict(value=value, unit=UNIT, h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, rank, world, local_rank):
    import torch
    from radiobear_gb300 import _native, catalog

    pool = cores = None
    if rank == 0 and not args.no_cpu_baseline:
        pool, cores = make_pool()          # spawn before the first GPU call

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

    grads = measure_gradients(args, dev, stream, flush)
    image = None if args.no_image else measure_image(args, dev, stream, flush)
    batched = measure_batch(args, dev, args.batch_variants) if args.batch_variants > 0 else None
    if rank != 0:
        return
    # roofline of the dominant kernel (the line sums, timed alone on their
    # stream) and of the Tb scan
    flops, counts = alpha_flops(wl)
    fp32_peak = eng.probe_fp32_peak()
    ach = flops / (ph['alpha'] * 1e-3) / 1e12
    rays = eng.raypath(a['R'], a['N'], a['b'], 71492.0, 66854.0)
    sbytes = scan_bytes(rays['nseg'], nf, nb)
    peaks = measured_peaks()
    hbm = peaks.get('hbm_gbs')
    scan_gbs = sbytes / (ph['brightness'] * 1e-3) / 1e9
    value = world * args.steps / (tot_ms * 1e-3)
    line = dict(
        metric=METRIC, value=value, unit=UNIT, n_gpus=world, steps=args.steps, warmup=args.warmup,
        ms_per_step=tot_ms / args.steps, higher_is_better=True, scaling='weak', vs_baseline=None,
        dtype='f32', data='synthetic',
        config=dict(workload=WORKLOAD, layers=nL, freqs=nf, rays=nb, lines=counts,
                    parallelism='replicas' if world > 1 else 'single',
                    l2='256 MiB buffer written between steps; per-step CUDA events',
                    precision='f32 compensated line sums, f64 ray geometry, f32x2 tau'),
        e2e=dict(value=1.0 / float(np.mean(e2e_times)), unit=UNIT, h2d_bytes_per_step=int(h2d),
                 d2h_bytes_per_step=int(d2h), api='rb_forward (C ABI, pinned host buffers)'),
        gpu_launches=int(launches_per_step * args.steps),
        roofline=dict(bound='fp32', kernel='rb_alpha_lines_kernel', achieved=ach, peak=fp32_peak,
                      unit='TFLOP/s', frac=ach / fp32_peak, traffic=read_profile_traffic(),
                      algorithmic_flops_per_launch=flops,
                      peak_source='in-run FFMA probe (no fp32 entry in MEASURED_PEAKS.json)'),
        roofline_scan=dict(bound='hbm', kernel='rb_tb_chunk2_kernel+rb_tb_combine_kernel', achieved=scan_gbs, peak=hbm,
                           unit='GB/s', frac=(scan_gbs / hbm) if hbm else None,
                           algorithmic_bytes_per_launch=sbytes,
                           peak_source='MEASURED_PEAKS.json hbm_gbs (of measured)'),
        phase_ms=ph, clocks=clocks, gradients=grads, batched=batched, image=image)
    if pool is not None:
        try:
            line['cpu_baseline'] = cpu_baseline(wl, args.cpu_sample_s, pool, cores)
        finally:
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
