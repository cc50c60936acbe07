"""Accuracy of the GPU results at the benchmarked sizes against the float64
oracle, for the ``-m gpu`` tests and the ``accuracy`` block of each
``bench.py`` workload.

TEST INFRASTRUCTURE ONLY (same rule as ``oracle/oracle.py``): these are the
checker, run outside any timed region; the ``radiobear_gb300`` package never
imports them.

* spectra (C1, 1000 layers x 256 freqs x 64 disc rays): max |dTb| over every
  ray and frequency and over the disc average, and the largest relative
  error of the absorption table;
* image rays (C2, 256 x 256 grid at 8 freqs): a sample of >= 256 rays that
  reach the planet, holding the 16 rays with the longest paths (limb rays
  crossing up to ~1900 segments) and the 16 outermost rays;
* gradients (C3, 1000 x 64 x 16): directional derivatives along the
  benchmark's random perturbations against the float64 autograd reference
  (``oracle/torch64.py``) and against central differences of the oracle
  (step 1e-4), plus the per-parameter error of every layer's gradient;
* batches (C4): sampled variants' Tb_avg and a gradient direction.
"""
from __future__ import annotations

import numpy as np

from oracle import adjoint as A
from oracle import parallel as OP


def spectra(pool, freqs, gas, C, R, N, b, w, lines, Req, Rpol, Tb, Tb_avg, layers=None):
    """GPU Tb [nb, nf] / Tb_avg [nf] (/ layers [nf, nL]) against the oracle."""
    ref_layers = OP.layers(pool, freqs, gas, C, lines)
    tb, nseg = OP.rays(pool, R, N, b, Req, Rpol, ref_layers, gas[C['T']])
    avg = np.tensordot(w, tb, axes=1)
    out = dict(rays=int(len(b)), max_abs_dTb_K=float(np.max(np.abs(Tb - tb))),
               max_abs_dTb_avg_K=float(np.max(np.abs(Tb_avg - avg))),
               reference='float64 oracle (numpy restatement pinned to the reference)')
    if layers is not None:
        out['alpha_max_rel_err'] = float(np.max(np.abs(layers - ref_layers) / np.abs(ref_layers)))
    return out


def image_sample(b, nseg, n=256, n_limb=16, seed=0):
    """Indices of >= n rays that reach the planet: the n_limb longest paths,
    the n_limb outermost, and a seeded random fill."""
    hit = np.nonzero(nseg > 0)[0]
    r = np.hypot(b[hit, 0], b[hit, 1])
    longest = hit[np.argsort(-nseg[hit], kind='stable')[:n_limb]]
    outer = hit[np.argsort(-r, kind='stable')[:n_limb]]
    chosen = list(dict.fromkeys(list(longest) + list(outer)))
    rest = np.setdiff1d(hit, chosen)
    fill = np.random.default_rng(seed).choice(rest, size=max(0, n - len(chosen)), replace=False)
    return np.array(chosen + sorted(fill.tolist()), dtype=np.int64), longest, outer


def image(pool, freqs, gas, C, R, N, b, lines, Req, Rpol, Tb_sel):
    """GPU Tb of the sampled rays [n, nf] against the oracle."""
    ref_layers = OP.layers(pool, freqs, gas, C, lines)
    tb, nseg = OP.rays(pool, R, N, b, Req, Rpol, ref_layers, gas[C['T']])
    return dict(rays=int(len(b)), max_path_segments=int(nseg.max()),
                max_abs_dTb_K=float(np.max(np.abs(Tb_sel - tb))),
                reference='float64 oracle'), tb, nseg


def gradients(pool, freqs, gas, C, R, N, b, w, lines, Req, Rpol, grad_gpu, g, n_dir=32, n_fd=8,
              seed=3, device='cpu', disc=False):
    """grad_gpu: dict(dT, dP, dlnX) of loss = sum_f g_f Tb_avg(f).  Returns
    the directional errors against the float64 autograd reference (n_dir
    perturbations) and against central differences (the first n_fd), and
    the per-parameter max error over the layers relative to the largest
    entry."""
    from oracle import torch64 as T64
    from oracle import oracle as O
    rng = np.random.default_rng(seed)
    dirs = [A.random_direction(rng, gas, C) for _ in range(n_dir)]
    bb = np.zeros((1, 2)) if disc else b
    ww = np.ones(1) if disc else w
    paths = [O.compute_ds(R, N, x, Req, Rpol) for x in bb]
    m = T64.Model(gas, C, lines, freqs, device=device, block=64 if device != 'cpu' else 8)
    lnX = np.log(np.stack([gas[C['NH3']], gas[C['H2O']], gas[C['H2S']]]))
    _, _, dT, dP, dX = T64.gradients(m, gas[C['T']], gas[C['P']], lnX, paths, ww, g, disc=disc)
    ref = dict(dT=dT, dP=dP, dlnX=dX)
    ad = np.array([A.dot(grad_gpu, d) for d in dirs])
    rd = np.array([A.dot(ref, d) for d in dirs])
    fd = OP.directional_fd(pool, gas, C, R, N, freqs, bb, lines, Req, Rpol, ww, g, dirs[:n_fd],
                           disc=disc)
    vec = {}
    for k, (x, y) in dict(T=(grad_gpu['dT'], dT), P=(grad_gpu['dP'], dP),
                          NH3=(grad_gpu['dlnX'][0], dX[0]), H2O=(grad_gpu['dlnX'][1], dX[1]),
                          H2S=(grad_gpu['dlnX'][2], dX[2])).items():
        vec[k] = float(np.max(np.abs(x - y)) / max(np.max(np.abs(y)), 1e-300))
    return dict(directions=n_dir, dir_rel_err_vs_fp64_autograd=float(np.max(np.abs(ad - rd) / np.abs(rd))),
                fd_directions=n_fd,
                dir_rel_err_vs_central_differences=float(np.max(np.abs(ad[:n_fd] - fd) / np.abs(fd))),
                fp64_autograd_vs_central_differences=float(np.max(np.abs(rd[:n_fd] - fd) / np.abs(fd))),
                layer_grad_max_err_rel=vec,
                reference='float64 torch autograd of the oracle restatement (oracle/torch64.py); '
                          'central differences of the numpy oracle, step 1e-4')
