"""The oracle on many host cores: absorption by blocks of layers, ray paths
and scans by ray, finite differences by perturbation, each in a worker of a
``spawn`` process pool (made before any GPU call, or with the spawn context,
so no worker is forked from a process that holds a CUDA context).

TEST INFRASTRUCTURE ONLY (same rule as ``oracle/oracle.py``): used by the
``-m gpu`` accuracy tests and by the accuracy / CPU-baseline legs of
``bench.py`` as the checker, never by the ``radiobear_gb300`` package.
"""
from __future__ import annotations

import os
import sys

import numpy as np

from oracle import oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _init():
    os.environ['OMP_NUM_THREADS'] = '1'
    os.environ['OPENBLAS_NUM_THREADS'] = '1'
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)


def make_pool(processes=None):
    """A spawn-context pool over the host cores; returns (pool, cores)."""
    import multiprocessing as mp
    cores = processes or os.cpu_count() or 1
    return mp.get_context('spawn').Pool(cores, initializer=_init), cores


def _alpha_job(args):
    freqs, gas, C, lines, kw = args
    per = O.alpha_per_gas(freqs, gas, C, lines, chunk=4, **kw)
    return per


def alpha_per_gas(pool, freqs, gas, C, lines, blocks=None, **kw):
    """O.alpha_per_gas over blocks of layers in the pool: [nL, nf, nC]."""
    nL = gas.shape[1]
    blocks = blocks or max(1, min(nL, 4 * getattr(pool, '_processes', 1)))
    cuts = np.linspace(0, nL, blocks + 1).astype(int)
    jobs = [(freqs, gas[:, a:b], C, lines, kw) for a, b in zip(cuts[:-1], cuts[1:]) if b > a]
    return np.concatenate(pool.map(_alpha_job, jobs), axis=0)


def layers(pool, freqs, gas, C, lines, scale=False, **kw):
    """Alpha.layers [nf, nL] (the oracle's total_alpha over the pool's blocks)."""
    per = alpha_per_gas(pool, freqs, gas, C, lines, **kw)
    tot, _ = O.total_alpha(per, O.layer_scale(scale, gas.shape[1]))
    return tot


def _ray_job(args):
    R, N, b, Req, Rpol, orientation, alpha, T, disc = args
    bb = [0.0, 0.0] if disc else b
    ds, lay = O.compute_ds(R, N, bb, Req, Rpol, orientation)
    tb, _, _, _ = O.brightness(ds, lay, alpha, T, disc=disc)
    return tb, (0 if ds is None else len(ds))


def rays(pool, R, N, b, Req, Rpol, alpha, T, orientation=(0.0, 0.0), disc=False):
    """Tb [nb, nf] and path lengths [nb] of every ray (Brightness.single)."""
    out = pool.map(_ray_job, [(R, N, np.asarray(bb, dtype=np.float64), Req, Rpol, orientation, alpha,
                               T, disc) for bb in b], chunksize=max(1, len(b) // (8 * pool._processes)))
    return np.array([o[0] for o in out]), np.array([o[1] for o in out])


def _loss_job(args):
    gas, C, R, N, freqs, b, lines, Req, Rpol, w, g, disc = args
    tb, _, avg = O.forward(gas, C, R, N, freqs, b, lines, Req, Rpol, weights=w, disc=disc)
    return float(np.dot(g, avg))


def directional_fd(pool, gas, C, R, N, freqs, b, lines, Req, Rpol, w, g, directions, h=1e-4,
                   disc=False):
    """Central differences (step h) of loss = sum_f g_f Tb_avg(f) along each
    direction (oracle.adjoint.perturb), every forward model in its own
    worker."""
    from oracle import adjoint as A
    jobs = []
    for d in directions:
        for s in (h, -h):
            jobs.append((A.perturb(gas, C, d, s), C, R, N, freqs, b, lines, Req, Rpol, w, g, disc))
    vals = pool.map(_loss_job, jobs, chunksize=1)
    return np.array([(vals[2 * k] - vals[2 * k + 1]) / (2.0 * h) for k in range(len(directions))])
