"""CPU: the algebra the packed brightness scan (rb_tb_chunk2_kernel) rests on,
restated in float64 numpy and checked against the oracle's direct
recurrence (oracle.brightness, brightness.py:53-117).

* Chunks: a path's steps are cut into chunks scanned from tau = 0 each;
  exp(-(tau_c + t)) = exp(-tau_c) exp(-t), so the chunk sums, scaled by
  exp(-tau) at each chunk's first node, add up to the path's sums.
* Node weights: sum_k (W_{k+1} + W_k) hd_k = sum_j W_j (hd_{j-1} + hd_j)
  inside a chunk, with hd_{-1} = hd_n = 0 at the chunk's ends; a chunk's
  first node carries W = exp(0) a_0 (none on the path's first chunk).
* Optical depth: a float32 running sum with its rounding errors collected
  by Fast2Sum and renormalised every 16 steps stays within a few float32
  ulp of the exact sum, including paths whose increments grow faster than
  the sum (deep layers), where Fast2Sum is not exact.
* Reverse sweep (rb_tb_adj_lambda / _suffix / _grad kernels): per-chunk
  sums of dTb/dtau, their suffix sums over the later chunks, then each
  chunk's nodes in reverse equal the oracle's vector-Jacobian product
  (oracle/adjoint.py brightness_vjp).
"""
import numpy as np
import pytest

from oracle import oracle as O


def _random_path(rng, nseg, nL=400, nf=5):
    ds = rng.uniform(0.1, 30.0, nseg + 1)                     # km
    layer = rng.integers(0, nL, nseg + 1)
    alpha = 10.0 ** rng.uniform(-9.0, -4.0, (nf, nL))         # cm^-1
    T = rng.uniform(100.0, 600.0, nL)
    return ds, layer, alpha, T


def _chunked(ds, layer, alpha, T, chunk):
    """The packed scan's decomposition in float64: per chunk the local
    optical depth and the node-weighted sums, then the combine."""
    hd = np.asarray(ds[:-1], dtype=float) * 1.0e5 / 2.0        # half ds, cm
    a = alpha[:, layer]                                        # [nf, nodes]
    Tn = T[layer]
    nsteps = len(hd)
    nf = alpha.shape[0]
    parts = []
    for i0 in range(0, nsteps, chunk):
        n = min(chunk, nsteps - i0)
        h = hd[i0:i0 + n]
        w = np.zeros(n + 1)                                    # node weights
        w[:-1] += h
        w[1:] += h
        x = (a[:, i0:i0 + n] + a[:, i0 + 1:i0 + n + 1]) * h    # step increments
        t = np.concatenate([np.zeros((nf, 1)), np.cumsum(x, axis=1)], axis=1)
        W = a[:, i0:i0 + n + 1] * np.exp(-t)
        if i0 == 0:
            W[:, 0] = 0.0                                      # W_0 = 0 on a path
        parts.append((t[:, -1], W @ w, W @ (Tn[i0:i0 + n + 1] * w)))
    tau0 = np.zeros(nf)
    iw = np.zeros(nf)
    tb = np.zeros(nf)
    for dt, piw, ptb in parts:
        sc = np.exp(-tau0)
        iw += sc * piw
        tb += sc * ptb
        tau0 = tau0 + dt
    return np.where(tb < O.T_CMB, O.T_CMB, tb / np.where(tb < O.T_CMB, 1.0, iw)), iw


@pytest.mark.parametrize('chunk', [1, 7, 64])
@pytest.mark.parametrize('nseg', [1, 63, 64, 65, 300])
def test_chunks_and_node_weights_reproduce_the_recurrence(chunk, nseg):
    rng = np.random.default_rng(nseg * 100 + chunk)
    ds, layer, alpha, T = _random_path(rng, nseg)
    tb_ref, _, _, iw_ref = O.brightness(ds, layer, alpha, T)
    tb, iw = _chunked(ds, layer, alpha, T, chunk)
    np.testing.assert_allclose(iw, iw_ref, rtol=1e-12)
    np.testing.assert_allclose(tb, tb_ref, rtol=1e-12)


def _fast2sum_tau(x, flush=16):
    """The kernel's optical depth in float32: th += x with the Fast2Sum
    error collected in ntl, renormalised every `flush` steps; returns
    th - ntl after each step (as float64)."""
    th = np.float32(0.0)
    ntl = np.float32(0.0)
    out = []
    for k, xk in enumerate(x.astype(np.float32)):
        s = np.float32(th + xk)
        ntl = np.float32(ntl + np.float32(np.float32(s - th) - xk))
        th = s
        out.append(float(th) - float(ntl))
        if k % flush == flush - 1:
            s = np.float32(th - ntl)
            ntl = np.float32(ntl + np.float32(s - th))
            th = s
    return np.array(out)


@pytest.mark.parametrize('growth', [1.0, 1.5, 3.0])
def test_fast2sum_optical_depth_tracks_the_exact_sum(growth):
    """Increments of one size, and increments growing geometrically (each
    step larger than the whole sum before it for growth > 2)."""
    rng = np.random.default_rng(int(growth * 10))
    n = 2000 if growth == 1.0 else int(30 / np.log10(growth))   # sums below ~1e25
    x = (rng.uniform(0.5, 1.5, n) * growth ** np.arange(n) * 1e-6).astype(np.float32)
    exact = np.cumsum(x.astype(np.float64))
    got = _fast2sum_tau(x)
    err = np.abs(got - exact) / exact
    # a plain float32 running sum drifts by ~n ulp; the collected errors
    # keep each prefix within a few ulp of its exact value
    assert np.max(err) < 4 * np.finfo(np.float32).eps, np.max(err)


def _chunked_vjp(ds, layer, alpha, T, gTb, chunk):
    """The reverse sweep as the adjoint kernels split it: each chunk's sum of
    dTb/dtau over its nodes (scaled by exp(-tau) at its first node), the
    suffix sums of those over the later chunks, then each chunk's nodes in
    reverse from its suffix (node i0 of a chunk belongs to the chunk before;
    node 0 takes only its segment term)."""
    nf, nL = alpha.shape
    d = np.asarray(ds[:-1], dtype=float) * 1.0e5                # cm
    lay = np.asarray(layer) % nL
    a = alpha[:, lay]
    Tn = T[lay]
    N = len(d)                                                  # steps
    dt = (a[:, :-1] + a[:, 1:]) * d / 2.0
    tau = np.concatenate([np.zeros((nf, 1)), np.cumsum(dt, axis=1)], axis=1)
    E = np.exp(-tau)
    E[:, 0] = 0.0
    c = np.zeros(N + 1)
    c[:-1] += d / 2.0
    c[1:] += d / 2.0
    iw = (a * E * c).sum(axis=1)
    tbl = (a * E * Tn * c).sum(axis=1)
    live = tbl >= O.T_CMB
    Tb = np.where(live, tbl / np.where(live, iw, 1.0), O.T_CMB)
    g = np.where(live, gTb, 0.0)
    rIW = np.where(live, 1.0 / np.where(live, iw, 1.0), 0.0)
    chunks = [(i0, min(chunk, N - i0)) for i0 in range(0, N, chunk)]
    # per-chunk sums of dTb/dtau over nodes i0+1 .. i0+ns
    S = []
    for i0, ns in chunks:
        k = np.arange(i0 + 1, i0 + ns + 1)
        wk = c[k] * (Tn[k] - Tb[:, None]) * rIW[:, None]
        S.append(-(wk * a[:, k] * E[:, k]).sum(axis=1))
    suffix = [sum(S[j + 1:], np.zeros(nf)) for j in range(len(S))]
    galpha = np.zeros((nf, nL))
    gT = np.zeros(nL)
    for (i0, ns), Ln in zip(chunks, suffix):
        Ln = Ln.copy()
        for t in range(i0 + ns, i0, -1):
            dprev = d[t - 1]
            dcur = d[t] if t < N else 0.0
            ck = 0.5 * (dprev + dcur)
            wk = ck * (Tn[t] - Tb) * rIW
            Lnext = Ln.copy()
            Ln = Ln - wk * a[:, t] * E[:, t]
            galpha[:, lay[t]] += g * (wk * E[:, t] + 0.5 * dprev * Ln + 0.5 * dcur * Lnext)
            gT[lay[t]] += np.sum(g * a[:, t] * E[:, t] * ck * rIW)
        if i0 == 0:
            galpha[:, lay[0]] += g * 0.5 * d[0] * Ln
    return galpha, gT


@pytest.mark.parametrize('chunk', [1, 7, 64])
@pytest.mark.parametrize('nseg', [1, 64, 65, 300])
def test_chunked_reverse_sweep_equals_the_vjp(chunk, nseg):
    from oracle import adjoint as A
    rng = np.random.default_rng(7 * nseg + chunk)
    ds, layer, alpha, T = _random_path(rng, nseg, nL=60)
    gTb = rng.normal(size=alpha.shape[0])
    ga_ref, gT_ref = A.brightness_vjp(ds, layer, alpha, T, gTb)
    ga, gT = _chunked_vjp(ds, layer, alpha, T, gTb, chunk)
    scale = np.max(np.abs(ga_ref))
    np.testing.assert_allclose(ga, ga_ref, rtol=0, atol=1e-10 * scale)
    np.testing.assert_allclose(gT, gT_ref, rtol=0, atol=1e-10 * np.max(np.abs(gT_ref)))


def _f32_dfs_add(h, l, v):
    """dfs_add of the adjoint kernels: (h, l) += v as a float pair."""
    f = np.float32
    s = f(h + v)
    bb = f(s - h)
    e = f(f(h - f(s - bb)) + f(v - bb))
    e = f(e + l)
    h2 = f(s + e)
    return h2, f(e - f(h2 - s))


def _f32_fast2sum_total(x, flush=16):
    """The forward scan's chunk total (th, -ntl) from its Fast2Sum steps."""
    f = np.float32
    th, ntl = f(0), f(0)
    for k, xk in enumerate(x):
        s = f(th + xk)
        ntl = f(ntl + f(f(s - th) - xk))
        th = s
        if k % flush == flush - 1:
            s = f(th - ntl)
            ntl = f(ntl + f(s - th))
            th = s
    return th, f(-ntl)


@pytest.mark.parametrize('profile', ['even', 'growth3', 'jump'])
def test_reverse_sweep_restarts_from_an_exact_chunk_sum(profile):
    """rb_tb_adj_grad_kernel subtracts a chunk's step increments in reverse
    from its local optical depth at the chunk's last node, so that depth
    must be the float-pair sum of the same float32 increments: the
    subtraction then returns every node's depth to float-pair accuracy.
    Started instead from the forward scan's Fast2Sum total (accurate to ~2
    ulp of the depth reached, not to ulp^2), steps larger than the sum
    before them (deep layers: 3x per step, or a jump from thin to opaque
    layers) leave up to ~1e-2 in the depth of the chunk's first nodes,
    i.e. ~1 % in exp(-tau) and in the gradients there."""
    rng = np.random.default_rng({'even': 1, 'growth3': 2, 'jump': 3}[profile])
    f = np.float32
    worst = {False: 0.0, True: 0.0}
    for _ in range(100):
        if profile == 'even':
            x = rng.uniform(0.5, 1.5, 64) * 10.0 ** rng.uniform(-3.0, 0.0)
        elif profile == 'growth3':
            n = int(rng.integers(10, 20))
            x = rng.uniform(0.5, 1.5, n) * 3.0 ** np.arange(n) * 10.0 ** rng.uniform(-6.0, -3.0)
        else:
            k = int(rng.integers(1, 60))
            x = np.concatenate([rng.uniform(0.5, 1.5, k) * 10.0 ** rng.uniform(-6.0, -2.0),
                                rng.uniform(0.5, 1.5, 64 - k) * 10.0 ** rng.uniform(0.0, 3.0)])
        x = x.astype(f)
        exact = np.concatenate([[0.0], np.cumsum(x.astype(np.float64))])
        h, l = f(0), f(0)
        for v in x:
            h, l = _f32_dfs_add(h, l, v)
        for fast, start in ((False, (h, l)), (True, _f32_fast2sum_total(x))):
            th, tl = start
            tau = [float(th) + float(tl)]
            for v in x[::-1]:
                th, tl = _f32_dfs_add(th, tl, f(-v))
                tau.append(float(th) + float(tl))
            tau = np.array(tau[::-1])
            live = exact < 80.0                       # nodes whose exp(-tau) is not 0
            err = np.max(np.abs(tau[live] - exact[live])) / max(1.0, exact[-1] * 2.0 ** -44)
            worst[fast] = max(worst[fast], err)
    assert worst[False] < 1e-8, worst
    if profile != 'even':
        assert worst[True] > 1e-5, worst


def _expint_cf(n, x):
    """A&S 5.1.22 by the modified Lentz method, as rb_expint.cuh."""
    tiny = 1e-300
    bb = x + n
    c = 1.0 / tiny
    d = 1.0 / bb
    h = d
    for i in range(1, 200):
        an = -float(i) * (n - 1 + i)
        bb += 2.0
        d = 1.0 / (an * d + bb)
        c = bb + an / c
        de = c * d
        h *= de
        if abs(de - 1.0) < 1e-16:
            break
    return h * np.exp(-x)


def _expint_series(n, x):
    """A&S 5.1.11 (E1) / 5.1.12 (E2) power series, as rb_expint.cuh."""
    euler = 0.57721566490153286061
    s = 0.0
    fact = 1.0 if n == 1 else -x
    for k in range(n, 60):
        fact *= -x / k
        term = fact / (k if n == 1 else k - 1)
        s += term
        if abs(term) < 1e-18 * abs(s) + 1e-300:
            break
    if n == 1:
        return -euler - np.log(x) - s
    return 1.0 + x * (np.log(x) - 1.0 + euler) - s


def test_disc_weighting_e2_and_its_derivative_e1():
    """The 'disc' weighting 2 E2(tau) (brightness.py:96, scipy.special.expn)
    and dE2/dx = -E1 of its adjoint: series up to x = 1, continued fraction
    above, 0 past 740; within 1e-14 relative of scipy from 1e-12 to 700."""
    from scipy.special import exp1, expn
    x = np.concatenate([np.logspace(-12, np.log10(700.0), 400), np.linspace(0.95, 1.05, 41)])
    for n, ref in ((2, expn(2, x)), (1, exp1(x))):
        got = np.array([_expint_series(n, v) if v <= 1.0 else _expint_cf(n, v) for v in x])
        np.testing.assert_allclose(got, ref, rtol=1e-14)
