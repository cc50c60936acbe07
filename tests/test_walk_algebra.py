"""CPU: the ray walk's reformulation (rb_raypath_kernel in
radiobear_gb300/csrc/rb_raypath.cu) restated in float64 numpy and checked
against the unmodified reference's own paths (tests/golden c0 and
benchmark fixtures, compute_ds of raypath.py:108-273).

* After the one refraction at the top the direction s is fixed, and each
  step of raypath.py:191-196 satisfies u_{i+1}^2 = u_i^2 + D_i exactly,
  u = r.s and D_i = E_i^2 (R_next^2 - R_cur^2), E^2 = k^2 sin^2(lat) +
  cos^2(lat) at the step's start point, so the walk carries w = u^2 and
  takes u_{i+1} = -/+ sqrt(w + D_i) (ingress / egress), ds = u_{i+1} - u_i.
  The first step's radii are evaluated at the latitude of findEdge's
  interpolated edge point, not at that of the shell point the step starts
  from (the reference takes pclat from the edge before the loop,
  raypath.py:143-146, and the loop's first rNextMag uses it, line 182).
* Blocks of 32 steps in parallel: with E^2 fixed for the block's start
  points, w after each step is a prefix sum of D; E^2 is guessed, the
  points computed and E^2 evaluated again until it no longer changes (at
  most four rounds, else the steps are taken one by one).  The fixed point
  is the sequential recurrence itself, bit for bit.
"""
import math

import numpy as np

from oracle import oracle as O
from tests import goldio as G


def _start(R, N, b, Req, Rpol, orientation, edge_latitude=True):
    """The walk's start: findEdge, the shell point and normal at the edge's
    latitude and longitude, the refracted direction (oracle helpers, the
    reference's first loop iteration)."""
    req = np.asarray(R, float)
    nr = np.asarray(N, float)
    if b[0] ** 2 + b[1] ** 2 >= 1.0:
        return None
    k = Rpol / Req
    tip, rotate = O.aspect(orientation, 1.0 - Rpol / Req)
    edge, _ = O.find_edge(b, req[0], tip, rotate, k)
    if edge is None:
        return None
    pclat, dlng = O._latlng(edge)
    geo = O.Ellipse(k)
    geo.calc(req[0], pclat, dlng)
    s = O._rotate2planet(rotate, tip, np.array([0.0, 0.0, -1.0]))
    n = geo.n
    t_inc = math.acos(-float(np.dot(s, n)))
    nratio = nr[0] / nr[1]
    t_tran = math.asin(nratio * math.sin(t_inc))
    s = nratio * s + (nratio * math.cos(t_inc) * n - math.cos(t_tran) * n)
    r0 = geo.r.copy()
    lat0 = math.radians(pclat) if edge_latitude else math.asin(r0[1] / math.sqrt(r0 @ r0))
    return dict(req=req, R2=req * req, k=k, r0=r0, s=s, lat0=lat0, rNorm=req[0])


def _e2(k, lat):
    if lat == 0.0:
        lat = 1.0e-6                      # shape.py:232-234
    return k * k * math.sin(lat) ** 2 + math.cos(lat) ** 2


def _e2_at(st, S):
    pt = st['r0'] + S * st['s']
    return _e2(st['k'], math.asin(pt[1] / math.sqrt(pt @ pt)))


def _folds(st, S, layer, direction):
    """The reference's incidence test at the new point: past 90 degrees it
    reflects s (handled in float64 by the kernel; none of these rays)."""
    pt = st['r0'] + S * st['s']
    pl, dl = O._latlng(pt)
    geo = O.Ellipse(st['k'])
    geo.calc(st['req'][layer], pl, dl)
    return -direction * float(np.dot(st['s'], geo.n)) < 0.0


def walk(st, block=0, max_rounds=4):
    """(ds, layers, [(rounds, steps) per parallel block]).  block = 0: one
    step at a time."""
    req, R2 = st['req'], st['R2']
    nL = len(req)
    u = float(np.dot(st['r0'], st['s']))
    w, S = u * u, 0.0
    layer, direction, first = 0, 1, True
    ds_out, lay_out, blocks = [], [], []
    while True:
        m = 0
        if block and not first and direction != 0:
            m = min(block, nL - 2 - layer) if direction == 1 else min(block, layer - 1)
        if m >= 2:
            L = layer + direction * np.arange(m)
            dR = R2[L + direction] - R2[L]
            e2 = np.full(m, _e2_at(st, S))          # predictor: E^2 of the block's start
            settled = False
            for rnd in range(1, max_rounds + 1):
                ws = np.empty(m + 1)
                ws[0] = w
                for j in range(m):
                    ws[j + 1] = ws[j] + e2[j] * dR[j]
                if np.any(ws[1:] < 0.0):             # a tangent or the exit in the block
                    break
                us = np.concatenate([[u], -np.sqrt(ws[1:]) if direction == 1 else np.sqrt(ws[1:])])
                dss = np.diff(us)
                if np.any(dss < 0.0):
                    break
                Ss = np.empty(m + 1)
                Ss[0] = S
                for j in range(m):
                    Ss[j + 1] = Ss[j] + dss[j]
                e2n = np.array([_e2_at(st, Ss[j]) for j in range(m)])
                if np.array_equal(e2n, e2):
                    settled = True
                    break
                e2 = e2n
            if settled and not any(_folds(st, Ss[j + 1], layer + direction * (j + 1), direction)
                                   for j in range(m)):
                blocks.append((rnd, m))
                ds_out += list(dss)
                lay_out += list(L)
                w, u, S = ws[-1], us[-1], Ss[-1]
                layer += direction * m
                continue
        # one step
        e2s = _e2(st['k'], st['lat0']) if first else _e2_at(st, S)
        first = False
        dvec = 1 if direction == 1 else (-1 if direction == -1 else 0)
        disc = w + e2s * (R2[layer + dvec] - R2[layer])
        if disc < 0.0:
            if direction != 1:
                break                                  # egress: leaves the atmosphere
            direction = 0                              # tangent chord
            ds = -2.0 * u
            if ds > st['rNorm']:
                break
            unext = -u
        else:
            unext = -math.sqrt(disc) if direction == 1 else math.sqrt(disc)
            ds = unext - u
            w = disc
        if ds < 0.0:
            break
        ds_out.append(ds)
        lay_out.append(layer)
        S, u = S + ds, unext
        layer += 0 if direction == 0 else direction
        if direction == 0:
            direction = -1
        elif _folds(st, S, layer, direction):
            raise AssertionError('fold: not restated')
        nxt = layer + (-1 if direction == -1 else 1)
        if not (-nL <= nxt < nL) or not (-nL <= layer < nL):   # raypath.py:253-264
            break
    return np.array(ds_out), np.array(lay_out, dtype=np.int64), blocks


def _cases():
    z, zb = G.load('c0'), G.load('benchmark')
    out = []
    for i, b in enumerate(z['rays_b']):
        out.append((z, b, (0.0, 0.0), G.REQ, G.RPOL, 'ray{}'.format(i)))
    for i, b in enumerate(z['tilt_b']):
        out.append((z, b, tuple(z['tilt_orientation']), G.REQ, G.RPOL, 'tilt{}'.format(i)))
    for i, b in enumerate(zb['b']):
        out.append((zb, b, (0.0, 0.0), float(zb['Req']), float(zb['Rpol']), 'ray{}'.format(i)))
    return out


def test_w_recurrence_reproduces_the_reference_paths():
    """Every fixture ray (on-axis, off-equator, limb with its tangent chord,
    tilted, the 1000-layer benchmark): the same layers, ds within 1e-9
    (measured <= 8.3e-10, the longest limb path)."""
    n = 0
    for z, b, orient, Req, Rpol, tag in _cases():
        st = _start(z['prop_R'], z['prop_N'], b, Req, Rpol, orient)
        ref = z[tag + '_ds']
        if st is None:
            assert ref.size == 0
            continue
        ds, lay, _ = walk(st)
        assert ds.size == ref.size and np.array_equal(lay, z[tag + '_layer']), tag
        assert np.max(np.abs(ds - ref) / ref) < 1e-9, tag
        n += 1
    assert n >= 19


def test_block_steps_reach_the_sequential_walk_bitwise():
    """32-step blocks settled by re-evaluating E^2: identical ds and layers
    to the step-by-step walk on every ray; equatorial and nadir rays settle
    in two rounds (the predictor and one check), off-equator and tilted
    rays within four; over 90 % of all steps run in blocks."""
    steps = in_blocks = 0
    for z, b, orient, Req, Rpol, tag in _cases():
        st = _start(z['prop_R'], z['prop_N'], b, Req, Rpol, orient)
        if st is None:
            continue
        d1, l1, _ = walk(st)
        d2, l2, blocks = walk(st, block=32)
        assert np.array_equal(d1, d2) and np.array_equal(l1, l2), tag
        assert all(r <= 4 for r, _ in blocks)
        if b[1] == 0.0 and orient == (0.0, 0.0):
            assert all(r == 2 for r, _ in blocks), tag
        steps += d1.size
        in_blocks += sum(m for _, m in blocks)
    assert in_blocks > 0.9 * steps


def test_first_step_takes_the_edge_latitude():
    """Planted in the restatement: the first step's radii at the latitude of
    the shell point instead of the edge's.  Off-equator and tilted rays then
    miss the reference's first segment by more than 1e-5 (up to 4e-3)."""
    worst = 0.0
    for z, b, orient, Req, Rpol, tag in _cases():
        if b[1] == 0.0 and orient == (0.0, 0.0):
            continue
        st = _start(z['prop_R'], z['prop_N'], b, Req, Rpol, orient, edge_latitude=False)
        if st is None:
            continue
        ds, _, _ = walk(st)
        worst = max(worst, abs(ds[0] / z[tag + '_ds'][0] - 1.0))
    assert worst > 1e-5
