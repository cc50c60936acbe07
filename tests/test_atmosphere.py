"""Atmosphere producer: computeProp and regrid on the GPU.

Pinned to ``tests/golden/f3.npz``, the reference's own
``AtmosphereBase.computeProp`` and ``regrid.regrid`` on an 80-layer
synthetic gas + cloud table: interpolation inside the table, and a grid
reaching above it (outward slope) and below it (dry adiabat)
(``tests/golden/make_golden.py f3``).  float64 throughout; the enclosed
mass is a parallel prefix sum on the device (the reference adds in layer
order), so properties agree to ~1e-13 relative.
"""
import numpy as np
import pytest

from oracle import atmosphere as OA
from radiobear_gb300 import synth
from tests import goldio as G

C = {k: i for i, k in enumerate(synth.GAS_COLUMNS)}
CL = {k: i for i, k in enumerate(synth.CLOUD_COLUMNS)}
J = synth.JUPITER
CASES = ('inside', 'extend', 'deeper')
RTOL = 1e-12


def f3():
    return G.load('f3')


def grid_of(z, name):
    from radiobear_gb300 import atmosphere as A
    n, pmin, pmax = z['case_' + name]
    return A.pressure_grid(z['gas_in'][C['P']], int(n), pmin or None, pmax or None)


def rel(a, b):
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), 1e-300)))


def rel_rows(a, b):
    """Relative error per table row, against max(|b|, 1e-12 x the row's
    largest magnitude) (rows of zeros must stay zero)."""
    floor = np.maximum(1e-12 * np.max(np.abs(b), axis=1, keepdims=True), 1e-300)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor)))


def test_oracle_props_match_reference():
    z = f3()
    assert rel(OA.compute_prop(z['gas_in'], C, J['Req'], J['p_ref'], J['GM_ref']), z['prop_in']) < 1e-14


@pytest.mark.parametrize('name', CASES)
def test_oracle_regrid_matches_reference(name):
    z = f3()
    g, c = OA.regrid(z['gas_in'], z['cloud_in'], C, CL, grid_of(z, name), J['Req'], J['p_ref'],
                     J['GM_ref'])
    assert rel(g, z['gas_' + name]) < 1e-14
    assert np.max(np.abs(c - z['cloud_' + name])) == 0.0
    p = OA.compute_prop(g, C, J['Req'], J['p_ref'], J['GM_ref'])
    assert rel(p, z['prop_' + name]) < 1e-14


def test_extend_case_extrapolates_both_ways():
    z = f3()
    P_in = z['gas_in'][C['P']]
    g = z['gas_extend']
    assert g[C['P']][0] < P_in[0] and g[C['P']][-1] > P_in[-1]
    T = g[C['T']]
    deep = g[C['P']] > P_in[-1]
    assert np.all(np.diff(T[deep]) > 0.0)                  # adiabat warms inward
    assert g[C['Z']][-1] == 0.0                            # renormalised at the deepest point


def test_pressure_grid_defaults():
    from radiobear_gb300 import atmosphere as A
    P = np.array([0.01, 1.0, 300.0])
    g = A.pressure_grid(P, 5)
    assert g[0] == 0.01 and abs(g[-1] - 300.0) < 1e-12 and g.size == 5
    g = A.pressure_grid(P, 4, 1e-3, 1e3)
    assert abs(g[0] - 1e-3) < 1e-18 and abs(g[-1] - 1e3) < 1e-9


@pytest.fixture(scope='module')
def engine():
    from radiobear_gb300 import _native
    e = _native.Engine(0)
    yield e
    e.close()


@pytest.mark.gpu
def test_gpu_props_match_reference(engine):
    from radiobear_gb300 import atmosphere as A
    z = f3()
    p = A.props(engine, z['gas_in'], C, J['Req'], J['p_ref'], J['GM_ref'])
    assert rel(p, z['prop_in']) < RTOL


@pytest.mark.gpu
@pytest.mark.parametrize('name', CASES)
def test_gpu_regrid_matches_reference(engine, name):
    from radiobear_gb300 import atmosphere as A
    z = f3()
    g, c = A.regrid(engine, z['gas_in'], C, grid_of(z, name), J['Req'], J['p_ref'], J['GM_ref'],
                    cloud=z['cloud_in'], Cl=CL)
    assert rel_rows(g, z['gas_' + name]) < RTOL
    assert np.max(np.abs(c - z['cloud_' + name])) <= 1e-12 * np.max(np.abs(z['cloud_' + name]))
    p = A.props(engine, g, C, J['Req'], J['p_ref'], J['GM_ref'])
    assert rel(p, z['prop_' + name]) < 1e-11


@pytest.mark.gpu
def test_gpu_batched_device_forms(engine):
    """rb_regrid_device / rb_atm_props_device over three tables of
    different layer counts equal one call per table."""
    import torch
    from radiobear_gb300 import atmosphere as A
    dev = torch.device('cuda')
    tabs = [synth.make_gas_table(n, 1e-2, pm) for n, pm in ((60, 100.0), (45, 300.0), (80, 30.0))]
    roles, chem = A.columns(C)
    ncol = chem.shape[1]
    nin = np.array([t.shape[1] for t in tabs], dtype=np.int32)
    gas = torch.tensor(np.concatenate([t[:ncol] for t in tabs], axis=1), dtype=torch.float64, device=dev)
    nout = 70
    grids = np.stack([A.pressure_grid(t[C['P']], nout, 3e-3, 600.0) for t in tabs])
    pg = torch.tensor(grids, dtype=torch.float64, device=dev)
    gout = torch.empty((ncol, 3 * nout), dtype=torch.float64, device=dev)
    prop = torch.empty((len(A.PROP_ROWS), 3 * nout), dtype=torch.float64, device=dev)
    s = torch.cuda.current_stream().cuda_stream
    from radiobear_gb300._native import _check, _ptr
    lib = engine.lib
    ip = A._ip
    _check(lib, lib.rb_regrid_device(engine._h, s, 3, ip(nin), ncol, ip(roles), _ptr(chem),
                                     gas.data_ptr(), 0, None, None, nout, pg.data_ptr(), nout,
                                     J['Req'], J['p_ref'], J['GM_ref'], gout.data_ptr(), None),
           'rb_regrid_device')
    nout_arr = np.full(3, nout, dtype=np.int32)
    _check(lib, lib.rb_atm_props_device(engine._h, s, 3, ip(nout_arr), ncol, ip(roles), _ptr(chem),
                                        gout.data_ptr(), J['Req'], J['p_ref'], J['GM_ref'],
                                        prop.data_ptr()), 'rb_atm_props_device')
    torch.cuda.synchronize()
    gout, prop = gout.cpu().numpy(), prop.cpu().numpy()
    for v, t in enumerate(tabs):
        g1, _ = A.regrid(engine, t, C, grids[v], J['Req'], J['p_ref'], J['GM_ref'])
        assert np.array_equal(gout[:, v * nout:(v + 1) * nout], g1)
        p1 = A.props(engine, g1, C, J['Req'], J['p_ref'], J['GM_ref'])
        assert rel(prop[:, v * nout:(v + 1) * nout], p1) < 1e-13
        cl = np.zeros((len(CL), t.shape[1]))
        for k in ('Z', 'T', 'P'):
            cl[CL[k]] = t[C[k]]
        go, _ = OA.regrid(t[:ncol], cl, C, CL, grids[v], J['Req'], J['p_ref'], J['GM_ref'])
        assert rel_rows(g1, go) < RTOL


@pytest.mark.gpu
def test_gpu_regrid_atm_dropin(engine):
    """regrid_atm / compute_prop mutate a reference-shaped atmosphere as
    regrid.regrid and computeProp do."""
    from argparse import Namespace
    from radiobear_gb300 import atmosphere as A
    z = f3()
    atm = Namespace(gas=z['gas_in'].copy(), cloud=z['cloud_in'].copy(),
                    config=Namespace(C=C, Cl=CL, Req=J['Req'], p_ref=J['p_ref'], GM_ref=J['GM_ref'],
                                     regridType='none'))
    assert A.regrid_atm(atm, engine=engine) == 0
    assert A.regrid_atm(atm, regridType=250, Pmin=3.0e-3, Pmax=1000.0, engine=engine) == 1
    assert rel_rows(atm.gas, z['gas_extend']) < RTOL
    A.compute_prop(atm, engine=engine)
    assert rel(atm.property, z['prop_extend']) < 1e-11
