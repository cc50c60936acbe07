"""rb_brightness_noalloc: the brightness scan for callers that cannot
allocate device memory (applications that own all device memory, plugins
inside a framework's allocator, real-time loops that forbid cudaMalloc).

It is checked through the C ABI against the allocating entry point
rb_brightness on the same reference ray paths and absorption, twice in a row
(the second call reuses the fixed scratch array left by the first).  This
file sorts last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes

import numpy as np
import pytest

from tests import goldio as G

pytestmark = pytest.mark.gpu

TB_ATOL = 1e-3          # the brightness tolerance used by the other GPU tests


def _lib():
    from radiobear_gb300 import _native
    lib = _native.load_library()
    f = lib.rb_brightness_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                  ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                  ctypes.c_void_p]
    return lib, f


def _inputs():
    z = G.load('c0')
    g = G.gas_table(z)
    nb = len(z['rays_b'])
    nL = g.shape[1]
    ms = 2 * nL + 4
    nseg = np.zeros(nb, dtype=np.int32)
    ds = np.zeros((nb, ms))
    lay = np.zeros((nb, ms), dtype=np.int32)
    for i in range(nb):
        r = z['ray{}_ds'.format(i)]
        nseg[i] = r.size
        ds[i, :r.size] = r
        lay[i, :r.size] = z['ray{}_layer'.format(i)]
    return g[G.C['T']], z['alpha_layers'], nseg, ds, lay


def test_noalloc_matches_allocating_entry_point_twice():
    import torch
    from radiobear_gb300 import _native
    T, layers, nseg, ds, lay = _inputs()
    nf, nL = layers.shape
    nb, ms = ds.shape
    eng = _native.Engine(0)
    try:
        ref = eng.brightness(T, layers, nseg, ds, lay)['Tb']
    finally:
        eng.close()
    lib, fn = _lib()
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(dev)
    d_a = torch.as_tensor(np.ascontiguousarray(layers.T), dtype=torch.float32, device=dev)
    d_T = torch.as_tensor(T, dtype=torch.float64, device=dev)
    d_n = torch.as_tensor(nseg, dtype=torch.int32, device=dev)
    d_ds = torch.as_tensor(ds, dtype=torch.float64, device=dev)
    d_l = torch.as_tensor(lay, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        d_Tb = torch.full((nb, nf), -1.0, dtype=torch.float64, device=dev)
        rc = fn(ctypes.c_void_p(stream.cuda_stream), nL, nf, d_a.data_ptr(), d_T.data_ptr(), nb,
                d_n.data_ptr(), d_ds.data_ptr(), d_l.data_ptr(), ms, d_Tb.data_ptr())
        assert rc == 0, lib.rb_last_error().decode()
        torch.cuda.synchronize(dev)
        got = d_Tb.cpu().numpy()
        assert np.max(np.abs(got - ref)) < TB_ATOL, call
        assert np.max(np.abs(got - G.load('c0')['Tb_rays'])) < TB_ATOL, call


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib, fn = _lib()
    nf, nL, nb, ms = 256, 1000, 512, 2004          # 512 * 16 * 256 > 524288
    rc = fn(None, nL, nf, ctypes.c_void_p(1), ctypes.c_void_p(1), nb, ctypes.c_void_p(1),
            ctypes.c_void_p(1), ctypes.c_void_p(1), ms, ctypes.c_void_p(1))
    assert rc == 1
    assert b'exceeds the fixed maximum' in lib.rb_last_error()


def test_noalloc_many_rays_one_frequency_and_exact_tcmb():
    """More rays than a grid's y or z dimension holds (65,535), one
    frequency, short paths: every ray matches rb_brightness, and rays with
    no path (off the planet) are T_cmb = 2.725 K exactly, as there."""
    import torch
    from radiobear_gb300 import _native
    rng = np.random.default_rng(7)
    nL, nf, nb, ms = 12, 1, 70000, 4
    T = np.linspace(120.0, 400.0, nL)
    layers = rng.uniform(1e-7, 1e-5, size=(nf, nL))
    nseg = rng.integers(0, ms + 1, size=nb).astype(np.int32)
    nseg[:5] = 0
    ds = rng.uniform(10.0, 200.0, size=(nb, ms))
    lay = np.sort(rng.integers(0, nL, size=(nb, ms)), axis=1).astype(np.int32)
    for i in range(nb):
        ds[i, nseg[i]:] = 0.0
        lay[i, nseg[i]:] = 0
    eng = _native.Engine(0)
    try:
        ref = eng.brightness(T, layers, nseg, ds, lay)['Tb']
    finally:
        eng.close()
    lib, fn = _lib()
    dev = torch.device('cuda', 0)
    torch.cuda.set_device(dev)
    d_a = torch.as_tensor(np.ascontiguousarray(layers.T), dtype=torch.float32, device=dev)
    d_T = torch.as_tensor(T, dtype=torch.float64, device=dev)
    d_n = torch.as_tensor(nseg, dtype=torch.int32, device=dev)
    d_ds = torch.as_tensor(ds, dtype=torch.float64, device=dev)
    d_l = torch.as_tensor(lay, dtype=torch.int32, device=dev)
    d_Tb = torch.full((nb, nf), -1.0, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = fn(ctypes.c_void_p(stream.cuda_stream), nL, nf, d_a.data_ptr(), d_T.data_ptr(), nb,
            d_n.data_ptr(), d_ds.data_ptr(), d_l.data_ptr(), ms, d_Tb.data_ptr())
    assert rc == 0, lib.rb_last_error().decode()
    torch.cuda.synchronize(dev)
    got = d_Tb.cpu().numpy()
    assert np.max(np.abs(got - ref)) < TB_ATOL
    off = nseg <= 1
    assert off.any()
    assert np.all(got[off] == 2.725) and np.all(ref[off] == 2.725)


def test_noalloc_rejects_a_grid_beyond_its_limits():
    lib, fn = _lib()
    # one ray, one frequency, a path of 128 * 65536 segments: the scratch
    # holds it but the chunk dimension of the grid does not
    rc = fn(None, 10, 1, ctypes.c_void_p(1), ctypes.c_void_p(1), 1, ctypes.c_void_p(1),
            ctypes.c_void_p(1), ctypes.c_void_p(1), 128 * 65536, ctypes.c_void_p(1))
    assert rc == 1
    assert b'launch grid' in lib.rb_last_error()
