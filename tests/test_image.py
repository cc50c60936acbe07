"""Image grids (C2-style): off-disc rays give T_cmb, the image of an
unrotated planet is mirror symmetric, and limb rays near the edge agree
with the oracle (tangent branch)."""
import numpy as np
import pytest

from radiobear_gb300 import synth
from tests import goldio as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope='module')
def image():
    from radiobear_gb300 import _native, catalog
    from radiobear_gb300._native import x_matrix
    z = G.load('c0')
    g = G.gas_table(z)
    e = _native.Engine(0)
    catalog.upload(e, G.c0_lines())
    e.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
    freqs = np.array([1.4, 3.0, 6.0, 10.0, 15.0, 22.0, 33.0, 44.0])
    b = synth.image_grid(96, 0.022)
    out = e.forward(g[G.C['P']], g[G.C['T']], x_matrix(g, G.C), z['prop_R'], z['prop_N'], freqs, b,
                    G.REQ, G.RPOL)
    yield z, g, freqs, b, out['Tb']
    e.close()


def test_off_disc_and_finite(image):
    """b beyond the unit circle is off the planet (raypath.py:126-127):
    exactly T_cmb.  Inside the oblate limb (axis ratio Rpol/Req) every ray
    sees the atmosphere; between the two, rays pass over the poles."""
    z, g, freqs, b, Tb = image
    off = np.hypot(b[:, 0], b[:, 1]) >= 1.0
    assert np.all(Tb[off] == 2.725)
    assert np.all(np.isfinite(Tb))
    k = G.RPOL / G.REQ
    inside = b[:, 0] ** 2 + (b[:, 1] / k) ** 2 < 0.98
    assert np.all(Tb[inside] > 2.725)


def test_mirror_symmetry(image):
    z, g, freqs, b, Tb = image
    n = 96
    img = Tb.reshape(n, n, -1)           # [y, x, f], x = (i - n/2) * spacing
    # x -> -x maps column i to n - i (column 0 has no partner)
    assert np.max(np.abs(img[:, 1:, :] - img[:, :0:-1, :])) < 1e-6


def test_limb_rays_match_oracle(image):
    from oracle import oracle as O
    z, g, freqs, b, Tb = image
    r = np.hypot(b[:, 0], b[:, 1])
    idx = np.where((r > 0.96) & (r < 1.0))[0][:4]
    assert idx.size == 4
    per = O.alpha_per_gas(freqs, g, G.C, G.c0_lines())
    layers, _ = O.total_alpha(per, O.layer_scale(False, g.shape[1]))
    for i in idx:
        ds, lay = O.compute_ds(z['prop_R'], z['prop_N'], b[i], G.REQ, G.RPOL)
        tb, _, _, _ = O.brightness(ds, lay, layers, g[G.C['T']])
        assert np.max(np.abs(Tb[i] - tb)) < 1e-3, (b[i], Tb[i], tb)
