"""Image / profile / spectrum pipeline around the GPU forward model
(radiobear_gb300.image): ``set_b`` requests, image rows and the FileIO text
formats, against ``tests/golden/f4.npz`` made by running the reference
(``tests/golden/make_golden.py f4``)."""
from argparse import Namespace

import numpy as np
import pytest

from radiobear_gb300 import image, synth
from tests import goldio as G

REQ, RPOL = G.REQ, G.RPOL


def f4():
    return G.load('f4')


@pytest.mark.parametrize('name,spacing,block', [('grid_a', 0.1, [1, 1]), ('grid_b', 0.1, [2, 4]),
                                                ('grid_c', 0.05, [3, 3]), ('grid_d', 0.25, [1, 1])])
def test_set_b_float_grids_and_blocks(name, spacing, block):
    rv = image.set_b(spacing, block)
    want = f4()['setb_' + name]
    got = np.asarray(rv.b)
    assert got.shape == want.shape
    assert np.array_equal(got, want)
    assert rv.data_type == 'image'
    assert rv.imSize[0] * rv.imSize[1] == len(rv.b)


@pytest.mark.parametrize('name,req', [('stamp', 'stamp:0.1:-0.2,0.2,-0.3,0.3'),
                                      ('line_angle', '0:1.2:0.1<30'), ('line_csv', '0.1,0.5,0.9,0.999'),
                                      ('line_flat', '0:1:0.25'), ('disc', 'disc')])
def test_set_b_string_requests(name, req):
    z = f4()
    rv = image.set_b(req, [1, 1], Rpol=RPOL, Req=REQ)
    assert rv.data_type == str(z['setb_' + name + '_type'])
    if name == 'disc':
        assert rv.b == ['disc']
        return
    assert np.array_equal(np.asarray(rv.b, dtype=np.float64), z['setb_' + name])


def test_set_b_lists():
    assert image.set_b([0.1, 0.2]).b == [[0.1, 0.2]]
    assert image.set_b([[0.1, 0.2]]).data_type == 'spectrum'
    rv = image.set_b([[0.1 * i, 0.0] for i in range(6)])
    assert rv.data_type == 'profile' and len(rv.b) == 6


def test_image_rows():
    rows = image.image_rows(np.arange(12.0), 4)
    assert rows == [[0.0, 1.0, 2.0, 3.0], [4.0, 5.0, 6.0, 7.0], [8.0, 9.0, 10.0, 11.0]]


def _cases(z):
    hdr = {'b': '# b request:  0.25  [1, 1]', 'freqs': '# freqs request: 22.0 GHz'}
    b = dict(image=[[0.0, 0.0]] * 25, spectrum=[[0.0, 0.0], [0.25, 0.1]],
             profile=[[0.1 * i, 0.0] for i in range(12)], disc=['disc'])
    types = dict(image='image', spectrum='spectrum', profile='profile', disc='spectrum')
    return {k: Namespace(type=types[k], header=hdr, f=z['data_{}_f'.format(k)].tolist(),
                         freqUnit='GHz', b=b[k], Tb=z['data_{}_Tb'.format(k)].tolist())
            for k in b}


@pytest.mark.parametrize('name,xaxis', [('image', 'frequency'), ('spectrum', 'frequency'),
                                        ('spectrum', 'wavelength'), ('profile', 'frequency'),
                                        ('profile', 'wavelength'), ('disc', 'frequency'),
                                        ('disc', 'wavelength')])
def test_fileio_formats_match_reference(tmp_path, name, xaxis):
    z = f4()
    data = _cases(z)[name]
    io = image.FileIO(scratch_spec=str(tmp_path / 'Scratch' / 'specoutputline.dat'))
    path = io.write(str(tmp_path / 'out.dat'), data, xaxis=xaxis)
    with open(path) as fp:
        assert fp.read() == str(z['file_{}_{}'.format(name, xaxis)])


@pytest.mark.gpu
def test_gpu_image_run_matches_oracle():
    """A 0.25-spaced image at one frequency in one device call: rows of 13,
    T_cmb off the planet, on-disc rays equal the oracle's Brightness.single
    within 1 mK."""
    from oracle import oracle as O
    from radiobear_gb300 import _native, catalog
    gas = synth.make_gas_table(120, 1.0e-2, 300.0)
    LP = {k: i for i, k in enumerate(synth.PROPERTY_COLUMNS)}
    prop = synth.compute_properties(gas)
    R, N = prop[LP['R']], prop[LP['N']]
    lines = G.c0_lines()
    e = _native.Engine(0)
    try:
        catalog.upload(e, lines)
        e.set_formalisms('nh3_hs_sjs', True, True, True, True, 'e')
        X = _native.x_matrix(gas, G.C)
        out = image.run(e, gas[G.C['P']], gas[G.C['T']], X, R, N, [22.0], 0.25, REQ, RPOL)
        assert out.type == 'image' and out.imSize == [13, 13]
        assert len(out.Tb) == 13 and all(len(r) == 13 for r in out.Tb)
        tb = np.asarray(out.Tb)
        b = np.asarray(out.b).reshape(13, 13, 2)
        assert tb[0, 0] == 2.725 and tb[12, 12] == 2.725      # corners are off the planet
        picks = [(6, 6), (6, 9), (3, 6), (8, 4)]
        rays = [b[i, j] for i, j in picks]
        tbs, _, _ = O.forward(gas, G.C, R, N, np.array([22.0]), rays, lines, REQ, RPOL)
        for k, (i, j) in enumerate(picks):
            assert abs(tb[i, j] - tbs[k, 0]) < 1e-3, (i, j, tb[i, j], tbs[k, 0])
        with pytest.raises(ValueError, match='only one frequency'):
            image.run(e, gas[G.C['P']], gas[G.C['T']], X, R, N, [22.0, 5.0], 0.25, REQ, RPOL)
    finally:
        e.close()
