"""Impact-parameter requests, image assembly and the output-file formats.

The host side of the reference's image / profile / spectrum pipeline around
the GPU forward model:

  * ``set_b`` restates ``set_utils.set_b`` (radiobear/set_utils.py:12-88):
    a list of pairs, one pair, ``'disc'``, a float grid spacing with image
    blocks, ``'stamp:bres:xmin,xmax,ymin,ymax'``, and line requests
    ``'start:stop:step[<angle]'`` / ``'n1,n2[<angle]'`` cut at the limb;
  * ``run`` computes every requested ray in one device call
    (``Engine.forward``) and groups image rows as ``Planet.bright_run``
    does (radiobear/planet_base.py:268-274);
  * ``FileIO`` writes the reference's text formats
    (radiobear/fileIO.py:19-102): header lines, then image rows,
    spectrum columns or profile rows.

Two reference defects are not reproduced (the b lists are): for a float
grid ``set_b`` computes ``imSize`` from ``len(b)`` of the float and raises
``TypeError``, and for a stamp from the length of the request string.
Here ``imSize`` is [columns, rows of this block] in both cases.
"""
from __future__ import annotations

import os
from argparse import Namespace

import numpy as np

SPEED_OF_LIGHT = 2.9979E8            # m/s, radiobear/utils.py:74
UNITS = {'Hz': 1.0, 'kHz': 1.0E3, 'MHz': 1.0E6, 'GHz': 1.0E9}   # utils.py:13


def proc_string(srq):
    """set_utils.proc_string (set_utils.py:131-146): csv list, start:stop:step
    (stop inclusive), start;stop;nstep (log), a number or a file of values."""
    if ',' in srq:
        return [float(x) for x in srq.split(',')]
    if ':' in srq:
        start, stop, step = [float(x) for x in srq.split(':')]
        return list(np.arange(start, stop + step / 2.0, step))
    if ';' in srq:
        start, stop, step = [float(x) for x in srq.split(';')]
        return list(np.logspace(np.log10(start), np.log10(stop), int(step)))
    try:
        return [float(srq)]
    except ValueError:
        return list(np.loadtxt(srq))


def image_grid(spacing):
    """The float-request grid: -1.5 .. 1.5 in steps of ``spacing`` about 0
    (set_utils.py:65-66)."""
    grid = -1.0 * np.flipud(np.arange(spacing, 1.5 + spacing, spacing))
    return np.concatenate((grid, np.arange(0.0, 1.5 + spacing, spacing)))


def set_b(b, block=(1, 1), **kwargs):
    """Process an impact-parameter request -> Namespace(b, data_type, block,
    imSize).  ``Rpol`` and ``Req`` (kwargs) are needed for line requests."""
    block = list(block)
    rv = Namespace(b=None, data_type=None, block=block, imSize=None)
    if isinstance(b, str):
        b = b.lower()
        if b.startswith('dis'):
            rv.b = [b]
            rv.data_type = 'spectrum'
        elif b.startswith('stamp'):
            bres = float(b.split(':')[1])
            bext = [float(x) for x in b.split(':')[2].split(',')]
            rv.b = []
            xs = np.arange(bext[0], bext[1] + bres / 2.0, bres)
            ys = np.arange(bext[2], bext[3] + bres / 2.0, bres)
            for x in xs:
                for y in ys:
                    rv.b.append([y, x])
            rv.imSize = [len(ys), len(xs)]
            rv.data_type = 'image'
        else:
            parts = b.split('<')
            angle_b = 0.0 if len(parts) == 1 else float(parts[1]) * np.pi / 180.0
            mag_b = proc_string(parts[0])
            ab = kwargs['Rpol'] / kwargs['Req']
            rab = ab / np.sqrt(np.power(np.sin(angle_b), 2.0) + np.power(ab * np.cos(angle_b), 2.0))
            rv.b = [[v * np.cos(angle_b), v * np.sin(angle_b)] for v in mag_b if v < 0.995 * rab]
            rv.data_type = 'profile'
        return rv
    if isinstance(b, float):
        grid = image_grid(b)
        bsplit = len(grid) / abs(block[1])
        last_row = block[0] / abs(block[1])
        if abs(block[1]) == 1:
            last_row = 0
        rv.b = []
        nrow = int(bsplit + last_row)
        for i in range(nrow):
            vrow = grid[i + int((block[0] - 1) * bsplit)]
            for vcol in grid:
                rv.b.append([vcol, vrow])
        rv.imSize = [len(grid), nrow]
        rv.data_type = 'image'
        return rv
    shape_b = np.shape(b)
    if len(shape_b) == 1:
        rv.data_type = 'spectrum'
        rv.b = [b]
    else:
        rv.data_type = 'spectrum' if shape_b[0] < 5 else 'profile'
        rv.b = b
    return rv


def b_type(b):
    """utils.b_type (radiobear/utils.py:139-149)."""
    if isinstance(b, str):
        return b.lower()
    if isinstance(b[0], str):
        return b[0].lower()
    if len(b) > 20:
        return 'image'
    if len(b) > 9:
        return 'profile'
    return 'spectrum'


def image_rows(tb_first_freq, row_len):
    """Group per-ray Tb values into image rows of ``row_len`` (one row
    completes every row_len rays, planet_base.py:268-274)."""
    rows, row = [], []
    for i, v in enumerate(tb_first_freq):
        row.append(float(v))
        if not (i + 1) % row_len:
            rows.append(row)
            row = []
    return rows


def run(engine, P, T, X, R, N, freqs, b, Req, Rpol, block=(1, 1), orientation=(0.0, 0.0),
        gtype='ellipse', limb='shape', freqUnit='GHz'):
    """The b loop of Planet.run (planet.py:117-139) as one device call.

    Returns a Namespace like the reference's data_return: f, freqUnit, b,
    Tb (image rows for an image, else [nb][nf]), type, header, imSize.
    An image takes one frequency (planet_base.py:201-202)."""
    freqs = np.atleast_1d(np.asarray(freqs, dtype=np.float64))
    rv = set_b(b, block, Rpol=Rpol, Req=Req)
    if rv.data_type == 'image' and freqs.size > 1:
        raise ValueError('Warning:  Image must be at only one frequency')
    header = {'b': '# b request:  {}  {}'.format(str(b), str(list(block)))}
    if b_type(rv.b) == 'disc':
        rays = np.zeros((1, 2))
        out = engine.forward(P, T, X, R, N, freqs, rays, Req, Rpol, orientation=orientation,
                             gtype=gtype, limb=limb, disc=True)
    else:
        rays = np.asarray(rv.b, dtype=np.float64).reshape(-1, 2)
        out = engine.forward(P, T, X, R, N, freqs, rays, Req, Rpol, orientation=orientation,
                             gtype=gtype, limb=limb)
    tb = np.asarray(out['Tb'])
    if rv.data_type == 'image':
        Tb = image_rows(tb[:, 0], rv.imSize[0])
    else:
        Tb = [list(map(float, row)) for row in tb]
    return Namespace(f=list(freqs), freqUnit=freqUnit, b=rv.b, Tb=Tb, type=rv.data_type,
                     header=header, imSize=rv.imSize, block=rv.block)


class FileIO:
    """Output writer with the reference's formats (fileIO.py:10-102)."""

    def __init__(self, directory='Output', scratch_spec='Scratch/specoutputline.dat'):
        self.directory = directory
        self.scratch_spec = scratch_spec

    def write(self, output_file, data, xaxis='frequency'):
        self.data = data
        xaxis = xaxis.lower()
        with open(output_file, 'w') as fp:
            self.writeHeader(data.header, fp)
            t = data.type.lower()
            if t == 'image':
                self.writeImage(fp)
            elif t == 'spectrum':
                self.writeSpectrum(fp, xaxis=xaxis)
            elif t == 'profile':
                self.writeProfile(fp, xaxis=xaxis)
            else:
                print("Invalid output type: {}".format(data.type))
        return output_file

    def writeHeader(self, header, fp):
        for hdr in sorted(header.keys()):
            fp.write(header[hdr] + '\n')

    def writeImage(self, fp):
        for row in self.data.Tb:
            s = ''
            for d in row:
                s += '{:7.2f}\t'.format(d)
            fp.write(s.strip() + '\n')

    def _wl_cm(self, f):
        return 100.0 * SPEED_OF_LIGHT / (f * UNITS[self.data.freqUnit])

    def writeSpectrum(self, fp, xaxis):
        d = os.path.dirname(self.scratch_spec)
        if d:
            os.makedirs(d, exist_ok=True)
        with open(self.scratch_spec, 'w') as fp_line:
            s = '# cm   K@b  \t' if xaxis.startswith('wave') else '# {}  K@b  \t'.format(self.data.freqUnit)
            if b_type(self.data.b) == 'disc':
                s += 'disc'
            else:
                for bv in self.data.b:
                    s += '({:5.3f},{:5.3f})\t'.format(bv[0], bv[1])
            fp.write(s.strip('\t') + '\n')
            for i, f in enumerate(self.data.f):
                s = '{:.4f}\t  '.format(self._wl_cm(f)) if xaxis.startswith('wave') else '{:.2f}\t  '.format(f)
                for j in range(len(self.data.b)):
                    s += '  {:9.4f}  \t'.format(self.data.Tb[j][i])
                s = s.strip() + '\n'
                fp_line.write(s)
                fp.write(s)

    def writeProfile(self, fp, xaxis):
        s = '# b  K@cm  \t' if xaxis.startswith('wave') else '# b  K@{} \t'.format(self.data.freqUnit)
        for f in self.data.f:
            if xaxis.startswith('wave'):
                s += '  {:.4f}   \t'.format(self._wl_cm(f))
            else:
                s += '  {:9.4f}   \t'.format(f)
        fp.write(s.strip() + '\n')
        for i, bv in enumerate(self.data.b):
            s = 'disc' if b_type(self.data.b) == 'disc' else '{:5.3f} {:5.3f}\t'.format(bv[0], bv[1])
            for j in range(len(self.data.f)):
                s += ' {:7.2f}\t '.format(self.data.Tb[i][j])
            fp.write(s.strip() + '\n')
