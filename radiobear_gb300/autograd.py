"""Differentiable forward model: ``torch.autograd.Function`` over the C ABI.

``TbModel`` holds the fixed parts of a retrieval (catalogues on an
``Engine``, layer radii and refractive indices, rays, quadrature weights,
frequencies, the abundances that are not retrieved) and maps per-layer

    T [nL] (K), P [nL] (bar), lnX [3, nL] (ln mole fraction of NH3, H2O, H2S)

float64 CUDA tensors to the disc-averaged brightness Tb_avg [nf] (K).  The
backward pass calls ``rb_adjoint_device`` (reverse sweep of the brightness
scan, alpha recomputed with its per-layer derivatives); the ray paths are
held fixed.  ``disc=True`` is the reference's ``b = 'disc'``: every ray is
the nadir ray with the 2 E2(tau) weighting (brightness.py:32-34, 96).  The reference has no derivatives: this is an addition beside
the drop-in path (see ``include/radiobear_gb300.h``).
"""
from __future__ import annotations

import numpy as np
import torch

from . import _native

# rows of the X input (_native.X_ROWS) taken from lnX
_LNX_ROWS = (_native.X_ROWS.index('NH3'), _native.X_ROWS.index('H2O'), _native.X_ROWS.index('H2S'))


class TbModel:
    def __init__(self, engine, R, N, freqs, b, weights, X_fixed, Req, Rpol, device=None,
                 orientation=(0.0, 0.0), gtype='ellipse', limb='shape', disc=False):
        self.engine = engine
        self.disc = bool(disc)
        if self.disc:
            b = np.zeros_like(np.atleast_2d(np.asarray(b, dtype=np.float64)))
        self.device = torch.device(device or 'cuda')
        f64 = dict(dtype=torch.float64, device=self.device)
        self.R = torch.as_tensor(np.ascontiguousarray(R, dtype=np.float64), **f64)
        self.N = torch.as_tensor(np.ascontiguousarray(N, dtype=np.float64), **f64)
        self.b = torch.as_tensor(np.ascontiguousarray(np.atleast_2d(b), dtype=np.float64), **f64)
        self.w = torch.as_tensor(np.ascontiguousarray(weights, dtype=np.float64), **f64)
        self.X = torch.as_tensor(np.ascontiguousarray(X_fixed, dtype=np.float64), **f64)
        self.freqs = np.ascontiguousarray(freqs, dtype=np.float64)
        self.Req, self.Rpol = float(Req), float(Rpol)
        self.orientation, self.gtype, self.limb = orientation, gtype, limb
        self.nL = self.R.numel()
        self.nb = self.b.shape[0]

    def x_matrix(self, lnX):
        X = self.X.clone()
        for k, row in enumerate(_LNX_ROWS):
            X[row] = torch.exp(lnX[k])
        return X.contiguous()

    def __call__(self, T, P, lnX):
        return TbFunction.apply(T, P, lnX, self)


class TbFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, T, P, lnX, model):
        for name, t, shape in (('T', T, (model.nL,)), ('P', P, (model.nL,)), ('lnX', lnX, (3, model.nL))):
            if t.dtype != torch.float64 or t.device.type != 'cuda' or tuple(t.shape) != shape:
                raise ValueError('{} must be a float64 CUDA tensor of shape {}'.format(name, shape))
        T, P, lnX = T.contiguous(), P.contiguous(), lnX.contiguous()
        X = model.x_matrix(lnX)
        nf = model.freqs.size
        Tb = torch.empty((model.nb, nf), dtype=torch.float64, device=T.device)
        avg = torch.empty(nf, dtype=torch.float64, device=T.device)
        stream = torch.cuda.current_stream(T.device).cuda_stream
        model.engine.forward_device(stream, model.nL, model.nb, P.data_ptr(), T.data_ptr(), X.data_ptr(),
                                    model.R.data_ptr(), model.N.data_ptr(), model.freqs,
                                    model.b.data_ptr(), model.Req, model.Rpol, Tb.data_ptr(),
                                    weights=model.w.data_ptr(), Tb_avg=avg.data_ptr(),
                                    orientation=model.orientation, gtype=model.gtype,
                                    limb=model.limb, disc=model.disc)
        ctx.model = model
        ctx.save_for_backward(T, P, X)
        return avg

    @staticmethod
    def backward(ctx, g):
        T, P, X = ctx.saved_tensors
        model = ctx.model
        g = g.to(torch.float64).contiguous()
        dT = torch.empty_like(T)
        dP = torch.empty_like(P)
        dlnX = torch.empty((3, model.nL), dtype=torch.float64, device=T.device)
        stream = torch.cuda.current_stream(T.device).cuda_stream
        model.engine.adjoint_device(stream, model.nL, model.nb, P.data_ptr(), T.data_ptr(),
                                    X.data_ptr(), model.R.data_ptr(), model.N.data_ptr(),
                                    model.freqs, model.b.data_ptr(), model.Req, model.Rpol,
                                    g.data_ptr(), dT.data_ptr(), dP.data_ptr(), dlnX.data_ptr(),
                                    weights=model.w.data_ptr(), orientation=model.orientation,
                                    gtype=model.gtype, limb=model.limb, disc=model.disc)
        return dT, dP, dlnX, None
