"""The forward/adjoint imaging pair as a torch.autograd.Function.

A x = D F C x: apodise the (real) model image, centred unscaled forward FFT,
degrid with the gridder's taps (standard) or W-kernels (W-projection); this
is the reference's model-visibility prediction (apodize_model, gridder.rs:
1554-1592; centered_fft2, fft.rs:34; degrid_sample_taps_planned_normalized,
gridder.rs:1278-1312; degrid_sample_planned, gridder.rs:3726-3747).
A^H y = C F^H G y is its exact adjoint (the gridder is the degridder's
conjugate transpose, F^H the unscaled inverse FFT), evaluated by cr_adjoint.

For chi^2 = sum_i w_i |v_i - (A x)_i|^2 the gradient is
-2 Re A^H W (v - A x), which `chi2_gradient` returns; backward() of the
Function maps an upstream gradient g on the model visibilities to
Re A^H g (real image, as A acts on real images).
"""
from __future__ import annotations

import numpy as np
import torch

from . import imaging as im


class ForwardOperator(torch.autograd.Function):
    """vis = A(model) for a fixed VisibilityBatch geometry (u, v, w)."""

    @staticmethod
    def forward(ctx, model, gridder, batch_uvw, wproj=None):
        ctx.gridder, ctx.batch, ctx.wproj = gridder, batch_uvw, wproj
        return im.predict(gridder, batch_uvw, model.detach().to(torch.float32).contiguous(), wproj)

    @staticmethod
    def backward(ctx, grad_vis):
        g = grad_vis.detach().to(torch.complex64).contiguous()
        b = ctx.batch
        ones = torch.ones(len(b), dtype=torch.float32, device=g.device)
        adj = im.adjoint(ctx.gridder, im.VisibilityBatch(b.u_lambda, b.v_lambda, g, ones,
                                                         b.w_lambda), ctx.wproj)
        return adj, None, None, None


def forward(model, gridder, batch, wproj=None):
    return ForwardOperator.apply(model, gridder, batch, wproj)


def chi2(model, gridder, batch, wproj=None):
    """sum_i w_i |v_i - (A x)_i|^2 with autograd support through A."""
    pred = forward(model, gridder, batch, wproj)
    r = batch.visibility - pred
    w = batch.weight if batch.weight is not None else torch.ones_like(r.real)
    return torch.sum(w * (r.real * r.real + r.imag * r.imag))


def chi2_gradient(model, gridder, batch, wproj=None):
    """-2 Re A^H W (v - A x), with the weighted residual visibilities gridded
    once by cr_adjoint."""
    pred = im.predict(gridder, batch, model, wproj)
    res = (batch.visibility - pred).to(torch.complex64)
    w = batch.weight if batch.weight is not None else torch.ones(len(batch), device=res.device)
    adj = im.adjoint(gridder, im.VisibilityBatch(batch.u_lambda, batch.v_lambda, res, w,
                                                 batch.w_lambda), wproj)
    return -2.0 * adj


def projected_gradient(model0, gridder, batch, wproj=None, iterations=50, step=None):
    """Non-negative least squares by projected gradient descent on chi^2.

    The step is 1/L with L estimated by a few power iterations of 2 A^H W A.
    Returns the model and the chi^2 after each iteration.
    """
    x = model0.clone()
    if step is None:
        y = torch.randn_like(x)
        for _ in range(8):
            y = y / torch.linalg.vector_norm(y)
            ay = im.predict(gridder, batch, y, wproj)
            w = batch.weight if batch.weight is not None else torch.ones(len(batch), device=y.device)
            y = 2.0 * im.adjoint(gridder, im.VisibilityBatch(batch.u_lambda, batch.v_lambda,
                                                             ay.to(torch.complex64), w,
                                                             batch.w_lambda), wproj)
        step = 1.0 / float(torch.linalg.vector_norm(y))
    history = []
    for _ in range(iterations):
        g = chi2_gradient(x, gridder, batch, wproj)
        x = torch.clamp(x - step * g, min=0.0)
        pred = im.predict(gridder, batch, x, wproj)
        r = batch.visibility - pred
        w = batch.weight if batch.weight is not None else torch.ones_like(r.real)
        history.append(float(torch.sum(w * (r.real ** 2 + r.imag ** 2))))
    return x, np.array(history)
