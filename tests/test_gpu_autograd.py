"""The forward/adjoint pair behind torch.autograd: gradients by autograd
equal the closed form -2 Re A^H W (v - A x); central finite differences on
random pixels agree; projected gradient descent lowers chi^2."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import casars_cuda as cc
from casars_cuda import autograd as AG

from gpu_common import random_batch

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def setup():
    ctx = cc.Context(0)
    nx, cell = 96, 1.2e-4
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell))
    gw = cc.WProjector(gg, 400.0, planes=8, sampling=4, support_law=(4, 8))
    du = 1.0 / (gg.grid_shape()[0] * cell)
    rng = np.random.default_rng(12)
    u, v, w, wt, vis = random_batch(rng, 8000, gg.grid_shape()[0], du, margin=10, w_max=400.0)
    dev = torch.device("cuda", 0)
    T = lambda a: torch.as_tensor(a, device=dev)
    truth = np.zeros((nx, nx), np.float32)
    truth[40, 50] = 1.0
    truth[60, 30] = 0.5
    b0 = cc.VisibilityBatch(T(u), T(v), T(vis), T(wt), T(w))
    model_vis = cc.predict(gg, b0, T(truth), gw)
    b = cc.VisibilityBatch(T(u), T(v), model_vis, T(wt), T(w))
    yield ctx, gg, gw, b, nx
    ctx.close()


def test_autograd_gradient_matches_closed_form(setup):
    ctx, gg, gw, b, nx = setup
    x = torch.zeros((nx, nx), dtype=torch.float32, device="cuda", requires_grad=True)
    loss = AG.chi2(x, gg, b, gw)
    loss.backward()
    g_closed = AG.chi2_gradient(x.detach(), gg, b, gw)
    err = torch.max(torch.abs(x.grad - g_closed)) / torch.max(torch.abs(g_closed))
    assert float(err) <= 1e-5


def chi2_f64(x, gg, b, gw):
    pred = cc.predict(gg, b, x, gw).to(torch.complex128)
    r = b.visibility.to(torch.complex128) - pred
    return float(torch.sum(b.weight.to(torch.float64) * (r.real ** 2 + r.imag ** 2)))


def test_finite_differences(setup):
    """chi^2 is quadratic in the image, so central differences are exact up
    to rounding; start near the truth so chi^2 itself stays small."""
    ctx, gg, gw, b, nx = setup
    rng = np.random.default_rng(1)
    truth = np.zeros((nx, nx), np.float32)
    truth[40, 50] = 1.0
    truth[60, 30] = 0.5
    x0 = torch.as_tensor(truth + rng.uniform(0, 0.01, (nx, nx)).astype(np.float32), device="cuda")
    g = AG.chi2_gradient(x0, gg, b, gw)
    h = 0.25
    for k in range(64):
        i, j = rng.integers(0, nx, 2)
        xp, xm = x0.clone(), x0.clone()
        xp[i, j] += h
        xm[i, j] -= h
        fd = (chi2_f64(xp, gg, b, gw) - chi2_f64(xm, gg, b, gw)) / (2 * h)
        assert abs(fd - float(g[i, j])) <= 1e-3 * max(1.0, abs(float(g[i, j])))


def test_projected_gradient_descends(setup):
    ctx, gg, gw, b, nx = setup
    x, hist = AG.projected_gradient(torch.zeros((nx, nx), device="cuda"), gg, b, gw, iterations=20)
    assert hist[-1] < 0.2 * hist[0]
    assert float(x.min()) >= 0.0
