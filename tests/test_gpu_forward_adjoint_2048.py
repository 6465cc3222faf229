"""The forward/adjoint pair at the differentiable-imaging size.

2048 x 2048 image of 50 Gaussian components (0.01-1 Jy, FWHM 1-5 px),
2,021,760 visibilities on 27-antenna tracks to 5 km, W-projection with 32
planes and the reference's support search (sampling 4).  The model
visibilities are A(model) with 0.01 Jy noise.

* dot-product test <A x, y> = <x, A^H y> to 1e-6 of ||A x|| ||y||;
* autograd's gradient equals -2 Re A^H W (v - A x), and central finite
  differences of chi^2 (FP64 sums) on 64 random pixels agree with it;
* the residual image of a model equals the oracle's FP64 residual image
  (compute_residual, lib.rs:70592-70644) within 1e-5 of its peak;
* 50 projected-gradient iterations under non-negativity lower chi^2.
"""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

import casars_cuda as cc
from casars_cuda import autograd as AG
from casars_cuda import synthetic as S
from oracle import oracle as O

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu
PLANES = 32


@pytest.fixture(scope="module")
def cfg():
    ctx = cc.Context(0)
    obs = S.pair_2048_observation(3)
    nx = obs.nx
    dev = torch.device("cuda", 0)
    model = S.gaussian_model(np.random.default_rng(33), 50, nx, nx, 0.01, 1.0)
    wmax = float(np.abs(obs.w).max())
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, obs.cell, obs.cell))
    gw = cc.WProjector(gg, wmax, planes=PLANES)
    T = lambda a: torch.as_tensor(a, device=dev)
    u, v, w = T(obs.u), T(obs.v), T(obs.w)
    wt = torch.ones(obs.rows, dtype=torch.float32, device=dev)
    uvw = cc.VisibilityBatch(u, v, torch.zeros(obs.rows, dtype=torch.complex64, device=dev), wt, w)
    vis = cc.predict(gg, uvw, T(model), gw)
    g = torch.Generator(device=dev)
    g.manual_seed(5)
    vis = vis + 0.01 * torch.complex(torch.randn(obs.rows, generator=g, device=dev),
                                     torch.randn(obs.rows, generator=g, device=dev))
    b = cc.VisibilityBatch(u, v, vis, wt, w)
    yield ctx, obs, gg, gw, b, model, wmax
    ctx.close()


def test_dot_product_full_size(cfg):
    ctx, obs, gg, gw, b, model, _ = cfg
    gen = torch.Generator(device="cuda")
    gen.manual_seed(7)
    x = torch.randn((obs.nx, obs.nx), generator=gen, device="cuda")
    y = torch.complex(torch.randn(obs.rows, generator=gen, device="cuda"),
                      torch.randn(obs.rows, generator=gen, device="cuda"))
    ax = cc.predict(gg, b, x, gw).to(torch.complex128)
    aty = cc.adjoint(gg, cc.VisibilityBatch(b.u_lambda, b.v_lambda, y, b.weight, b.w_lambda), gw)
    lhs = float(torch.sum(torch.conj(ax) * y.to(torch.complex128)).real)
    rhs = float(torch.sum(x.to(torch.float64) * aty.to(torch.float64)))
    bound = float(torch.linalg.vector_norm(ax) * torch.linalg.vector_norm(y.to(torch.complex128)))
    assert abs(lhs - rhs) <= 1e-6 * bound


def _chi2_f64(x, gg, b, gw):
    pred = cc.predict(gg, b, x, gw).to(torch.complex128)
    r = b.visibility.to(torch.complex128) - pred
    return float(torch.sum(b.weight.to(torch.float64) * (r.real ** 2 + r.imag ** 2)))


def test_gradient_and_finite_differences(cfg):
    ctx, obs, gg, gw, b, model, _ = cfg
    rng = np.random.default_rng(4)
    x0 = torch.as_tensor(model + rng.uniform(0, 1e-3, model.shape).astype(np.float32),
                         device="cuda")
    xg = x0.clone().requires_grad_(True)
    AG.chi2(xg, gg, b, gw).backward()
    g = AG.chi2_gradient(x0, gg, b, gw)
    assert float(torch.max(torch.abs(xg.grad - g)) / torch.max(torch.abs(g))) <= 1e-5
    h = 0.25
    pix = [tuple(rng.integers(obs.nx // 4, 3 * obs.nx // 4, 2)) for _ in range(64)]
    gv = np.array([float(g[i, j]) for i, j in pix])
    scale = float(np.max(np.abs(gv)))
    for (i, j), gij in zip(pix, gv):
        xp, xm = x0.clone(), x0.clone()
        xp[i, j] += h
        xm[i, j] -= h
        fd = (_chi2_f64(xp, gg, b, gw) - _chi2_f64(xm, gg, b, gw)) / (2 * h)
        assert abs(fd - gij) <= 1e-3 * scale


def test_residual_image_matches_oracle(cfg):
    ctx, obs, gg, gw, b, model, wmax = cfg
    nx = obs.nx
    geom = O.Geometry(nx, nx, obs.cell, obs.cell)
    og = O.StdGridder(geom)
    ow = O.WProjector(geom, og, wmax, planes=PLANES, threads=16)
    vis = b.visibility.cpu().numpy()
    wt = np.ones(obs.rows, np.float32)
    p, d, acc = ow.grid_dirty(obs.u, obs.v, obs.w, wt, vis, threads=16)
    psf_o, res_o, peak_o = ow.dirty_products(p, d, acc)
    half = (0.5 * model).astype(np.float32)
    rg, _ = ow.residual(ow.model_grid(half.astype(np.float64)), obs.u, obs.v, obs.w, wt, vis,
                        threads=16)
    ref = 2.0 * ow.corrected_image(O.centered_ifft2(rg)) / acc.normalization_sumwt / peak_o
    hb = cc.VisibilityBatch(obs.u, obs.v, vis, wt, obs.w)
    psf, res, state, sums = cc.dirty_image(gg, hb, gw)
    assert peak_norm_err(res, res_o) <= 1e-5
    got, _ = cc.residual_image(gg, hb, half, state, gw)
    assert peak_norm_err(got, ref) <= 1e-5


def test_projected_gradient_50_iterations(cfg):
    ctx, obs, gg, gw, b, model, _ = cfg
    x, hist = AG.projected_gradient(torch.zeros((obs.nx, obs.nx), device="cuda"), gg, b, gw,
                                    iterations=50)
    assert float(x.min()) >= 0.0
    assert hist[-1] < 0.5 * hist[0]
    assert np.all(np.diff(hist) <= 1e-6 * hist[0])
