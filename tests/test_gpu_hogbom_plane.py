"""run_hogbom_plane_minor_cycle on the GPU against the oracle, bit for bit:
component positions, peaks and fluxes, the updated model and residual
(float32 arithmetic in the same order).  Tolerance 0 runs the persistent
loop with the plane rules; a positive tolerance the single-block replay of
the order-dependent scan."""
import numpy as np
import pytest

import casars_cuda as cc
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


@pytest.mark.parametrize("tol", [0.0, 1e-3])
def test_known_answer(ctx, tol):
    residual = np.zeros((3, 3), np.float32)
    residual[1, 1] = 4.0
    residual[2, 2] = np.nan
    psf = np.zeros((3, 3), np.float32)
    psf[1, 1] = 1.0
    mask = np.ones((3, 3), np.uint8)
    clean = cc.CleanConfig(niter=1, gain=0.5)
    out = cc.run_hogbom_plane_minor_cycle(
        ctx, np.zeros((3, 3), np.float32), residual, psf, mask,
        cc.HogbomPlaneMinorCycleControl(clean, 1, 0.1, tol))
    assert out.actual_updates == 2 and out.reported_updates == 1
    c0 = out.components[0]
    assert c0.position == (1, 1) and c0.peak_value_jy_per_beam == 4.0 and c0.component_jy == 2.0
    assert out.model[1, 1] == 3.0 and out.residual[1, 1] == 1.0


def _image(rng, nx, ny, tol):
    x = np.arange(nx)[:, None] - nx / 2
    y = np.arange(ny)[None, :] - ny / 2
    psf = np.exp(-(x ** 2 + y ** 2) / 18.0).astype(np.float32)
    res = (0.05 * rng.normal(size=(nx, ny))).astype(np.float32)
    for _ in range(12):
        res[rng.integers(nx), rng.integers(ny)] += rng.uniform(-1, 1)
    # near-ties: copies of the peak within and just past the tolerance
    top = float(np.abs(res).max())
    for f in (1 + 0.4 * tol, 1 - 0.3 * tol, 1 + 1.5 * tol):
        res[rng.integers(nx), rng.integers(ny)] = np.float32(top * f)
    res[rng.integers(nx), rng.integers(ny)] = np.inf
    mask = (rng.uniform(size=(nx, ny)) > 0.1).astype(np.uint8)
    return res, psf, mask


@pytest.mark.parametrize("tol,nx,ny", [(0.0, 64, 48), (1e-3, 64, 48), (2e-2, 37, 80),
                                       (1e-3, 160, 128)])
def test_matches_oracle(ctx, tol, nx, ny):
    rng = np.random.default_rng(int(tol * 1e4) + nx)
    res, psf, mask = _image(rng, nx, ny, tol)
    model = np.zeros((nx, ny), np.float32)
    clean = cc.CleanConfig(niter=200, gain=0.1, threshold_jy_per_beam=0.02)
    out = cc.run_hogbom_plane_minor_cycle(ctx, model, res, psf, mask,
                                          cc.HogbomPlaneMinorCycleControl(clean, 150, 0.05, tol))
    ref = O.hogbom_plane(res, psf, 0.1, 150, 0.05, tol, threshold=0.02, mask=mask)
    assert out.actual_updates == ref["actual"] > 10
    assert out.reported_updates == ref["reported"]
    pos = np.array([c.position for c in out.components])
    np.testing.assert_array_equal(pos[:, 0], ref["x"])
    np.testing.assert_array_equal(pos[:, 1], ref["y"])
    np.testing.assert_array_equal([c.peak_value_jy_per_beam for c in out.components],
                                  ref["peak"])
    np.testing.assert_array_equal([c.component_jy for c in out.components], ref["flux"])
    np.testing.assert_array_equal(out.model, ref["model"])
    np.testing.assert_array_equal(out.residual, ref["residual"])


def test_device_arrays(ctx):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(77)
    res, psf, mask = _image(rng, 96, 96, 1e-3)
    dev = torch.device("cuda", 0)
    clean = cc.CleanConfig(niter=50, gain=0.2)
    out = cc.run_hogbom_plane_minor_cycle(
        ctx, torch.zeros(96, 96, device=dev), torch.as_tensor(res).to(dev),
        torch.as_tensor(psf).to(dev), torch.as_tensor(mask).to(dev),
        cc.HogbomPlaneMinorCycleControl(clean, 40, 0.0, 1e-3))
    ref = O.hogbom_plane(res, psf, 0.2, 40, 0.0, 1e-3, mask=mask)
    assert out.actual_updates == ref["actual"] == 41
    np.testing.assert_array_equal(out.residual.cpu().numpy(), ref["residual"])
    with pytest.raises(cc.CasarsCudaError):
        cc.run_hogbom_plane_minor_cycle(ctx, np.zeros((4, 4), np.float32),
                                        np.ones((4, 4), np.float32), np.ones((4, 4), np.float32),
                                        None, cc.HogbomPlaneMinorCycleControl(clean, 1, 0.0,
                                                                              -1.0))
