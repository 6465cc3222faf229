"""The oracle's Clark minor cycle on the reference's own small case
(clark_minor_cycle_refreshes_image_residual_between_subcycles,
casa-imaging lib.rs:94275-94400): a 5 x 5 residual, a 3 x 3 PSF patch with
exterior peak 0.2, gain 0.2, three components; the model changes, the
residual changes, and the first component is 0.2 at the peak (2, 2)."""
import numpy as np

from oracle import clark as OC


def _kat():
    residual = np.array([[0.0, 0.0, 0.0, 0.0, 0.0],
                         [0.0, 0.2, 0.4, 0.1, 0.0],
                         [0.0, 0.3, 1.0, 0.3, 0.0],
                         [0.0, 0.1, 0.4, 0.2, 0.0],
                         [0.0, 0.0, 0.0, 0.0, 0.0]], np.float32)
    psf = np.zeros((5, 5), np.float32)
    psf[2, 2] = 1.0
    psf[1, 2] = psf[3, 2] = psf[2, 1] = psf[2, 3] = 0.1
    patch = dict(patch=np.array([[0.0, 0.1, 0.0], [0.1, 1.0, 0.1], [0.0, 0.1, 0.0]], np.float32),
                 rx=1, ry=1, max_exterior_abs=np.float32(0.2))
    return residual, psf, patch


def test_clark_kat():
    residual, psf, patch = _kat()
    out = OC.clark_minor_cycle(np.zeros_like(residual), residual, psf, patch, 0.2, 3)
    assert out["updated"] and out["actual"] > 0
    assert not np.array_equal(out["residual"], residual)
    (x, y), flux = out["components"][0]
    assert (x, y) == (2, 2) and abs(flux - 0.2) < 1e-7
    assert abs(float(out["model"].sum()) - sum(f for _, f in out["components"])) < 1e-6


def test_patch_from_ncent():
    psf = np.zeros((20, 20), np.float32)
    psf[10, 10] = 1.0
    psf[2, 3] = -0.3
    psf[10, 12] = 0.5
    p = OC.psf_patch(psf, 1)            # 4 x 4 window from (8, 8)
    assert p["patch"].shape == (4, 4) and p["rx"] == 2 and p["ry"] == 2
    assert p["patch"][2, 2] == 1.0 and p["patch"][2, 3] == 0.0
    assert p["max_exterior_abs"] == np.float32(0.5)


def test_convolution_is_the_centred_circular_one():
    rng = np.random.default_rng(1)
    for nx, ny in ((8, 8), (7, 9)):
        psf = rng.normal(size=(nx, ny)).astype(np.float32)
        delta = np.zeros((nx, ny), np.float32)
        delta[2, 3] = 1.5
        conv = OC.fft_convolve_real(psf, delta)
        # literally fft_convolve_real's centred transforms (ifftshift, DFT,
        # fftshift), their product, the centred inverse
        cf = lambda a: np.fft.fftshift(np.fft.fft2(np.fft.ifftshift(a)))
        lit = np.fft.fftshift(np.fft.ifft2(np.fft.ifftshift(cf(psf) * cf(delta)))).real
        np.testing.assert_allclose(conv, lit, atol=1e-5)
        for x in range(nx):
            for y in range(ny):
                want = 1.5 * psf[(x - 2 + nx // 2) % nx, (y - 3 + ny // 2) % ny]
                assert abs(conv[x, y] - want) < 1e-5
