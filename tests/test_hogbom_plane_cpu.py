"""The oracle's run_hogbom_plane_minor_cycle and its tolerance peak search,
pinned to the reference's known answer (casa-imaging lib.rs:78093-78130)
and to a direct restatement of the scan."""
import numpy as np

from oracle import oracle as O


def test_plane_minor_cycle_known_answer():
    # hogbom_plane_minor_cycle_updates_model_and_records_components
    residual = np.zeros((3, 3), np.float32)
    residual[1, 1] = 4.0
    residual[2, 2] = np.nan
    psf = np.zeros((3, 3), np.float32)
    psf[1, 1] = 1.0
    mask = np.ones((3, 3), np.uint8)
    out = O.hogbom_plane(residual, psf, gain=0.5, cycle_limit=1, cycle_threshold=0.1,
                         tol=1e-3, threshold=0.0, mask=mask, inclusive=True)
    assert out["actual"] == 2 and out["reported"] == 1
    assert (out["x"][0], out["y"][0]) == (1, 1)
    assert out["peak"][0] == 4.0 and out["flux"][0] == 2.0
    assert out["model"][1, 1] == 3.0 and out["residual"][1, 1] == 1.0


def _scan(image, tol, mask=None):
    k1 = np.float32(1.0) + np.float32(tol)
    best = None
    nx, ny = image.shape
    for y in range(ny):
        for x in range(nx):
            if mask is not None and not mask[x, y]:
                continue
            v = np.float32(image[x, y])
            if not np.isfinite(v):
                continue
            if best is None or abs(v) > np.float32(abs(best[1]) * k1):
                best = ((x, y), float(v))
    return best


def test_relative_peak_keeps_the_earlier_near_tie():
    img = np.zeros((4, 3), np.float32)
    img[3, 0] = 1.0              # scanned first (y = 0)
    img[0, 1] = 1.0005           # larger, but within 1e-3 of it
    img[2, 2] = -1.0011          # beyond the tolerance: replaces it
    assert O.peak_relative(img, 1e-3) == ((2, 2), float(np.float32(-1.0011)))
    img[2, 2] = 1.0009
    assert O.peak_relative(img, 1e-3) == ((3, 0), 1.0)
    assert O.peak_relative(img, 0.0) == ((2, 2), float(np.float32(1.0009)))
    assert O.peak_relative(img, 4e-4) == ((0, 1), float(np.float32(1.0005)))
    img[:, :] = np.nan
    assert O.peak_relative(img, 1e-3) is None


def test_relative_peak_matches_the_scan():
    rng = np.random.default_rng(5)
    for trial in range(20):
        nx, ny = rng.integers(3, 40, 2)
        img = rng.normal(size=(nx, ny)).astype(np.float32)
        # near-ties around the largest value, and some non-finite values
        top = np.abs(img).max()
        for _ in range(6):
            img[rng.integers(nx), rng.integers(ny)] = top * (1 + rng.uniform(-2e-3, 2e-3))
        img[rng.integers(nx), rng.integers(ny)] = np.inf
        mask = (rng.uniform(size=(nx, ny)) > 0.2).astype(np.uint8)
        for tol in (0.0, 1e-3, 5e-2):
            assert O.peak_relative(img, tol, mask) == _scan(img, tol, mask)
