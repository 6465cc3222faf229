"""The oracle's multiscale CLEAN against the reference's own tests.

oracle/multiscale.py restates build_multiscale_state, the scale-biased
candidate selection, the windowed subtraction over all scales and
run_multiscale_cotton_schwab (crates/casa-imaging/src/lib.rs:63543-64405).
Pinned here: the scale masks' CASA edges (lib.rs:93979-93997), the
divergence rule (lib.rs:94000-94034), the reported-update count
(lib.rs:90160-90165), the support-bounded kernel update (lib.rs:89588-89601:
equal to the full update at the image edges), the unit volume of the scale
images, and the scale-0 case reducing to a point-component CLEAN.
"""
import json
import os

import numpy as np

from oracle import multiscale as M
from oracle import oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
KATS = {k["name"]: k for k in json.load(open(os.path.join(HERE, "golden", "reference_kats.json")))["kats"]}


def test_scale_mask_edges():
    k = KATS["multiscale_scale_mask_edges"]
    shape = tuple(k["input"]["shape"])
    scales = k["input"]["scales"]
    kernels = [M.make_multiscale_kernel(shape, s) for s in scales]
    masks = M.scale_masks(np.ones(shape, bool), scales, kernels)
    for si, key in ((0, "scale0"), (1, "scale8")):
        for pos, want in k["expected"][key].items():
            x, y = (int(t) for t in pos.strip("()").split(","))
            assert bool(masks[si][x, y]) == want, (key, pos)


def test_divergence_rule_and_reported_updates():
    # casa_multiscale_divergence_stop_reason: after at least one update, a
    # candidate 1.5 times stronger than the cycle's first stops the cycle
    def rule(strength, initial, updates):
        return "DivergenceDetected" if updates > 0 and abs(strength) > abs(initial) * 1.5 else None

    k = KATS["multiscale_divergence_rule"]
    for case, want in zip(k["input"]["cases"], k["expected"]):
        assert rule(case["strength"], case["initial"], case["updates"]) == want
    r = KATS["multiscale_reported_updates"]
    for (a, n), want in zip(r["input"]["cases"], r["expected"]):
        assert min(a, n) == want


def test_scale_images_unit_volume_and_support():
    for shape, s in (((32, 32), 6.0), ((64, 48), 5.0), ((64, 64), 12.0), ((33, 31), 3.5)):
        k = M.make_multiscale_kernel(shape, s)
        assert abs(float(k.sum(dtype=np.float64)) - 1.0) < 1e-5
        x0, y0, x1, y1 = M.kernel_support(k)
        cx, cy = shape[0] // 2, shape[1] // 2
        assert x0 <= cx <= x1 and y0 <= cy <= y1 and x1 - x0 <= 2 * s + 1
    d = M.make_multiscale_kernel((16, 16), 0.0)
    assert d[8, 8] == 1.0 and d.sum() == 1.0


def test_support_bounded_add_equals_full_add_at_edges():
    k = M.make_multiscale_kernel((32, 32), 6.0)
    sup = M.kernel_support(k)
    for pos in ((0, 0), (3, 29), (16, 16), (31, 31)):
        bounded = np.zeros((32, 32), np.float32)
        M.add_shifted_kernel(bounded, k, sup, pos, 0.7)
        full = np.zeros((32, 32), np.float32)
        M.add_shifted_kernel(full, k, (0, 0, 31, 31), pos, 0.7)
        assert np.max(np.abs(full - bounded)) <= np.finfo(np.float32).eps


def test_scale_zero_is_point_clean():
    """With the single scale 0 the state is the residual itself and each
    component is gain * peak / psf peak at the peak pixel."""
    rng = np.random.default_rng(1)
    n = 48
    x = np.arange(n)[:, None] - n // 2
    y = np.arange(n)[None, :] - n // 2
    psf = np.exp(-(x * x + y * y) / 8.0).astype(np.float32)
    res = (0.01 * rng.normal(size=(n, n))).astype(np.float32)
    res[20, 30] += 1.0
    st = M.MultiscaleState(res, psf, [0.0], 0.0)
    np.testing.assert_allclose(st.dirty[0], res, atol=1e-6)
    model = np.zeros_like(res)
    comps, stop = M.minor_cycle(st, model, 0.1, 5)
    assert len(comps) == 5 and comps[0][0] == (20, 30) and comps[0][1] == 0
    assert abs(model[20, 30] - sum(c[3] for c in comps if c[0] == (20, 30))) < 1e-6


def test_multiscale_prefers_the_matching_scale():
    """An extended Gaussian source is taken at a nonzero scale first."""
    n = 64
    x = np.arange(n)[:, None] - n // 2
    y = np.arange(n)[None, :] - n // 2
    psf = np.exp(-(x * x + y * y) / 4.0).astype(np.float32)
    src = M.make_multiscale_kernel((n, n), 6.0) * 50.0
    res = M.fft_convolve_real(psf, src)
    st = M.MultiscaleState(res, psf, [0.0, 3.0, 6.0], 0.0)
    c = st.candidate(M.full_window((n, n)))
    assert c["scale"] == 2 and c["pos"] == (32, 32)
