"""Robust RMS (the n-sigma threshold) on the device against the oracle.

cr_robust_rms restates robust_rms_jy_per_beam (lib.rs:74130-74183): finite
values (outside the clean mask when the mask is not all true), Chauvenet
clipping for the unmasked case, then f32(MADFM) * 1.4826.  On the same
images the device gives the oracle's MADFM, value count and RMS bit for bit:
the medians are exact selections, and the clipping windows (FP64 sums in
another order) keep the same values on these inputs.  Edge cases: no finite
value, one value, two values, a constant image, ties at the median, signed
zeros, all-true masks, and planes of a stack evaluated together.  The
Cotton-Schwab loop with nsigma > 0 stops where the oracle's loop stops.
"""
import json
import os

import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import oracle as O

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
KATS = {k["name"]: k for k in json.load(open(os.path.join(HERE, "golden", "reference_kats.json")))["kats"]}


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def _same(got, want):
    assert got[2] == want[2], (got, want)          # values counted
    assert got[1] == want[1], (got, want)          # MADFM, FP64
    assert got[0] == want[0], (got, want)          # RMS, float32


def _noise(seed, shape, outliers=True):
    rng = np.random.default_rng(seed)
    img = rng.normal(0.0, 0.01, shape).astype(np.float32)
    if outliers:
        for _ in range(30):
            img[rng.integers(0, shape[0]), rng.integers(0, shape[1])] = rng.uniform(-2, 5)
        img[3, 4] = np.nan
        img[5, 9] = np.inf
    return img


@pytest.mark.parametrize("shape", [(64, 48), (257, 130), (1024, 1024), (2048, 2048)])
def test_unmasked_images_bit_exact(ctx, shape):
    img = _noise(1, shape)
    _same(cc.robust_rms(ctx, img), O.robust_rms(img))


def test_masked_images_bit_exact(ctx):
    img = _noise(2, (300, 200))
    rng = np.random.default_rng(3)
    mask = (rng.uniform(size=img.shape) < 0.3).astype(np.uint8)   # 1 = clean region
    _same(cc.robust_rms(ctx, img, mask), O.robust_rms(img, mask))
    # a mask that is all true does not restrict the values
    ones = np.ones(img.shape, np.uint8)
    _same(cc.robust_rms(ctx, img, ones), O.robust_rms(img))


def test_device_inputs_and_plane_stacks(ctx):
    import torch
    imgs = np.stack([_noise(s, (128, 96)) for s in range(5)])
    masks = np.zeros(imgs.shape, np.uint8)
    masks[1, 10:40, 20:50] = 1
    masks[3] = 1
    masks[4, ::3] = 1
    planes = [4, 0, 3, 1]
    rms, mad, cnt = cc.robust_rms(ctx, torch.as_tensor(imgs).cuda(),
                                  torch.as_tensor(masks).cuda(), planes)
    for k, p in enumerate(planes):
        _same((float(rms[k]), float(mad[k]), int(cnt[k])), O.robust_rms(imgs[p], masks[p]))
    rms2, mad2, cnt2 = cc.robust_rms(ctx, imgs, None, planes)
    for k, p in enumerate(planes):
        _same((float(rms2[k]), float(mad2[k]), int(cnt2[k])), O.robust_rms(imgs[p]))


def test_edge_cases(ctx):
    cases = {
        "no finite value": np.full((8, 8), np.nan, np.float32),
        "one value": np.array([[np.nan, 3.5], [np.inf, -np.inf]], np.float32),
        "two values": np.array([[1.0, 4.0]], np.float32),
        "constant": np.full((16, 16), 0.25, np.float32),
        "ties at the median": np.array([[1, 2, 2, 2, 2, 3, 9, -4]], np.float32),
        "signed zeros": np.array([[0.0, -0.0, -0.0, 0.0, 1.0, -1.0]], np.float32),
        "even count, gap above": np.array([[5, 1, 2, 100, 7, 3]], np.float32),
    }
    for name, img in cases.items():
        got, want = cc.robust_rms(ctx, img), O.robust_rms(img)
        assert got == want, name
    assert cc.robust_rms(ctx, cases["no finite value"])[2] == 0
    # every masked pixel inside the clean region: no value remains
    img = _noise(4, (16, 16), outliers=False)
    m = np.ones(img.shape, np.uint8)
    m[0, 0] = 0
    img[0, 0] = np.nan
    assert cc.robust_rms(ctx, img, m) == O.robust_rms(img, m) == (0.0, 0.0, 0)


def test_chauvenet_fixture(ctx):
    vals = np.array(KATS["chauvenet_clipping_counts"]["input"]["values"], np.float32)
    img = vals.reshape(1, -1)
    got = cc.robust_rms(ctx, img)
    want = O.robust_rms(img)
    _same(got, want)
    kept = O.chauvenet_clip(vals, -1.0, 5)
    assert got[2] == len(kept) == KATS["chauvenet_clipping_counts"]["expected"][
        "automatic_zscore_until_converged"]["len"]


def test_cotton_schwab_stops_at_the_nsigma_threshold(ctx):
    """The n-sigma rule in the major/minor loop: a noisy observation cleaned
    with nsigma = 5 and no absolute threshold stops with
    NsigmaThresholdReached after the same cycles and components as the
    oracle's loop, with the same thresholds to 1e-4."""
    nx = 256
    obs = S.observation(1000.0, 1.0, 30.0, 1.4e9, nx, 8, 0.1, 1.0, 21, "nsigma")
    rng = np.random.default_rng(21)
    obs.vis = S.visibilities(obs.u, obs.v, np.zeros_like(obs.w), obs.sky, nx, nx, obs.cell,
                             0.1, rng, w_term=False)
    wt = np.ones(obs.rows, np.float32)
    og = O.StdGridder(O.Geometry(nx, nx, obs.cell, obs.cell), 128)
    p, d, acc = og.grid_dirty(obs.u, obs.v, wt, obs.vis, threads=8)
    psf_o, res_o, peak_o = og.dirty_products(p, d, acc)

    def refresh(model):
        rg, _, _ = og.residual(og.model_grid(model.astype(np.float64)), obs.u, obs.v, wt,
                               obs.vis, threads=8)
        return og.corrected_image(O.centered_ifft2(rg)) / acc.normalization_sumwt / peak_o

    kw = dict(niter=2000, gain=0.1, minor_cycle_length=40, nsigma=5.0)
    ref = O.cotton_schwab(res_o, psf_o, refresh, sidelobe=0.2, **kw)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, obs.cell, obs.cell), 128)
    out = cc.run_cotton_schwab(gg, cc.VisibilityBatch(obs.u, obs.v, obs.vis, wt),
                               cc.CleanConfig(**kw), max_psf_sidelobe=0.2)
    assert ref["stop_reason"] == "NsigmaThresholdReached"
    assert out.stop_reason == ref["stop_reason"]
    assert out.major_cycles == ref["major_cycles"] >= 2
    assert out.minor_iterations == ref["actual"]
    np.testing.assert_allclose(out.nsigma_thresholds, ref["nsigma_thresholds"], rtol=1e-4)
    assert [c[0] for c in out.components] == [tuple(c[0]) for c in ref["components"]]
    # residual errors scale with the image before cleaning (float32 sums of
    # full-amplitude visibilities), not with the small residual left after it
    err = float(np.max(np.abs(out.residual - ref["residual"])))
    assert err <= 1e-5 * float(np.max(np.abs(res_o)))
    assert err <= 1e-4 * float(np.max(np.abs(ref["residual"])))
    # the device's threshold on the oracle's residual images is the oracle's
    assert cc.nsigma_threshold(ctx, ref["residual"], 5.0) == O.nsigma_threshold(ref["residual"], 5.0)
