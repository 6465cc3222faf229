"""Host logic of the request-level entry points (casars_cuda/run.py), on CPU.

run_imaging and run_standard_mfs_dirty_grid_plan take the reference's
request shape (ImagingRequest, types.rs:2291-2337) with several visibility
batches: these are merged field by field (missing weights and sumwt factors
as ones, w and gridable kept only when given), per-sample weights are split
back per batch, and invalid requests are refused before any device work.
"""
import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import run as R

torch = pytest.importorskip("torch")


def _batch(n, seed, weight=True, w=False, gridable=False, as_torch=False):
    rng = np.random.default_rng(seed)
    u, v = rng.normal(size=n), rng.normal(size=n)
    vis = (rng.normal(size=n) + 1j * rng.normal(size=n)).astype(np.complex64)
    wt = rng.uniform(0.5, 2.0, n).astype(np.float32) if weight else None
    ww = rng.normal(size=n) if w else None
    g = (rng.random(n) < 0.9) if gridable else None
    if as_torch:
        t = lambda a: None if a is None else torch.as_tensor(a)
        return cc.VisibilityBatch(t(u), t(v), t(vis), t(wt), t(ww), None, t(g))
    return cc.VisibilityBatch(u, v, vis, wt, ww, None, g)


def test_merge_concatenates_fields_and_fills_ones():
    a, b = _batch(5, 1, w=True), _batch(3, 2, weight=False, w=True)
    m = R._merge([a, b])
    assert len(m) == 8
    np.testing.assert_array_equal(m.u_lambda, np.concatenate([a.u_lambda, b.u_lambda]))
    np.testing.assert_array_equal(m.visibility, np.concatenate([a.visibility, b.visibility]))
    np.testing.assert_array_equal(m.weight, np.concatenate([a.weight, np.ones(3, np.float32)]))
    np.testing.assert_array_equal(m.sumwt_factor, np.ones(8, np.float32))
    np.testing.assert_array_equal(m.w_lambda, np.concatenate([a.w_lambda, b.w_lambda]))
    assert m.gridable is None
    assert R._merge([a]) is a


def test_merge_torch_batches():
    a, b = _batch(4, 3, as_torch=True), _batch(2, 4, as_torch=True)
    m = R._merge([a, b])
    assert isinstance(m.u_lambda, torch.Tensor) and m.u_lambda.shape == (6,)
    assert torch.equal(m.weight, torch.cat([a.weight, b.weight]))


def test_merge_refuses_a_field_given_in_some_batches_only():
    with pytest.raises(ValueError):
        R._merge([_batch(3, 5, gridable=True), _batch(3, 6)])
    with pytest.raises(ValueError):
        R._merge([_batch(3, 5, w=True), _batch(3, 6)])


def test_split_weights_per_batch():
    a, b, c = _batch(2, 7), _batch(3, 8), _batch(4, 9)
    wt = np.arange(9, dtype=np.float32)
    parts = R._split_weights([a, b, c], wt)
    assert [p.weight.tolist() for p in parts] == [[0, 1], [2, 3, 4], [5, 6, 7, 8]]
    assert parts[1].u_lambda is b.u_lambda and parts[2].visibility is c.visibility


def _request(**kw):
    geom = cc.ImageGeometry(64, 64, 1e-4, 1e-4)
    return R.ImagingRequest(geom, kw.pop("batches", [_batch(4, 10)]), **kw)


@pytest.mark.parametrize("kw, msg", [
    (dict(deconvolver="multiscale"), "deconvolver"),
    (dict(w_term_mode="awproject"), "w_term_mode"),
    (dict(batches=[]), "no visibility batches"),
])
def test_run_imaging_refuses_invalid_requests(kw, msg):
    with pytest.raises(ValueError, match=msg):
        R.run_imaging(None, _request(**kw))


@pytest.mark.parametrize("kw, msg", [
    (dict(w_term_mode="wproject"), "w-term"),
    (dict(batches=[]), "no visibility batches"),
])
def test_dirty_grid_plan_refuses_invalid_requests(kw, msg):
    with pytest.raises(ValueError, match=msg):
        R.run_standard_mfs_dirty_grid_plan(None, _request(**kw))
