"""The row-block read-ahead feed (cr_row_feed_*) against the oracle.

Rows of a small observation (4 correlations XX, XY, YX, YY over 6 channels,
seeded flags, bad weights and visibilities, non-gridable rows) are fed in
row blocks through page-locked slots, the way stream_imaging_source_read_
ahead_blocks (casars-imager/src/lib.rs:36608-36760) streams MeasurementSet
row blocks:

* the Stokes-I PSF and residual images agree with the oracle's images of the
  whole prepared data within 1e-5 of the peak, with the oracle's gridded
  count and sums of weights, for read-ahead depths 1, 2 and 3 and a ragged
  last block;
* the summary counts the blocks, the kept samples and the uploaded bytes;
* a feed keeps accumulating after finish, and misuse (a slot that was not
  acquired, too many rows, nothing usable fed) is reported as the reference's
  error kinds.
"""
import numpy as np
import pytest

import casars_cuda as cc
from casars_cuda import synthetic as S
from oracle import oracle as O
from oracle import rows as OR

from gpu_common import peak_norm_err

pytestmark = pytest.mark.gpu

CORR = [9, 10, 11, 12]


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def rows():
    obs = S.cube_observation(channels=6, nx=128, hours=1.0, dump_s=90.0, n_sources=4, seed=21)
    R, C, K = obs.rows, obs.channels, 4
    rng = np.random.default_rng(23)
    vis = S.cube_visibilities(obs).T
    data = np.empty((R, C, K), np.complex64)
    data[:, :, 0] = vis * (1 + 0.05j)
    data[:, :, 3] = vis * (1 - 0.03j)
    data[:, :, 1] = 0.01 * (rng.normal(size=(R, C)) + 1j * rng.normal(size=(R, C)))
    data[:, :, 2] = 0.01 * (rng.normal(size=(R, C)) + 1j * rng.normal(size=(R, C)))
    data[5, 2, 0] = np.nan
    flag = (rng.random((R, C, K)) < 0.1).astype(np.uint8)
    weight = rng.uniform(0.5, 2.0, (R, K)).astype(np.float32)
    spectrum = rng.uniform(0.5, 2.0, (R, C, K)).astype(np.float32)
    spectrum[8, 0, 0] = 0.0
    gridable = (rng.random(R) > 0.05).astype(np.uint8)
    uvw = np.stack([obs.u_m, obs.v_m, rng.normal(0.0, 50.0, R)], 1)
    return obs, uvw, data, flag, weight, spectrum, gridable


@pytest.fixture(scope="module")
def reference(rows):
    obs, uvw, data, flag, weight, spectrum, gridable = rows
    corr0, corr1, transform, factor = OR.plane_polarization("I", CORR)
    ref = OR.prepare(uvw, obs.lambda_scale, data, flag, weight, spectrum, gridable, corr0,
                     corr1, transform, factor)
    og = O.StdGridder(O.Geometry(obs.nx, obs.nx, obs.cell, obs.cell), 128)
    p, d, acc = og.grid_dirty(ref["u"], ref["v"], ref["weight"], ref["vis"],
                              ref["sumwt_factor"], ref["gridable"], threads=8)
    psf_o, res_o, _ = og.dirty_products(p, d, acc)
    return ref, psf_o, res_o, acc


def _feed(ctx, rows, block_rows, live):
    obs, uvw, data, flag, weight, spectrum, gridable = rows
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(obs.nx, obs.nx, obs.cell, obs.cell), 128)
    feed = cc.RowFeed(gg, obs.lambda_scale, cc.Polarization.for_plane("I", CORR), 4,
                      block_rows, live, has_flag=True, has_weight_spectrum=True,
                      has_gridable=True)
    return gg, feed


def _producer(rows, block_rows, start=0, stop=None):
    obs, uvw, data, flag, weight, spectrum, gridable = rows
    stop = obs.rows if stop is None else stop
    pos = [start]

    def produce(slot):
        r0 = pos[0]
        if r0 >= stop:
            return None
        n = min(block_rows, stop - r0)
        sl = slice(r0, r0 + n)
        slot.uvw_m[:n] = uvw[sl]
        slot.data[:n] = data[sl]
        slot.flag[:n] = flag[sl]
        slot.weight[:n] = weight[sl]
        slot.weight_spectrum[:n] = spectrum[sl]
        slot.gridable[:n] = gridable[sl]
        pos[0] = r0 + n
        return n

    return produce


@pytest.mark.parametrize("block_rows,live", [(97, 3), (97, 1), (250, 2), (100000, 2)])
def test_feed_matches_oracle(ctx, rows, reference, block_rows, live):
    obs = rows[0]
    ref, psf_o, res_o, acc = reference
    gg, feed = _feed(ctx, rows, block_rows, live)
    try:
        blocks = cc.stream_row_blocks(feed, _producer(rows, block_rows))
        psf, res, state, sums, summary = feed.finish()
    finally:
        feed.close()
    assert blocks == -(-obs.rows // block_rows)
    assert summary.row_blocks == blocks
    assert summary.streamed_samples == len(ref["u"])
    C, K = obs.channels, 4
    per_row = 24 + C * K * 8 + K * 4 + C * K + C * K * 4 + 1
    assert summary.source_bytes == obs.rows * per_row
    assert 1 <= summary.live_row_block_high_water <= live
    assert summary.consumer_elapsed_s > 0.0
    assert sums.gridded_samples == acc.gridded
    assert sums.normalization_sumwt == pytest.approx(acc.normalization_sumwt, rel=1e-10)
    assert peak_norm_err(psf, psf_o) <= 1e-5
    assert peak_norm_err(res, res_o) <= 1e-5


def test_feed_accumulates_after_finish(ctx, rows, reference):
    obs = rows[0]
    ref, psf_o, res_o, acc = reference
    half = obs.rows // 2
    gg, feed = _feed(ctx, rows, 64, 2)
    try:
        cc.stream_row_blocks(feed, _producer(rows, 64, 0, half))
        _, _, _, first, s1 = feed.finish()
        cc.stream_row_blocks(feed, _producer(rows, 64, half))
        psf, res, _, sums, s2 = feed.finish()
    finally:
        feed.close()
    assert 0 < first.gridded_samples < sums.gridded_samples == acc.gridded
    assert s2.row_blocks == -(-half // 64) + -(-(obs.rows - half) // 64)
    assert s2.streamed_samples == len(ref["u"]) and s1.streamed_samples < len(ref["u"])
    assert peak_norm_err(psf, psf_o) <= 1e-5
    assert peak_norm_err(res, res_o) <= 1e-5


def test_feed_misuse_is_reported(ctx, rows):
    gg, feed = _feed(ctx, rows, 32, 2)
    try:
        with pytest.raises(cc.CasarsCudaError) as e:
            feed.finish()
        assert e.value.kind == "NoUsableSamples"
        slot = feed.acquire()
        with pytest.raises(cc.CasarsCudaError) as e:
            feed.submit(slot, 33)
        assert e.value.kind == "InvalidRequest"
        other = feed.acquire()
        assert other.slot != slot.slot
        feed.submit(other, 0)
        with pytest.raises(cc.CasarsCudaError):
            feed.submit(other, 1)          # handed back already
        feed.submit(slot, 0)
        with pytest.raises(cc.CasarsCudaError) as e:
            feed.finish()
        assert e.value.kind == "NoUsableSamples"
    finally:
        feed.close()
