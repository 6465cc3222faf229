"""The timed CPU path against the FP64 oracle.

The CPU baseline and `bench.py --impl reference` time the reference's
W-projection loops restated in the reference's own precision (Complex32
kernels and grids, float32 products: oracle `grid_dirty_f32` /
`degrid_f32`, gridder.rs:3680-3747); the FP64 functions are the parity
checker.  The two must compute the same thing: grids and predictions agree
to float32 rounding (1e-6 of the peak), and the counts and sums of weights
are the same decisions.
"""
import numpy as np

from oracle import oracle as O

from gpu_common import peak_norm_err, random_batch


def test_wproj_f32_restatement_matches_fp64():
    nx, cell = 128, 2e-5
    og = O.StdGridder(O.Geometry(nx, nx, cell, cell), 100)
    ow = O.WProjector(og.geom, og, 2000.0, planes=8, sampling=8, support_min=4, support_max=8)
    rng = np.random.default_rng(21)
    margin = int(ow.support.max()) + 2
    u, v, w, wt, vis = random_batch(rng, 4000, og.gnx, og.du, margin=margin, w_max=2000.0)
    psf, dirty, acc = ow.grid_dirty(u, v, w, wt, vis)
    psf32, dirty32, acc32 = ow.grid_dirty_f32(u, v, w, wt, vis)
    assert acc32.gridded == acc.gridded and acc32.skipped == acc.skipped
    assert abs(acc32.normalization_sumwt - acc.normalization_sumwt) <= 1e-6 * acc.normalization_sumwt
    assert peak_norm_err(psf32, psf) <= 1e-6
    assert peak_norm_err(dirty32, dirty) <= 1e-6
    grid = (rng.normal(size=(og.gnx, og.gny)) + 1j * rng.normal(size=(og.gnx, og.gny))) \
        .astype(np.complex64)
    pred = ow.degrid(grid, u, v, w)
    pred32 = ow.degrid_f32(grid, u, v, w)
    assert peak_norm_err(pred32, pred) <= 1e-6
