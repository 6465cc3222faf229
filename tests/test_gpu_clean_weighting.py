"""Hogbom minor cycle, weighting and the forward/adjoint pair on the GPU.

Hogbom and weighting are bit-exact against the oracle on identical inputs
(component positions, fluxes, residual and model images; imaging weights).
The forward/adjoint pair passes the dot-product test <A x, y> = <x, A^H y>
to 1e-6 of ||A x|| ||y|| (the usual normalisation of the test: the
Cauchy-Schwarz bound of both sides) and to 1e-5 of |<A x, y>| itself.
"""
import json
import os

import numpy as np
import pytest

import casars_cuda as cc
from oracle import oracle as O

from gpu_common import peak_norm_err, random_batch

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
KATS = {k["name"]: k for k in json.load(open(os.path.join(HERE, "golden", "reference_kats.json")))["kats"]}


@pytest.fixture(scope="module")
def ctx():
    c = cc.Context(0)
    yield c
    c.close()


def test_hogbom_kats(ctx):
    img = np.array(KATS["hogbom_y_major_tie_break"]["input"]["image"], np.float32)
    out = cc.run_hogbom_minor_cycle(ctx, np.zeros_like(img), img, np.zeros_like(img), 1.0, 0,
                                    inclusive=True)
    assert tuple(out.positions[0]) == (1, 0) and out.peaks[0] == -4.0
    k = KATS["hogbom_inclusive_budget"]
    res = np.array(k["input"]["residual"], np.float32)
    psf = np.array(k["input"]["psf"], np.float32)
    out = cc.run_hogbom_minor_cycle(ctx, np.zeros_like(res), res, psf, 0.5, 1)
    assert out.actual_updates == 2 and out.reported_updates == 1
    assert abs(out.model[3, 3] - 0.9) < 1e-6


def test_hogbom_trace_lists_the_cycle_components(ctx, tmp_path, monkeypatch):
    """CASA_RS_HOGBOM_TRACE: one line per component of the device cycle, in
    order, with the returned positions, peaks and fluxes."""
    path = tmp_path / "trace.jsonl"
    monkeypatch.setenv("CASA_RS_HOGBOM_TRACE", str(path))
    rng = np.random.default_rng(5)
    res = (0.01 * rng.normal(size=(64, 64))).astype(np.float32)
    res[20, 30] = 1.0
    res[40, 12] = -0.7
    psf = np.zeros((64, 64), np.float32)
    psf[32, 32] = 1.0
    out = cc.run_hogbom_minor_cycle(ctx, np.zeros_like(res), res, psf, 0.2, 25,
                                    reffreq_hz=1.25e9)
    lines = [json.loads(x) for x in path.read_text().splitlines()]
    assert len(lines) == out.actual_updates > 0
    for k, rec in enumerate(lines):
        assert rec["event"] == "component" and rec["backend"] == "cuda"
        assert rec["cycle_update"] == k and rec["reffreq_hz"] == 1.25e9
        assert (rec["x"], rec["y"]) == tuple(int(v) for v in out.positions[k])
        assert rec["peak"] == float(out.peaks[k]) and rec["component"] == float(out.fluxes[k])


@pytest.mark.parametrize("shape,masked", [((64, 64), False), ((200, 150), True), ((512, 512), False)])
def test_hogbom_bit_exact_against_oracle(ctx, shape, masked):
    rng = np.random.default_rng(3)
    nx, ny = shape
    x = np.arange(nx)[:, None] - nx // 2
    y = np.arange(ny)[None, :] - ny // 2
    psf = np.exp(-(x * x + y * y) / 18.0).astype(np.float32)
    psf += (0.02 * rng.normal(size=shape)).astype(np.float32)
    psf[nx // 2, ny // 2] = 1.0
    res = (0.01 * rng.normal(size=shape)).astype(np.float32)
    for _ in range(12):
        px, py = rng.integers(10, nx - 10), rng.integers(10, ny - 10)
        res[px, py] += rng.uniform(0.1, 1.0)
    res[5, 7] = res[7, 5] = 2.0  # an exact tie
    mask = (rng.uniform(size=shape) > 0.05).astype(np.uint8) if masked else None
    ref = O.hogbom(res, psf, 0.1, 300, threshold=0.005, mask=mask)
    out = cc.run_hogbom_minor_cycle(ctx, np.zeros_like(res), res, psf, 0.1, 300, threshold=0.005,
                                    mask=mask)
    assert out.actual_updates == ref["actual"] and out.reported_updates == ref["reported"]
    np.testing.assert_array_equal(out.positions[:, 0], ref["x"])
    np.testing.assert_array_equal(out.positions[:, 1], ref["y"])
    np.testing.assert_array_equal(out.fluxes, ref["flux"])
    np.testing.assert_array_equal(out.residual, ref["residual"])
    np.testing.assert_array_equal(out.model, ref["model"])
    assert {0: None, 1: "GlobalThresholdReached"}[ref["stop_reason"]] == out.stop_reason


def test_hogbom_stop_rules(ctx):
    res = np.zeros((16, 16), np.float32)
    res[4, 4] = 1.0
    psf = np.zeros((16, 16), np.float32)
    psf[8, 8] = 1.0
    out = cc.run_hogbom_minor_cycle(ctx, np.zeros_like(res), res, psf, 0.5, 50, cycle_threshold=0.2)
    ref = O.hogbom(res, psf, 0.5, 50, cycle_threshold=0.2)
    assert out.actual_updates == ref["actual"] and out.stop_reason == "CycleThresholdReached"
    out = cc.run_hogbom_minor_cycle(ctx, np.zeros_like(res), res, psf, 0.5, 5,
                                    mask=np.zeros((16, 16), np.uint8))
    assert out.actual_updates == 0 and out.stop_reason == "NoCleanablePixels"


@pytest.mark.parametrize("mode,robust", [("uniform", 0.0), ("briggs", 0.5), ("briggs", -1.0), ("natural", 0.0)])
def test_weighting_bit_exact(ctx, mode, robust):
    rng = np.random.default_rng(4)
    nx = 128
    cell = 2e-5
    geom = O.Geometry(nx, nx, cell, cell)
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell))
    du = 1.0 / (nx * cell)
    u = rng.uniform(-60 * du, 60 * du, 50000)
    v = rng.uniform(-60 * du, 60 * du, 50000)
    wt = np.ones(len(u), np.float32)
    wt[::17] = 0.0
    ref, dens, f2 = O.apply_weighting(geom, u, v, wt, mode, robust)
    got, f2g = cc.apply_weighting(gg, cc.VisibilityBatch(u, v, np.zeros(len(u), np.complex64), wt),
                                  mode, robust)
    assert np.float32(f2g) == np.float32(f2)
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("wproj", [False, True])
def test_forward_adjoint_dot_product(ctx, wproj):
    rng = np.random.default_rng(8)
    nx = 128
    cell = 1e-4 if not wproj else 1.2e-4
    gg = cc.StandardGridder(ctx, cc.ImageGeometry(nx, nx, cell, cell))
    gw = cc.WProjector(gg, 500.0, planes=8, sampling=4, support_law=(4, 10)) if wproj else None
    du = 1.0 / (gg.grid_shape()[0] * cell)
    u, v, w, wt, vis = random_batch(rng, 20000, gg.grid_shape()[0], du, margin=14, w_max=500.0,
                                    weights=False)
    b = cc.VisibilityBatch(u, v, vis, wt, w)
    x = rng.normal(size=(nx, nx)).astype(np.float32)
    ax = cc.predict(gg, b, x, gw)
    aty = cc.adjoint(gg, b, gw)
    lhs = np.sum(np.conj(ax.astype(np.complex128)) * vis.astype(np.complex128)).real
    rhs = np.sum(x.astype(np.float64) * aty.astype(np.float64))
    bound = np.linalg.norm(ax.astype(np.complex128)) * np.linalg.norm(vis.astype(np.complex128))
    assert abs(lhs - rhs) <= 1e-6 * bound
    assert abs(lhs - rhs) <= 1e-5 * max(abs(lhs), abs(rhs))
