"""run_imaging over the library: the request / result shape of casa-imaging's
top-level entry point (run_imaging, lib.rs:3468; ImagingRequest,
types.rs:2291-2337; ImagingResult) for the standard and W-projection
gridders, natural / uniform / Briggs weighting and the Hogbom or Clark
deconvolver, and the standard-MFS plan entry points around it
(run_standard_mfs_plan, lib.rs:1742; run_standard_mfs_dirty_grid_plan,
lib.rs:1966; finish_standard_mfs_dirty_grid_result, lib.rs:2000).  Mosaic,
AW-projection, MT-MFS, multiscale, masks and initial models are outside
this library."""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import clean as CL
from . import imaging as im

try:
    import torch
except Exception:  # pragma: no cover
    torch = None


@dataclass
class ImagingRequest:
    """ImagingRequest (types.rs:2291-2337), the fields this library serves."""
    geometry: im.ImageGeometry
    visibility_batches: List[im.VisibilityBatch]
    clean: CL.CleanConfig = field(default_factory=lambda: CL.CleanConfig(niter=0))
    weighting: str = "natural"          # natural | uniform | briggs
    robust: float = 0.0
    deconvolver: str = "hogbom"         # hogbom | clark
    w_term_mode: str = "none"           # none | wproject
    w_project_planes: Optional[int] = None
    oversampling: int = 100
    padding: float = 1.2
    # ImagingFftPlan.dirty_products.precision (lib.rs:1314-1319): auto | f32 | f64
    fft_precision: str = "auto"


@dataclass
class ImagingResult:
    """ImagingResult: image planes and the diagnostics the controller reports."""
    psf: object
    residual: object
    model: object
    image: object
    sumwt: float
    beam: Optional[im.BeamFit]
    psf_state: im.PsfState
    major_cycles: int = 0
    minor_iterations: int = 0
    stop_reason: Optional[str] = None
    components: list = field(default_factory=list)


def _cat(parts):
    parts = [p for p in parts]
    if any(p is None for p in parts):
        if all(p is None for p in parts):
            return None
        raise ValueError("a field is given in some batches and not in others")
    if torch is not None and isinstance(parts[0], torch.Tensor):
        return torch.cat([p.reshape(-1) for p in parts])
    return np.concatenate([np.asarray(p).reshape(-1) for p in parts])


def _merge(batches: List[im.VisibilityBatch]) -> im.VisibilityBatch:
    if len(batches) == 1:
        return batches[0]
    n = [len(b) for b in batches]
    ones = lambda b, k: (torch.ones(k, dtype=torch.float32, device=b.u_lambda.device)
                         if torch is not None and isinstance(b.u_lambda, torch.Tensor)
                         else np.ones(k, np.float32))
    return im.VisibilityBatch(
        _cat([b.u_lambda for b in batches]), _cat([b.v_lambda for b in batches]),
        _cat([b.visibility for b in batches]),
        _cat([b.weight if b.weight is not None else ones(b, k) for b, k in zip(batches, n)]),
        _cat([b.w_lambda for b in batches]) if any(b.w_lambda is not None for b in batches)
        else None,
        _cat([b.sumwt_factor if b.sumwt_factor is not None else ones(b, k)
              for b, k in zip(batches, n)]),
        _cat([b.gridable for b in batches]) if any(b.gridable is not None for b in batches)
        else None)


def run_imaging(ctx: im.Context, request: ImagingRequest) -> ImagingResult:
    """run_imaging (lib.rs:3468): weighting, the dirty products, the
    Cotton-Schwab loop with the chosen minor cycle (none when niter = 0),
    and the restored image (the residual when no component was found)."""
    if request.deconvolver not in ("hogbom", "clark"):
        raise ValueError("deconvolver must be hogbom or clark")
    if request.w_term_mode not in ("none", "wproject"):
        raise ValueError("w_term_mode must be none or wproject")
    if not request.visibility_batches:
        raise ValueError("no visibility batches")
    batch = _merge(request.visibility_batches)
    previous = ctx.image_fft_precision
    ctx.set_image_fft_precision(request.fft_precision)
    try:
        return _run(ctx, request, batch)
    finally:
        ctx.set_image_fft_precision(previous)


def _run(ctx: im.Context, request: ImagingRequest, batch: im.VisibilityBatch) -> ImagingResult:
    gg = im.StandardGridder(ctx, request.geometry, request.oversampling, request.padding)
    wp = None
    if request.w_term_mode == "wproject":
        if batch.w_lambda is None:
            raise ValueError("wproject needs w_lambda")
        w = batch.w_lambda
        max_w = float(torch.max(torch.abs(w))) if torch is not None and \
            isinstance(w, torch.Tensor) else float(np.max(np.abs(w)))
        wp = im.WProjector(gg, max_w, planes=request.w_project_planes)
    if request.weighting != "natural":
        wt, _ = im.apply_weighting(gg, batch, request.weighting, request.robust)
        batch = im.VisibilityBatch(batch.u_lambda, batch.v_lambda, batch.visibility, wt,
                                   batch.w_lambda, batch.sumwt_factor, batch.gridable)
    geom = request.geometry
    cell = (geom.cell_x_rad, geom.cell_y_rad)
    if request.clean.niter == 0:
        psf, residual, state, _ = im.dirty_image(gg, batch, wp)
        beam, _, _ = im.fit_beam(psf, cell, request.clean.psf_cutoff, ctx=ctx)
        model = CL._zeros_like(residual)
        return ImagingResult(psf, residual, model, residual, float(state.reported_sumwt), beam,
                             state)
    run = CL.run_clark_cotton_schwab if request.deconvolver == "clark" else CL.run_cotton_schwab
    out = run(gg, batch, request.clean, wp)
    image = out.restored if out.restored is not None else out.residual
    return ImagingResult(out.psf, out.residual, out.model, image,
                         float(out.psf_state.reported_sumwt), out.beam, out.psf_state,
                         out.major_cycles, out.minor_iterations, out.stop_reason,
                         out.components)


def run_standard_mfs_plan(ctx: im.Context, request: ImagingRequest) -> ImagingResult:
    """run_standard_mfs_plan (lib.rs:1742) over weighted batches: the
    canonical standard-MFS run, i.e. run_imaging with the standard gridder
    (no w-term)."""
    if request.w_term_mode != "none":
        raise ValueError("the standard-MFS plan takes no w-term")
    return run_imaging(ctx, request)


@dataclass
class StandardMfsDirtyGridResult:
    """StandardMfsDirtyGridResult (lib.rs:1861): the raw result of a
    dirty-only plan -- PSF and dirty grids held on the device by an
    accumulator -- with the sums of every replayed block."""
    request: ImagingRequest
    accumulator: im.DirtyAccumulator
    block_sums: List[im.GridSums]

    @property
    def gridded_samples(self) -> int:
        return sum(s.gridded_samples for s in self.block_sums)

    @property
    def skipped_samples(self) -> int:
        return sum(s.skipped_samples for s in self.block_sums)


def _split_weights(batches: List[im.VisibilityBatch], weights) -> List[im.VisibilityBatch]:
    out, at = [], 0
    for b in batches:
        n = len(b)
        w = weights[at:at + n]
        at += n
        out.append(im.VisibilityBatch(b.u_lambda, b.v_lambda, b.visibility, w, b.w_lambda,
                                      b.sumwt_factor, b.gridable))
    return out


def run_standard_mfs_dirty_grid_plan(ctx: im.Context,
                                     request: ImagingRequest) -> StandardMfsDirtyGridResult:
    """run_standard_mfs_dirty_grid_plan (lib.rs:1966): the request's batches
    replayed one block at a time into device-resident grids (grid
    accumulation only, no FFT).  Non-natural weighting takes its density
    over all blocks first, as the reference's weighting plan does."""
    if request.w_term_mode != "none":
        raise ValueError("the standard-MFS dirty plan takes no w-term")
    if not request.visibility_batches:
        raise ValueError("no visibility batches")
    gg = im.StandardGridder(ctx, request.geometry, request.oversampling, request.padding)
    blocks = list(request.visibility_batches)
    if request.weighting != "natural":
        merged = _merge(blocks)
        wt, _ = im.apply_weighting(gg, merged, request.weighting, request.robust)
        blocks = _split_weights(blocks, wt)
    acc = im.DirtyAccumulator(gg)
    sums = [acc.add(b) for b in blocks]
    return StandardMfsDirtyGridResult(request, acc, sums)


def finish_standard_mfs_dirty_grid_result(ctx: im.Context,
                                          result: StandardMfsDirtyGridResult):
    """finish_standard_mfs_dirty_grid_result (lib.rs:2000): the dirty
    products of a raw grid result -- (psf, residual, PsfState) -- with the
    image-stage FFT precision of the result's request."""
    previous = ctx.image_fft_precision
    ctx.set_image_fft_precision(result.request.fft_precision)
    try:
        psf, residual, state, _ = result.accumulator.finish()
    finally:
        ctx.set_image_fft_precision(previous)
    return psf, residual, state
