//! The `Cuda` arms of casa-imaging's backend enums.
//!
//! casa-imaging picks a grid backend per stage (`StandardMfsBackend`,
//! lib.rs:268-281, chosen in `StandardMfsExecutionPlan`, lib.rs:1357-1366)
//! and a minor-cycle backend (`StandardMfsMinorCycleBackend`,
//! lib.rs:1125-1131).  Its Metal arms build an executor and hand it a
//! replay of the routed visibility runs (lib.rs:48760-48830).  A `Cuda`
//! variant of each enum dispatches to `StandardMfsCudaExecutor` with the
//! same replay: every run arrives as a borrowed `Samples` view.  Runs are
//! accumulated into device-resident grids (standard gridder) or gathered
//! into one host batch (W-projection, residual refreshes), so the device
//! sees one planned pass per stage.

use crate::{
    call, cr_psf_state, cr_sums, dirty_image, hogbom, residual_image, sys, CudaError,
    DirtyProducts, Gridder, MinorCycleControl, MinorCycleOutcome, Result, Samples, WProjector,
};
use std::ptr::null_mut;

/// A replay of routed visibility runs: calls the consumer once per run.
pub type Replay<'r> = dyn FnMut(&mut dyn FnMut(&Samples<'_>) -> Result<()>) -> Result<()> + 'r;

/// The samples of every replayed run, concatenated on the host.
#[derive(Default)]
struct Gathered {
    u: Vec<f64>,
    v: Vec<f64>,
    w: Vec<f64>,
    weight: Vec<f32>,
    sumwt_factor: Vec<f32>,
    gridable: Vec<bool>,
    vis: Vec<[f32; 2]>,
}

impl Gathered {
    fn push(&mut self, s: &Samples<'_>) {
        let n = s.u_lambda.len();
        self.u.extend_from_slice(s.u_lambda);
        self.v.extend_from_slice(s.v_lambda);
        if s.w_lambda.is_empty() {
            self.w.extend(std::iter::repeat(0.0).take(n));
        } else {
            self.w.extend_from_slice(s.w_lambda);
        }
        self.weight.extend_from_slice(s.weight);
        if s.sumwt_factor.is_empty() {
            self.sumwt_factor.extend(std::iter::repeat(1.0).take(n));
        } else {
            self.sumwt_factor.extend_from_slice(s.sumwt_factor);
        }
        if s.gridable.is_empty() {
            self.gridable.extend(std::iter::repeat(true).take(n));
        } else {
            self.gridable.extend_from_slice(s.gridable);
        }
        self.vis.extend_from_slice(s.visibility);
    }

    fn samples(&self) -> Samples<'_> {
        Samples {
            u_lambda: &self.u,
            v_lambda: &self.v,
            w_lambda: &self.w,
            weight: &self.weight,
            sumwt_factor: &self.sumwt_factor,
            gridable: &self.gridable,
            visibility: &self.vis,
        }
    }

    fn collect(replay: &mut Replay<'_>) -> Result<Gathered> {
        let mut g = Gathered::default();
        replay(&mut |s: &Samples<'_>| {
            g.push(s);
            Ok(())
        })?;
        if g.u.is_empty() {
            return Err(CudaError::NoUsableSamples);
        }
        Ok(g)
    }
}

/// The device executor behind `StandardMfsBackend::Cuda`.
pub struct StandardMfsCudaExecutor<'g> {
    gridder: &'g Gridder<'g>,
    wproj: Option<&'g WProjector<'g>>,
}

impl<'g> StandardMfsCudaExecutor<'g> {
    pub fn new(gridder: &'g Gridder<'g>, wproj: Option<&'g WProjector<'g>>) -> Self {
        StandardMfsCudaExecutor { gridder, wproj }
    }

    /// Initial PSF and residual images of the replayed runs
    /// (`accumulate_dirty_psf_and_residual_standard_streaming_grid`,
    /// lib.rs:68306, then `dirty_grids_to_psf_and_residual_owned`,
    /// lib.rs:48987-49130).  The standard gridder accumulates run by run into
    /// device-resident grids (`cr_accumulator_*`, the
    /// `StandardMfsDirtyAccumulator` of lib.rs:3259-3380); W-projection
    /// grids the gathered runs in one planned pass.
    pub fn dirty_products_replay(&self, replay: &mut Replay<'_>) -> Result<DirtyProducts> {
        if self.wproj.is_some() {
            let g = Gathered::collect(replay)?;
            return dirty_image(self.gridder, self.wproj, &g.samples());
        }
        let ctx = self.gridder_ctx();
        let mut acc: *mut sys::cr_accumulator = null_mut();
        call(|e| unsafe { sys::cr_accumulator_create(ctx, self.gridder.raw(), &mut acc, e) })?;
        let result = (|| -> Result<DirtyProducts> {
            replay(&mut |s: &Samples<'_>| {
                let batch = s.batch()?;
                let mut sums = cr_sums::default();
                call(|e| unsafe { sys::cr_accumulator_add(ctx, acc, &batch, &mut sums, e) })
            })?;
            let n = self.gridder.nx * self.gridder.ny;
            let mut out = DirtyProducts { psf: vec![0.0; n], residual: vec![0.0; n],
                                          state: cr_psf_state::default(),
                                          sums: cr_sums::default() };
            call(|e| unsafe {
                sys::cr_accumulator_finish(ctx, acc, out.psf.as_mut_ptr(),
                                           out.residual.as_mut_ptr(), sys::CR_HOST,
                                           &mut out.state, &mut out.sums, e)
            })?;
            Ok(out)
        })();
        unsafe { sys::cr_accumulator_destroy(acc) };
        result
    }

    /// A residual refresh of the replayed runs against `model`
    /// (`compute_residual_w_project`, lib.rs:70646-70700, and the standard
    /// residual path of lib.rs:48760-48830): one fused degrid + residual
    /// grid pass, then the image stage with the dirty products' state.
    pub fn residual_image_replay(&self, replay: &mut Replay<'_>, model: &[f32],
                                 state: &cr_psf_state) -> Result<Vec<f32>> {
        let g = Gathered::collect(replay)?;
        residual_image(self.gridder, self.wproj, &g.samples(), model, state)
    }

    fn gridder_ctx(&self) -> *mut sys::cr_ctx {
        self.gridder.ctx.raw()
    }
}

/// `StandardMfsMinorCycleBackend::Cuda`: the Hogbom minor cycle of
/// `run_hogbom_minor_cycle_with_progress` (lib.rs:59675-59711) as one
/// persistent device loop.
pub fn hogbom_minor_cycle(gridder: &Gridder<'_>, model: &mut [f32], residual: &mut [f32],
                          psf: &[f32], mask: Option<&[bool]>, control: &MinorCycleControl)
                          -> Result<MinorCycleOutcome> {
    hogbom(gridder.ctx, model, residual, psf, mask, gridder.nx, gridder.ny, control)
}
