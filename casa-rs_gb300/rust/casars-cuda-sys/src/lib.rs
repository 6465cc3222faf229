//! Bindings of libcasars_cuda for casa-imaging.
//!
//! `sys` holds the raw declarations of `include/casars_cuda.h` (written by
//! `gen_sys.py`).  The types below own the library's handles and turn its
//! status codes into `CudaError`, whose variants follow `ImagingError`
//! (`crates/casa-imaging/src/error.rs:7-24`).  Images are x-major with y
//! contiguous (`Array2` standard layout), complex arrays are interleaved
//! `f32` pairs (`Complex32` memory), and every call here passes host memory
//! (`CR_HOST`): the library copies in and out around its device work.
//! `backend` shows the `StandardMfsBackend::Cuda` and
//! `StandardMfsMinorCycleBackend::Cuda` arms built on them.

pub mod backend;
pub mod sys;

use std::ffi::CStr;
use std::fmt;
use std::marker::PhantomData;
use std::os::raw::{c_char, c_void};
use std::ptr::{null, null_mut};

pub use sys::{cr_beam, cr_grid_info, cr_psf_state, cr_sums, cr_timings, cr_wproj_info};

/// A failed library call, mapped onto `ImagingError`'s variants.
#[derive(Clone, Debug, PartialEq, Eq)]
pub enum CudaError {
    /// `CR_INVALID`: `ImagingError::InvalidRequest`.
    InvalidRequest(String),
    /// `CR_NO_SAMPLES`: `ImagingError::NoUsableSamples`.
    NoUsableSamples,
    /// `CR_NORMALIZATION`: `ImagingError::Normalization`.
    Normalization(String),
    /// `CR_BUFFER_SMALL`, `CR_CUDA`, `CR_TIMEOUT`: `ImagingError::Unsupported`
    /// with the library's message.
    Unsupported(String),
}

impl fmt::Display for CudaError {
    fn fmt(&self, f: &mut fmt::Formatter<'_>) -> fmt::Result {
        match self {
            CudaError::InvalidRequest(m) => write!(f, "invalid request: {m}"),
            CudaError::NoUsableSamples => {
                write!(f, "no usable visibility samples remain after validation and flagging")
            }
            CudaError::Normalization(m) => write!(f, "FFT/grid normalization failed: {m}"),
            CudaError::Unsupported(m) => write!(f, "unsupported mode: {m}"),
        }
    }
}

impl std::error::Error for CudaError {}

pub type Result<T> = std::result::Result<T, CudaError>;

/// Status code plus the library's message (freed here) to a `Result`.
fn check(code: i32, err: *mut c_char) -> Result<()> {
    let msg = if err.is_null() {
        String::new()
    } else {
        // SAFETY: the library fills `err` with a NUL-terminated string that
        // the caller releases with cr_free_error.
        let s = unsafe { CStr::from_ptr(err) }.to_string_lossy().into_owned();
        unsafe { sys::cr_free_error(err) };
        s
    };
    match code {
        sys::CR_OK => Ok(()),
        sys::CR_INVALID => Err(CudaError::InvalidRequest(msg)),
        sys::CR_NO_SAMPLES => Err(CudaError::NoUsableSamples),
        sys::CR_NORMALIZATION => Err(CudaError::Normalization(msg)),
        sys::CR_TIMEOUT => Err(CudaError::Unsupported(format!("device wait timed out: {msg}"))),
        _ => Err(CudaError::Unsupported(msg)),
    }
}

/// Runs `f` with an error slot and maps its status.
fn call<F: FnOnce(*mut *mut c_char) -> i32>(f: F) -> Result<()> {
    let mut err: *mut c_char = null_mut();
    let code = f(&mut err);
    check(code, err)
}

fn want_len(what: &str, got: usize, want: usize) -> Result<()> {
    if got != want {
        return Err(CudaError::InvalidRequest(format!("{what} has {got} elements, expected {want}")));
    }
    Ok(())
}

/// Why a minor cycle ended (`CleanStopReason`, lib.rs:74690-74712).
#[derive(Clone, Copy, Debug, PartialEq, Eq)]
pub enum StopReason {
    /// The cycle ran out of its iteration budget.
    IterationBudget,
    GlobalThreshold,
    CycleThreshold,
    NSigmaThreshold,
    NoCleanablePixels,
    DivergenceDetected,
}

impl StopReason {
    fn from_code(code: i32) -> StopReason {
        match code {
            sys::CR_STOP_GLOBAL_THRESHOLD => StopReason::GlobalThreshold,
            sys::CR_STOP_CYCLE_THRESHOLD => StopReason::CycleThreshold,
            sys::CR_STOP_NSIGMA_THRESHOLD => StopReason::NSigmaThreshold,
            sys::CR_STOP_NO_CLEANABLE_PIXELS => StopReason::NoCleanablePixels,
            -1 => StopReason::DivergenceDetected,
            _ => StopReason::IterationBudget,
        }
    }
}

/// One device and the stream the library works on.
pub struct Context {
    raw: *mut sys::cr_ctx,
}

// The library serialises calls on one context internally.
unsafe impl Send for Context {}
unsafe impl Sync for Context {}

impl Context {
    pub fn new(device: i32) -> Result<Context> {
        let mut raw = null_mut();
        call(|e| unsafe { sys::cr_ctx_create(device, &mut raw, e) })?;
        Ok(Context { raw })
    }

    pub fn raw(&self) -> *mut sys::cr_ctx {
        self.raw
    }

    /// `DirtyProductFftPolicy.precision` (lib.rs:1280-1312): 64 or 32 bits
    /// for the image-domain transforms of single-plane calls.
    pub fn set_image_fft_precision(&self, bits: i32) -> Result<()> {
        check(unsafe { sys::cr_ctx_set_image_fft_precision(self.raw, bits) }, null_mut())
    }

    /// How the FP64-grade image transforms run: 0 the library's float-pair
    /// kernels where the grid allows, 1 cuFFT FP64.
    pub fn set_image_fft_engine(&self, engine: i32) -> Result<()> {
        check(unsafe { sys::cr_ctx_set_image_fft_engine(self.raw, engine) }, null_mut())
    }

    /// Run the following calls on `stream` (a `cudaStream_t`); null returns
    /// to the context's own non-blocking stream.  The legacy default stream
    /// is passed as `cudaStreamLegacy` (`1 as *mut c_void`).
    ///
    /// # Safety
    /// `stream` must stay a valid stream of this context's device while the
    /// context uses it.
    pub unsafe fn set_stream(&self, stream: *mut c_void) -> Result<()> {
        call(|e| sys::cr_ctx_set_stream(self.raw, stream, e))
    }

    /// The stream the calls run on.
    pub fn stream(&self) -> *mut c_void {
        unsafe { sys::cr_ctx_stream(self.raw) }
    }

    /// Per-call stage timings on (the default) or off; with them off, calls
    /// whose outputs stay on the device return once their work is queued.
    pub fn set_timings(&self, enable: bool) -> Result<()> {
        check(unsafe { sys::cr_ctx_set_timings(self.raw, enable as i32) }, null_mut())
    }

    /// A workspace budget in bytes (0: none), for tests of allocation failure.
    pub fn set_alloc_limit(&self, bytes: i64) -> Result<()> {
        check(unsafe { sys::cr_ctx_set_alloc_limit(self.raw, bytes) }, null_mut())
    }

    /// Poll limits of the bounded device waits, for tests of the timeout
    /// path: 0 gives up at once (the call then fails with
    /// `CudaError::Unsupported`, the `CR_TIMEOUT` mapping), a negative value
    /// restores the default.
    pub fn set_wait_limits(&self, barrier_polls: i64, mbar_polls: i64) -> Result<()> {
        check(unsafe { sys::cr_ctx_set_wait_limits(self.raw, barrier_polls, mbar_polls) },
              null_mut())
    }

    /// Repeated all-device cube calls captured into CUDA graphs (the
    /// default) or run eagerly.
    pub fn set_cube_graphs(&self, enable: bool) -> Result<()> {
        check(unsafe { sys::cr_ctx_set_cube_graphs(self.raw, enable as i32) }, null_mut())
    }

    /// Records per cube gridding work item: 0 lets the tuner choose.
    pub fn set_cube_grid_chunk(&self, chunk: i32) -> Result<()> {
        check(unsafe { sys::cr_ctx_set_cube_grid_chunk(self.raw, chunk) }, null_mut())
    }

    /// Device scratch the context holds, in bytes.
    pub fn workspace_bytes(&self) -> i64 {
        unsafe { sys::cr_ctx_workspace_bytes(self.raw) }
    }

    pub fn synchronize(&self) -> Result<()> {
        call(|e| unsafe { sys::cr_ctx_synchronize(self.raw, e) })
    }

    /// Per-stage device times of the last call (milliseconds).
    pub fn last_timings(&self) -> cr_timings {
        let mut t = cr_timings::default();
        unsafe { sys::cr_ctx_last_timings(self.raw, &mut t) };
        t
    }

    /// Kernels this context has launched.
    pub fn launch_count(&self) -> i64 {
        unsafe { sys::cr_ctx_launch_count(self.raw) }
    }

    pub fn version() -> String {
        unsafe { CStr::from_ptr(sys::cr_version()) }.to_string_lossy().into_owned()
    }
}

impl Drop for Context {
    fn drop(&mut self) {
        unsafe { sys::cr_ctx_destroy(self.raw) };
    }
}

/// `StandardGridder::new` (gridder.rs:371-443) on the device.
pub struct Gridder<'c> {
    ctx: &'c Context,
    raw: *mut sys::cr_gridder,
    pub info: cr_grid_info,
    pub nx: usize,
    pub ny: usize,
}

impl<'c> Gridder<'c> {
    /// `padding` 1.2 and `oversampling` 100 are the reference's defaults.
    pub fn new(ctx: &'c Context, nx: usize, ny: usize, cell_x_rad: f64, cell_y_rad: f64,
               padding: f64, oversampling: i32) -> Result<Gridder<'c>> {
        let geom = sys::cr_geometry { nx: nx as i32, ny: ny as i32, cell_x_rad, cell_y_rad };
        let mut raw = null_mut();
        let mut info = cr_grid_info::default();
        call(|e| unsafe {
            sys::cr_gridder_create(ctx.raw, &geom, padding, oversampling, &mut raw, &mut info, e)
        })?;
        Ok(Gridder { ctx, raw, info, nx, ny })
    }

    pub fn raw(&self) -> *mut sys::cr_gridder {
        self.raw
    }

    pub fn grid_len(&self) -> usize {
        (self.info.grid_nx * self.info.grid_ny) as usize
    }
}

impl Drop for Gridder<'_> {
    fn drop(&mut self) {
        unsafe { sys::cr_gridder_destroy(self.raw) };
    }
}

/// `WProjector::new` (gridder.rs:3403-3586) on the device.
pub struct WProjector<'g> {
    raw: *mut sys::cr_wproj,
    pub info: cr_wproj_info,
    _g: PhantomData<&'g Gridder<'g>>,
}

impl<'g> WProjector<'g> {
    /// `planes` / `sampling` 0 choose the reference's defaults; a support law
    /// of (0, 0) runs the reference's support search.
    pub fn new(g: &'g Gridder<'_>, max_abs_w: f64, planes: i32, sampling: i32,
               support_min: i32, support_max: i32) -> Result<WProjector<'g>> {
        let mut raw = null_mut();
        let mut info = cr_wproj_info::default();
        call(|e| unsafe {
            sys::cr_wproj_create(g.ctx.raw, g.raw, max_abs_w, planes, sampling, support_min,
                                 support_max, &mut raw, &mut info, e)
        })?;
        Ok(WProjector { raw, info, _g: PhantomData })
    }

    pub fn raw(&self) -> *mut sys::cr_wproj {
        self.raw
    }
}

impl Drop for WProjector<'_> {
    fn drop(&mut self) {
        unsafe { sys::cr_wproj_destroy(self.raw) };
    }
}

fn wp_raw(wp: Option<&WProjector<'_>>) -> *mut sys::cr_wproj {
    wp.map_or(null_mut(), |w| w.raw)
}

/// A borrowed `VisibilityBatch` (types.rs:1376-1405): per sample u, v, w in
/// wavelengths, weight, sumwt factor, gridable flag, Complex32 visibility.
#[derive(Clone, Copy)]
pub struct Samples<'a> {
    pub u_lambda: &'a [f64],
    pub v_lambda: &'a [f64],
    /// Empty for the standard gridder.
    pub w_lambda: &'a [f64],
    pub weight: &'a [f32],
    /// Empty means 1 for every sample.
    pub sumwt_factor: &'a [f32],
    /// Empty means every sample is gridable (`bool` is one byte, 0 or 1).
    pub gridable: &'a [bool],
    /// `[re, im]` pairs, the memory of `Complex32`.
    pub visibility: &'a [[f32; 2]],
}

impl<'a> Samples<'a> {
    fn batch(&self) -> Result<sys::cr_vis_batch> {
        let n = self.u_lambda.len();
        want_len("v_lambda", self.v_lambda.len(), n)?;
        want_len("weight", self.weight.len(), n)?;
        want_len("visibility", self.visibility.len(), n)?;
        for (name, len) in [("w_lambda", self.w_lambda.len()),
                            ("sumwt_factor", self.sumwt_factor.len()),
                            ("gridable", self.gridable.len())] {
            if len != 0 {
                want_len(name, len, n)?;
            }
        }
        let opt = |len: usize, p: *const u8| if len == 0 { null() } else { p };
        Ok(sys::cr_vis_batch {
            n: n as i64,
            u: self.u_lambda.as_ptr(),
            v: self.v_lambda.as_ptr(),
            w: opt(self.w_lambda.len(), self.w_lambda.as_ptr() as *const u8) as *const f64,
            weight: self.weight.as_ptr(),
            sumwt_factor: opt(self.sumwt_factor.len(), self.sumwt_factor.as_ptr() as *const u8)
                as *const f32,
            gridable: opt(self.gridable.len(), self.gridable.as_ptr() as *const u8),
            vis: self.visibility.as_ptr() as *const f32,
            location: sys::CR_HOST,
        })
    }
}

/// PSF and residual images with their normalisation state.
pub struct DirtyProducts {
    pub psf: Vec<f32>,
    pub residual: Vec<f32>,
    pub state: cr_psf_state,
    pub sums: cr_sums,
}

/// `compute_dirty_psf_and_residual{,_w_project}` (lib.rs:70390-70458 for
/// W-projection): grid, transform, correct and normalise by the PSF peak.
pub fn dirty_image(g: &Gridder<'_>, wp: Option<&WProjector<'_>>, samples: &Samples<'_>)
                   -> Result<DirtyProducts> {
    let batch = samples.batch()?;
    let n = g.nx * g.ny;
    let mut out = DirtyProducts { psf: vec![0.0; n], residual: vec![0.0; n],
                                  state: cr_psf_state::default(), sums: cr_sums::default() };
    call(|e| unsafe {
        sys::cr_dirty_image(g.ctx.raw, g.raw, wp_raw(wp), &batch, out.psf.as_mut_ptr(),
                            out.residual.as_mut_ptr(), sys::CR_HOST, &mut out.state,
                            &mut out.sums, e)
    })?;
    Ok(out)
}

/// `compute_residual{,_w_project}` (lib.rs:70646-70700 for W-projection):
/// the residual image of `model` under the state of the dirty products.
pub fn residual_image(g: &Gridder<'_>, wp: Option<&WProjector<'_>>, samples: &Samples<'_>,
                      model: &[f32], state: &cr_psf_state) -> Result<Vec<f32>> {
    let batch = samples.batch()?;
    let n = g.nx * g.ny;
    want_len("model", model.len(), n)?;
    let mut residual = vec![0.0f32; n];
    let mut sums = cr_sums::default();
    call(|e| unsafe {
        sys::cr_residual_image(g.ctx.raw, g.raw, wp_raw(wp), &batch, model.as_ptr(),
                               sys::CR_HOST, state, residual.as_mut_ptr(), sys::CR_HOST,
                               &mut sums, e)
    })?;
    Ok(residual)
}

/// A materialised plan: the samples' sorted, deduplicated grid records kept
/// on the device for every residual refresh of one Cotton-Schwab loop.
pub struct Plan<'g> {
    g: &'g Gridder<'g>,
    raw: *mut sys::cr_plan,
    pub sums: cr_sums,
}

impl<'g> Plan<'g> {
    pub fn new(g: &'g Gridder<'g>, wp: Option<&WProjector<'_>>, samples: &Samples<'_>)
               -> Result<Plan<'g>> {
        let batch = samples.batch()?;
        let mut raw = null_mut();
        let mut sums = cr_sums::default();
        call(|e| unsafe {
            sys::cr_plan_create(g.ctx.raw, g.raw, wp_raw(wp), &batch, &mut raw, &mut sums, e)
        })?;
        Ok(Plan { g, raw, sums })
    }

    /// The `refresh_residual` callback of `run_hogbom_cotton_schwab`
    /// (lib.rs:59354-59636).
    pub fn residual_image(&self, model: &[f32], state: &cr_psf_state) -> Result<Vec<f32>> {
        let n = self.g.nx * self.g.ny;
        want_len("model", model.len(), n)?;
        let mut residual = vec![0.0f32; n];
        call(|e| unsafe {
            sys::cr_plan_residual_image(self.g.ctx.raw, self.raw, model.as_ptr(), sys::CR_HOST,
                                        state, residual.as_mut_ptr(), sys::CR_HOST, e)
        })?;
        Ok(residual)
    }
}

impl Drop for Plan<'_> {
    fn drop(&mut self) {
        unsafe { sys::cr_plan_destroy(self.raw) };
    }
}

/// The controls of one Hogbom or multiscale minor cycle
/// (`HogbomMinorCycleControl`-like, lib.rs:59748-59883).
#[derive(Clone, Copy, Debug)]
pub struct MinorCycleControl {
    pub gain: f32,
    pub threshold: f32,
    pub cycle_threshold: f32,
    pub nsigma_threshold: f32,
    pub cycle_niter: i64,
}

/// The components of one minor cycle.
#[derive(Clone, Debug, Default)]
pub struct MinorCycleOutcome {
    pub positions: Vec<[usize; 2]>,
    /// Hogbom: the residual peak; multiscale: the candidate strength.
    pub peaks: Vec<f32>,
    pub fluxes: Vec<f32>,
    /// Multiscale only: the scale index of each component.
    pub scales: Vec<usize>,
    pub actual_updates: i64,
    pub reported_updates: i64,
    pub stop_reason: Option<StopReason>,
}

fn mask_ptr(mask: Option<&[bool]>, n: usize) -> Result<*const u8> {
    match mask {
        None => Ok(null()),
        Some(m) => {
            want_len("mask", m.len(), n)?;
            Ok(m.as_ptr() as *const u8)
        }
    }
}

/// `run_hogbom_minor_cycle` (lib.rs:59748-59883): `model` and `residual`
/// are updated in place.
pub fn hogbom(ctx: &Context, model: &mut [f32], residual: &mut [f32], psf: &[f32],
              mask: Option<&[bool]>, nx: usize, ny: usize, c: &MinorCycleControl)
              -> Result<MinorCycleOutcome> {
    let n = nx * ny;
    want_len("model", model.len(), n)?;
    want_len("residual", residual.len(), n)?;
    want_len("psf", psf.len(), n)?;
    let mp = mask_ptr(mask, n)?;
    let cap = c.cycle_niter.max(1) as usize;
    let (mut cx, mut cy) = (vec![0i32; cap], vec![0i32; cap]);
    let (mut pk, mut fl) = (vec![0f32; cap], vec![0f32; cap]);
    let (mut actual, mut reported, mut stop) = (0i64, 0i64, 0i32);
    call(|e| unsafe {
        sys::cr_hogbom(ctx.raw, model.as_mut_ptr(), residual.as_mut_ptr(), psf.as_ptr(), mp,
                       nx as i32, ny as i32, sys::CR_HOST, c.gain, c.threshold,
                       c.cycle_threshold, c.nsigma_threshold, c.cycle_niter, 0,
                       cx.as_mut_ptr(), cy.as_mut_ptr(), pk.as_mut_ptr(), fl.as_mut_ptr(),
                       &mut actual, &mut reported, &mut stop, e)
    })?;
    let k = actual as usize;
    Ok(MinorCycleOutcome {
        positions: (0..k).map(|i| [cx[i] as usize, cy[i] as usize]).collect(),
        peaks: pk[..k].to_vec(),
        fluxes: fl[..k].to_vec(),
        scales: Vec::new(),
        actual_updates: actual,
        reported_updates: reported,
        stop_reason: if stop == 0 { None } else { Some(StopReason::from_code(stop)) },
    })
}

/// `run_multiscale_cotton_schwab`'s deconvolver state on the device
/// (build_multiscale_state, lib.rs:64172-64230): scale images, PSF cross
/// terms and the residual convolved with every scale.
pub struct Multiscale<'c> {
    _ctx: PhantomData<&'c Context>,
    raw: *mut sys::cr_multiscale,
    nx: usize,
    ny: usize,
}

impl<'c> Multiscale<'c> {
    pub fn new(ctx: &'c Context, psf: &[f32], mask: Option<&[bool]>, nx: usize, ny: usize,
               scales: &[f32], small_scale_bias: f32) -> Result<Multiscale<'c>> {
        want_len("psf", psf.len(), nx * ny)?;
        let mp = mask_ptr(mask, nx * ny)?;
        let mut raw = null_mut();
        call(|e| unsafe {
            sys::cr_multiscale_create(ctx.raw, psf.as_ptr(), mp, nx as i32, ny as i32,
                                      sys::CR_HOST, scales.as_ptr(), scales.len() as i32,
                                      small_scale_bias, &mut raw, e)
        })?;
        Ok(Multiscale { _ctx: PhantomData, raw, nx, ny })
    }

    /// refresh_multiscale_dirty_conv_scales (lib.rs:63261-63267).
    pub fn set_residual(&mut self, residual: &[f32]) -> Result<()> {
        want_len("residual", residual.len(), self.nx * self.ny)?;
        call(|e| unsafe {
            sys::cr_multiscale_set_residual(self.raw, residual.as_ptr(), sys::CR_HOST, e)
        })
    }

    /// The residual convolved with scale 0.
    pub fn residual(&self) -> Result<Vec<f32>> {
        let mut out = vec![0.0f32; self.nx * self.ny];
        call(|e| unsafe {
            sys::cr_multiscale_residual(self.raw, out.as_mut_ptr(), sys::CR_HOST, e)
        })?;
        Ok(out)
    }

    /// (some scale has a candidate, masked peak |residual|).
    pub fn peak(&self) -> Result<(bool, f32)> {
        let (mut has, mut pk) = (0i32, 0f32);
        call(|e| unsafe { sys::cr_multiscale_peak(self.raw, &mut has, &mut pk, e) })?;
        Ok((has != 0, pk))
    }

    /// One multiscale minor cycle (lib.rs:63700-63800); `model` in place.
    pub fn minor_cycle(&mut self, model: &mut [f32], c: &MinorCycleControl)
                       -> Result<MinorCycleOutcome> {
        want_len("model", model.len(), self.nx * self.ny)?;
        let cap = c.cycle_niter.max(1) as usize;
        let (mut cx, mut cy, mut cs) = (vec![0i32; cap], vec![0i32; cap], vec![0i32; cap]);
        let (mut st, mut fl) = (vec![0f32; cap], vec![0f32; cap]);
        let (mut actual, mut reported, mut stop) = (0i64, 0i64, 0i32);
        call(|e| unsafe {
            sys::cr_multiscale_minor_cycle(self.raw, model.as_mut_ptr(), sys::CR_HOST, c.gain,
                                           c.threshold, c.cycle_threshold, c.nsigma_threshold,
                                           c.cycle_niter, cx.as_mut_ptr(), cy.as_mut_ptr(),
                                           cs.as_mut_ptr(), st.as_mut_ptr(), fl.as_mut_ptr(),
                                           &mut actual, &mut reported, &mut stop, e)
        })?;
        let k = actual as usize;
        Ok(MinorCycleOutcome {
            positions: (0..k).map(|i| [cx[i] as usize, cy[i] as usize]).collect(),
            peaks: st[..k].to_vec(),
            fluxes: fl[..k].to_vec(),
            scales: cs[..k].iter().map(|&s| s as usize).collect(),
            actual_updates: actual,
            reported_updates: reported,
            stop_reason: if stop == 0 { None } else { Some(StopReason::from_code(stop)) },
        })
    }
}

impl Drop for Multiscale<'_> {
    fn drop(&mut self) {
        unsafe { sys::cr_multiscale_destroy(self.raw) };
    }
}

/// `robust_rms_jy_per_beam` (lib.rs:74474-74626) of one image: the n-sigma
/// threshold's noise estimate (`nsigma * rms`).
pub fn robust_rms(ctx: &Context, image: &[f32], mask: Option<&[bool]>, nx: usize, ny: usize)
                  -> Result<f32> {
    want_len("image", image.len(), nx * ny)?;
    let mp = mask_ptr(mask, nx * ny)?;
    let (mut rms, mut madfm, mut count) = (0f32, 0f64, 0i64);
    let plane = 0i32;
    call(|e| unsafe {
        sys::cr_robust_rms(ctx.raw, image.as_ptr(), mp, 1, nx as i32, ny as i32, sys::CR_HOST,
                           &plane, 1, &mut rms, &mut madfm, &mut count, e)
    })?;
    Ok(rms)
}

/// `fit_beam_from_psf` (beam.rs:27-103); `None` when no attempt converged.
pub fn fit_beam(ctx: &Context, psf: &[f32], nx: usize, ny: usize, cell_x_rad: f64,
                cell_y_rad: f64, cutoff: f32) -> Result<Option<cr_beam>> {
    want_len("psf", psf.len(), nx * ny)?;
    let mut beam = cr_beam::default();
    let (mut fitted, mut attempts, mut used) = (0i32, 0i32, 0f32);
    call(|e| unsafe {
        sys::cr_fit_beam(ctx.raw, psf.as_ptr(), nx as i32, ny as i32, sys::CR_HOST, cell_x_rad,
                         cell_y_rad, cutoff, &mut beam, &mut fitted, &mut attempts, &mut used, e)
    })?;
    Ok(if fitted != 0 { Some(beam) } else { None })
}

/// `restore_model` (beam.rs:105-120) plus the residual.
pub fn restore(ctx: &Context, model: &[f32], residual: Option<&[f32]>, nx: usize, ny: usize,
               cell_x_rad: f64, cell_y_rad: f64, beam: &cr_beam) -> Result<Vec<f32>> {
    want_len("model", model.len(), nx * ny)?;
    if let Some(r) = residual {
        want_len("residual", r.len(), nx * ny)?;
    }
    let mut out = vec![0.0f32; nx * ny];
    call(|e| unsafe {
        sys::cr_restore(ctx.raw, model.as_ptr(), residual.map_or(null(), |r| r.as_ptr()),
                        nx as i32, ny as i32, sys::CR_HOST, cell_x_rad, cell_y_rad, beam,
                        out.as_mut_ptr(), sys::CR_HOST, e)
    })?;
    Ok(out)
}

/// The device side of `stream_imaging_source_read_ahead_blocks`
/// (casars-imager/src/lib.rs:36608-36760): MeasurementSet row blocks of one
/// spectral window pass through `max_live_row_blocks` page-locked slots;
/// each submitted block is uploaded while the previous one is prepared and
/// gridded by the feed's worker thread.  The reader (casa-ms) writes a
/// block's columns straight into the slot `acquire` hands out.  The context
/// belongs to the feed until `finish` returns.
pub struct RowFeed<'g> {
    g: &'g Gridder<'g>,
    raw: *mut sys::cr_row_feed,
    channels: usize,
    correlations: usize,
}

/// One acquired staging slot: page-locked arrays of `max_rows` rows in the
/// row-run layout (`[row][channel][correlation]`, DATA as `f32` pairs).
pub struct RowBlockSlot<'f> {
    raw: sys::cr_row_block,
    channels: usize,
    correlations: usize,
    _feed: PhantomData<&'f ()>,
}

impl RowBlockSlot<'_> {
    pub fn max_rows(&self) -> usize {
        self.raw.max_rows as usize
    }

    fn slice<'a, T>(p: *mut T, n: usize) -> Option<&'a mut [T]> {
        // SAFETY: the slot's arrays hold max_rows rows, stay allocated while
        // the feed lives, and belong to this slot until it is submitted.
        if p.is_null() { None } else { Some(unsafe { std::slice::from_raw_parts_mut(p, n) }) }
    }

    pub fn uvw_m(&mut self) -> &mut [f64] {
        Self::slice(self.raw.uvw_m, self.max_rows() * 3).unwrap()
    }
    pub fn data(&mut self) -> &mut [f32] {
        Self::slice(self.raw.data, self.max_rows() * self.channels * self.correlations * 2).unwrap()
    }
    pub fn weight(&mut self) -> &mut [f32] {
        Self::slice(self.raw.weight, self.max_rows() * self.correlations).unwrap()
    }
    pub fn flag(&mut self) -> Option<&mut [u8]> {
        Self::slice(self.raw.flag, self.max_rows() * self.channels * self.correlations)
    }
    pub fn weight_spectrum(&mut self) -> Option<&mut [f32]> {
        Self::slice(self.raw.weight_spectrum, self.max_rows() * self.channels * self.correlations)
    }
    pub fn gridable(&mut self) -> Option<&mut [u8]> {
        Self::slice(self.raw.gridable, self.max_rows())
    }
}

impl<'g> RowFeed<'g> {
    #[allow(clippy::too_many_arguments)]
    pub fn new(g: &'g Gridder<'g>, lambda_scale: &[f64], polarization: sys::cr_polarization,
               correlations: usize, row_block_rows: usize, max_live_row_blocks: i32,
               has_flag: bool, has_weight_spectrum: bool, has_gridable: bool)
               -> Result<RowFeed<'g>> {
        let cfg = sys::cr_row_feed_config {
            max_live_row_blocks, row_block_rows: row_block_rows as i64,
            channels: lambda_scale.len() as i32, correlations: correlations as i32,
            lambda_scale: lambda_scale.as_ptr(), polarization,
            has_flag: has_flag as i32, has_weight_spectrum: has_weight_spectrum as i32,
            has_gridable: has_gridable as i32,
        };
        let mut raw = null_mut();
        call(|e| unsafe { sys::cr_row_feed_create(g.ctx.raw, g.raw, &cfg, &mut raw, e) })?;
        Ok(RowFeed { g, raw, channels: lambda_scale.len(), correlations })
    }

    /// The next free slot; waits while every slot is live.
    pub fn acquire(&self) -> Result<RowBlockSlot<'_>> {
        // SAFETY: plain-old-data out parameter, filled by the call.
        let mut blk: sys::cr_row_block = unsafe { std::mem::zeroed() };
        call(|e| unsafe { sys::cr_row_feed_acquire(self.raw, &mut blk, e) })?;
        Ok(RowBlockSlot { raw: blk, channels: self.channels, correlations: self.correlations,
                          _feed: PhantomData })
    }

    /// Queue the slot's first `rows` rows (0 hands the slot back unused).
    pub fn submit(&self, slot: RowBlockSlot<'_>, rows: usize) -> Result<()> {
        call(|e| unsafe { sys::cr_row_feed_submit(self.raw, slot.raw.slot, rows as i64, e) })
    }

    /// Images of every block submitted so far, and the read-ahead summary
    /// (`ImagingSourceReadAheadSummary`, lib.rs:36324-36335).
    pub fn finish(&self) -> Result<(DirtyProducts, sys::cr_row_feed_summary)> {
        let n = self.g.nx * self.g.ny;
        let mut out = DirtyProducts { psf: vec![0.0; n], residual: vec![0.0; n],
                                      state: cr_psf_state::default(), sums: cr_sums::default() };
        let mut summary = sys::cr_row_feed_summary::default();
        call(|e| unsafe {
            sys::cr_row_feed_finish(self.raw, out.psf.as_mut_ptr(), out.residual.as_mut_ptr(),
                                    sys::CR_HOST, &mut out.state, &mut out.sums, &mut summary, e)
        })?;
        Ok((out, summary))
    }
}

impl Drop for RowFeed<'_> {
    fn drop(&mut self) {
        unsafe { sys::cr_row_feed_destroy(self.raw) };
    }
}
