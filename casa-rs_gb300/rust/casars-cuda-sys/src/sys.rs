// Raw declarations of include/casars_cuda.h, written by gen_sys.py; do not edit.
#![allow(non_camel_case_types)]

use std::os::raw::{c_char, c_int, c_void};

pub const CR_OK: i32 = 0;
pub const CR_INVALID: i32 = 1;
pub const CR_NO_SAMPLES: i32 = 2;
pub const CR_BUFFER_SMALL: i32 = 3;
pub const CR_CUDA: i32 = 4;
pub const CR_NORMALIZATION: i32 = 5;
pub const CR_TIMEOUT: i32 = 6;
pub const CR_HOST: i32 = 0;
pub const CR_DEVICE: i32 = 1;
pub const CR_WEIGHT_NATURAL: i32 = 0;
pub const CR_WEIGHT_UNIFORM: i32 = 1;
pub const CR_WEIGHT_BRIGGS: i32 = 2;
pub const CR_STOP_NONE: i32 = 0;
pub const CR_STOP_GLOBAL_THRESHOLD: i32 = 1;
pub const CR_STOP_CYCLE_THRESHOLD: i32 = 2;
pub const CR_STOP_NSIGMA_THRESHOLD: i32 = 3;
pub const CR_STOP_NO_CLEANABLE_PIXELS: i32 = 4;

#[repr(C)]
pub struct cr_ctx {
    _private: [u8; 0],
}

#[repr(C)]
pub struct cr_gridder {
    _private: [u8; 0],
}

#[repr(C)]
pub struct cr_wproj {
    _private: [u8; 0],
}

#[repr(C)]
pub struct cr_plan {
    _private: [u8; 0],
}

#[repr(C)]
pub struct cr_cube_plan {
    _private: [u8; 0],
}

#[repr(C)]
pub struct cr_accumulator {
    _private: [u8; 0],
}

#[repr(C)]
pub struct cr_multiscale {
    _private: [u8; 0],
}

#[repr(C)]
pub struct cr_row_feed {
    _private: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cr_geometry {
    pub nx: i32,
    pub ny: i32,
    pub cell_x_rad: f64,
    pub cell_y_rad: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cr_grid_info {
    pub grid_nx: i64,
    pub grid_ny: i64,
    pub blc_x: i64,
    pub blc_y: i64,
    pub du: f64,
    pub dv: f64,
    pub oversampling: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cr_wproj_info {
    pub planes: i32,
    pub sampling: i32,
    pub w_scale: f64,
    pub max_support: i32,
    pub kernel_width: i32,
    pub cube_elements: i64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct cr_vis_batch {
    pub n: i64,
    pub u: *const f64,
    pub v: *const f64,
    pub w: *const f64,
    pub weight: *const f32,
    pub sumwt_factor: *const f32,
    pub gridable: *const u8,
    pub vis: *const f32,
    pub location: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct cr_row_runs {
    pub rows: i64,
    pub channels: i32,
    pub correlations: i32,
    pub uvw_m: *const f64,
    pub lambda_scale: *const f64,
    pub data: *const f32,
    pub flag: *const u8,
    pub weight: *const f32,
    pub weight_spectrum: *const f32,
    pub gridable: *const u8,
    pub location: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cr_polarization {
    pub mode: i32,
    pub corr0: i32,
    pub corr1: i32,
    pub transform: i32,
    pub sumwt_factor: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cr_sums {
    pub normalization_sumwt: f64,
    pub reported_sumwt: f64,
    pub gridded: i64,
    pub skipped: i64,
    pub unique_records: i64,
    pub taps: i64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cr_psf_state {
    pub psf_peak: f32,
    pub normalization_sumwt: f32,
    pub reported_sumwt: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cr_timings {
    pub plan_ms: f32,
    pub grid_ms: f32,
    pub degrid_ms: f32,
    pub fft_ms: f32,
    pub other_ms: f32,
    pub grid_kernel_ms: f32,
    pub degrid_kernel_ms: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct cr_cube_batch {
    pub rows: i64,
    pub channels: i32,
    pub u_m: *const f64,
    pub v_m: *const f64,
    pub lambda_scale: *const f64,
    pub vis: *const f32,
    pub weight: *const f32,
    pub flags: *const u8,
    pub location: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct cr_row_feed_config {
    pub max_live_row_blocks: i32,
    pub row_block_rows: i64,
    pub channels: i32,
    pub correlations: i32,
    pub lambda_scale: *const f64,
    pub polarization: cr_polarization,
    pub has_flag: i32,
    pub has_weight_spectrum: i32,
    pub has_gridable: i32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct cr_row_block {
    pub slot: i32,
    pub max_rows: i64,
    pub uvw_m: *mut f64,
    pub data: *mut f32,
    pub flag: *mut u8,
    pub weight: *mut f32,
    pub weight_spectrum: *mut f32,
    pub gridable: *mut u8,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cr_row_feed_summary {
    pub row_blocks: i64,
    pub streamed_samples: i64,
    pub source_bytes: i64,
    pub live_row_block_high_water: i32,
    pub producer_send_blocked_s: f64,
    pub consumer_recv_blocked_s: f64,
    pub consumer_elapsed_s: f64,
    pub producer_consumer_overlap_s: f64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct cr_beam {
    pub major_fwhm_rad: f64,
    pub minor_fwhm_rad: f64,
    pub position_angle_rad: f64,
}

#[link(name = "casars_cuda")]
extern "C" {
    pub fn cr_ctx_create(device: i32, out: *mut *mut cr_ctx, err: *mut *mut c_char) -> c_int;
    pub fn cr_ctx_destroy(ctx: *mut cr_ctx);
    pub fn cr_free_error(err: *mut c_char);
    pub fn cr_ctx_set_stream(ctx: *mut cr_ctx, stream: *mut c_void, err: *mut *mut c_char) -> c_int;
    pub fn cr_ctx_stream(ctx: *mut cr_ctx) -> *mut c_void;
    pub fn cr_ctx_synchronize(ctx: *mut cr_ctx, err: *mut *mut c_char) -> c_int;
    pub fn cr_ctx_last_timings(ctx: *mut cr_ctx, out: *mut cr_timings) -> c_int;
    pub fn cr_ctx_launch_count(ctx: *mut cr_ctx) -> i64;
    pub fn cr_ctx_workspace_bytes(ctx: *mut cr_ctx) -> i64;
    pub fn cr_ctx_set_wait_limits(ctx: *mut cr_ctx, barrier_polls: i64, mbar_polls: i64) -> c_int;
    pub fn cr_ctx_set_image_fft_precision(ctx: *mut cr_ctx, bits: i32) -> c_int;
    pub fn cr_ctx_set_image_fft_engine(ctx: *mut cr_ctx, engine: i32) -> c_int;
    pub fn cr_ctx_set_alloc_limit(ctx: *mut cr_ctx, bytes: i64) -> c_int;
    pub fn cr_ctx_set_timings(ctx: *mut cr_ctx, enable: i32) -> c_int;
    pub fn cr_version() -> *const c_char;
    pub fn cr_gridder_create(ctx: *mut cr_ctx, geom: *const cr_geometry, padding: f64, oversampling: i32, out: *mut *mut cr_gridder, info: *mut cr_grid_info, err: *mut *mut c_char) -> c_int;
    pub fn cr_gridder_destroy(g: *mut cr_gridder);
    pub fn cr_gridder_tables(g: *mut cr_gridder, taps: *mut f32, corr_x: *mut f32, corr_y: *mut f32, err: *mut *mut c_char) -> c_int;
    pub fn cr_wproj_create(ctx: *mut cr_ctx, g: *mut cr_gridder, max_abs_w: f64, planes: i32, sampling: i32, support_min: i32, support_max: i32, out: *mut *mut cr_wproj, info: *mut cr_wproj_info, err: *mut *mut c_char) -> c_int;
    pub fn cr_wproj_destroy(wp: *mut cr_wproj);
    pub fn cr_wproj_tables(wp: *mut cr_wproj, support: *mut i32, kernels: *mut f32, norm: *mut f32, err: *mut *mut c_char) -> c_int;
    pub fn cr_grid_dirty(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, batch: *const cr_vis_batch, psf_grid: *mut f32, dirty_grid: *mut f32, out_location: i32, sums: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_degrid(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, batch: *const cr_vis_batch, model_grid: *const f32, grid_location: i32, pred: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_grid_residual(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, batch: *const cr_vis_batch, model_grid: *const f32, grid_location: i32, residual_grid: *mut f32, out_location: i32, sums: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_plan_create(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, batch: *const cr_vis_batch, out: *mut *mut cr_plan, sums: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_plan_destroy(plan: *mut cr_plan);
    pub fn cr_plan_grid_dirty(ctx: *mut cr_ctx, plan: *mut cr_plan, psf_grid: *mut f32, dirty_grid: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_plan_degrid(ctx: *mut cr_ctx, plan: *mut cr_plan, model_grid: *const f32, grid_location: i32, pred: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_plan_grid_residual(ctx: *mut cr_ctx, plan: *mut cr_plan, model_grid: *const f32, grid_location: i32, residual_grid: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_plan_residual_image(ctx: *mut cr_ctx, plan: *mut cr_plan, model: *const f32, model_location: i32, state: *const cr_psf_state, residual_out: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_grid_to_image(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, grid: *const f32, grid_location: i32, scale: f32, image: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_image_to_grid(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, model: *const f32, model_location: i32, grid: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_dirty_image(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, batch: *const cr_vis_batch, psf: *mut f32, residual: *mut f32, out_location: i32, state: *mut cr_psf_state, sums: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_residual_image(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, batch: *const cr_vis_batch, model: *const f32, model_location: i32, state: *const cr_psf_state, residual: *mut f32, out_location: i32, sums: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_predict(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, batch: *const cr_vis_batch, model: *const f32, model_location: i32, pred: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_adjoint(ctx: *mut cr_ctx, g: *mut cr_gridder, wp: *mut cr_wproj, batch: *const cr_vis_batch, image: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_accumulator_create(ctx: *mut cr_ctx, g: *mut cr_gridder, out: *mut *mut cr_accumulator, err: *mut *mut c_char) -> c_int;
    pub fn cr_accumulator_destroy(acc: *mut cr_accumulator);
    pub fn cr_accumulator_add(ctx: *mut cr_ctx, acc: *mut cr_accumulator, batch: *const cr_vis_batch, batch_sums: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_accumulator_finish(ctx: *mut cr_ctx, acc: *mut cr_accumulator, psf: *mut f32, residual: *mut f32, out_location: i32, state: *mut cr_psf_state, total: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_ctx_set_cube_graphs(ctx: *mut cr_ctx, enable: i32) -> c_int;
    pub fn cr_ctx_set_cube_grid_chunk(ctx: *mut cr_ctx, chunk: i32) -> c_int;
    pub fn cr_cube_grid_dirty(ctx: *mut cr_ctx, g: *mut cr_gridder, batch: *const cr_cube_batch, weighting: i32, robust: f32, psf_grids: *mut f32, dirty_grids: *mut f32, out_location: i32, sums: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_cube_degrid(ctx: *mut cr_ctx, g: *mut cr_gridder, batch: *const cr_cube_batch, weighting: i32, robust: f32, model_grids: *const f32, grid_location: i32, pred: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_cube_grid_degrid(ctx: *mut cr_ctx, g: *mut cr_gridder, batch: *const cr_cube_batch, weighting: i32, robust: f32, psf_grids: *mut f32, dirty_grids: *mut f32, model_grids: *const f32, grid_location: i32, pred: *mut f32, out_location: i32, sums: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_cube_sample_taps(ctx: *mut cr_ctx, g: *mut cr_gridder, batch: *const cr_cube_batch, weighting: i32, robust: f32, start_x: *mut i32, start_y: *mut i32, row_x: *mut i32, row_y: *mut i32, imaging_weight: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_cube_plan_create(ctx: *mut cr_ctx, g: *mut cr_gridder, batch: *const cr_cube_batch, weighting: i32, robust: f32, out: *mut *mut cr_cube_plan, sums: *mut cr_sums, err: *mut *mut c_char) -> c_int;
    pub fn cr_cube_plan_destroy(plan: *mut cr_cube_plan);
    pub fn cr_cube_plan_channels(plan: *const cr_cube_plan) -> i32;
    pub fn cr_cube_plan_set_fft_precision(plan: *mut cr_cube_plan, bits: i32) -> c_int;
    pub fn cr_cube_plan_grid_dirty(ctx: *mut cr_ctx, plan: *mut cr_cube_plan, psf_grids: *mut f32, dirty_grids: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_cube_plan_degrid(ctx: *mut cr_ctx, plan: *mut cr_cube_plan, model_grids: *const f32, grid_location: i32, pred: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_cube_plan_grid_residual(ctx: *mut cr_ctx, plan: *mut cr_cube_plan, model_grids: *const f32, grid_location: i32, planes: *const u8, residual_grids: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_cube_plan_dirty_images(ctx: *mut cr_ctx, plan: *mut cr_cube_plan, psf_images: *mut f32, residual_images: *mut f32, out_location: i32, states: *mut cr_psf_state, err: *mut *mut c_char) -> c_int;
    pub fn cr_cube_plan_residual_images(ctx: *mut cr_ctx, plan: *mut cr_cube_plan, models: *const f32, model_location: i32, planes: *const u8, states: *const cr_psf_state, residual_images: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_row_runs_prepare(ctx: *mut cr_ctx, runs: *const cr_row_runs, pol: *const cr_polarization, u: *mut f64, v: *mut f64, w: *mut f64, weight: *mut f32, sumwt_factor: *mut f32, gridable: *mut u8, vis: *mut f32, density_u: *mut f64, density_v: *mut f64, out_location: i32, n_out: *mut i64, err: *mut *mut c_char) -> c_int;
    pub fn cr_polarization_for_plane(plane: i32, corr_types: *const i32, correlations: i32, out: *mut cr_polarization, err: *mut *mut c_char) -> c_int;
    pub fn cr_apply_weighting_rows(ctx: *mut cr_ctx, g: *mut cr_gridder, batch: *const cr_vis_batch, density_u: *const f64, density_v: *const f64, mode: i32, robust: f32, out_weight: *mut f32, out_location: i32, f2: *mut f32, err: *mut *mut c_char) -> c_int;
    pub fn cr_row_feed_create(ctx: *mut cr_ctx, g: *mut cr_gridder, config: *const cr_row_feed_config, out: *mut *mut cr_row_feed, err: *mut *mut c_char) -> c_int;
    pub fn cr_row_feed_destroy(feed: *mut cr_row_feed);
    pub fn cr_row_feed_acquire(feed: *mut cr_row_feed, block: *mut cr_row_block, err: *mut *mut c_char) -> c_int;
    pub fn cr_row_feed_submit(feed: *mut cr_row_feed, slot: i32, rows: i64, err: *mut *mut c_char) -> c_int;
    pub fn cr_row_feed_finish(feed: *mut cr_row_feed, psf: *mut f32, residual: *mut f32, out_location: i32, state: *mut cr_psf_state, total: *mut cr_sums, summary: *mut cr_row_feed_summary, err: *mut *mut c_char) -> c_int;
    pub fn cr_fit_beam(ctx: *mut cr_ctx, psf: *const f32, nx: i32, ny: i32, location: i32, cell_x_rad: f64, cell_y_rad: f64, cutoff: f32, beam: *mut cr_beam, fitted: *mut i32, attempts: *mut i32, cutoff_used: *mut f32, err: *mut *mut c_char) -> c_int;
    pub fn cr_restore(ctx: *mut cr_ctx, model: *const f32, residual: *const f32, nx: i32, ny: i32, location: i32, cell_x_rad: f64, cell_y_rad: f64, beam: *const cr_beam, restored: *mut f32, out_location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_psf_sidelobe(ctx: *mut cr_ctx, psf: *const f32, nx: i32, ny: i32, location: i32, cell_x_rad: f64, cell_y_rad: f64, beam: *const cr_beam, level: *mut f32, err: *mut *mut c_char) -> c_int;
    pub fn cr_apply_weighting(ctx: *mut cr_ctx, g: *mut cr_gridder, batch: *const cr_vis_batch, mode: i32, robust: f32, out_weight: *mut f32, out_location: i32, f2: *mut f32, err: *mut *mut c_char) -> c_int;
    pub fn cr_apply_weighting_plane(ctx: *mut cr_ctx, g: *mut cr_gridder, batch: *const cr_vis_batch, mode: i32, robust: f32, out_weight: *mut f32, out_location: i32, f2: *mut f32, err: *mut *mut c_char) -> c_int;
    pub fn cr_hogbom(ctx: *mut cr_ctx, model: *mut f32, residual: *mut f32, psf: *const f32, mask: *const u8, nx: i32, ny: i32, location: i32, gain: f32, threshold: f32, cycle_threshold: f32, nsigma_threshold: f32, cycle_niter: i64, inclusive: i32, comp_x: *mut i32, comp_y: *mut i32, comp_peak: *mut f32, comp_flux: *mut f32, actual: *mut i64, reported: *mut i64, stop_reason: *mut i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_hogbom_plane(ctx: *mut cr_ctx, model: *mut f32, residual: *mut f32, psf: *const f32, mask: *const u8, nx: i32, ny: i32, location: i32, gain: f32, threshold: f32, cycle_threshold: f32, peak_relative_tolerance: f32, cycle_limit: i64, inclusive: i32, comp_x: *mut i32, comp_y: *mut i32, comp_peak: *mut f32, comp_flux: *mut f32, actual: *mut i64, reported: *mut i64, err: *mut *mut c_char) -> c_int;
    pub fn cr_hogbom_planes(ctx: *mut cr_ctx, model: *mut f32, residual: *mut f32, psf: *const f32, mask: *const u8, nplanes: i32, nx: i32, ny: i32, planes: *const i32, n: i32, gain: f32, threshold: f32, cycle_threshold: f32, nsigma_threshold: f32, nsigma_thresholds: *const f32, cycle_niter: i64, inclusive: i32, comp_x: *mut i32, comp_y: *mut i32, comp_peak: *mut f32, comp_flux: *mut f32, actual: *mut i64, reported: *mut i64, stop_reason: *mut i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_clark(ctx: *mut cr_ctx, model: *mut f32, residual: *mut f32, psf: *const f32, mask: *const u8, nx: i32, ny: i32, location: i32, ncent: i32, gain: f32, threshold: f32, cycle_threshold: f32, nsigma_threshold: f32, cycle_niter: i64, comp_x: *mut i32, comp_y: *mut i32, comp_peak: *mut f32, comp_flux: *mut f32, actual: *mut i64, stop_reason: *mut i32, max_exterior_abs: *mut f32, err: *mut *mut c_char) -> c_int;
    pub fn cr_multiscale_create(ctx: *mut cr_ctx, psf: *const f32, mask: *const u8, nx: i32, ny: i32, location: i32, scales: *const f32, nscales: i32, small_scale_bias: f32, out: *mut *mut cr_multiscale, err: *mut *mut c_char) -> c_int;
    pub fn cr_multiscale_destroy(ms: *mut cr_multiscale);
    pub fn cr_multiscale_set_residual(ms: *mut cr_multiscale, residual: *const f32, location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_multiscale_residual(ms: *mut cr_multiscale, out: *mut f32, location: i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_multiscale_peak(ms: *mut cr_multiscale, has_candidate: *mut i32, peak0: *mut f32, err: *mut *mut c_char) -> c_int;
    pub fn cr_multiscale_minor_cycle(ms: *mut cr_multiscale, model: *mut f32, location: i32, gain: f32, threshold: f32, cycle_threshold: f32, nsigma_threshold: f32, cycle_niter: i64, comp_x: *mut i32, comp_y: *mut i32, comp_scale: *mut i32, comp_strength: *mut f32, comp_flux: *mut f32, actual: *mut i64, reported: *mut i64, stop_reason: *mut i32, err: *mut *mut c_char) -> c_int;
    pub fn cr_robust_rms(ctx: *mut cr_ctx, images: *const f32, masks: *const u8, nimages: i32, nx: i32, ny: i32, location: i32, planes: *const i32, nplanes: i32, rms: *mut f32, madfm: *mut f64, counts: *mut i64, err: *mut *mut c_char) -> c_int;
    pub fn cr_probe_tap_rate(ctx: *mut cr_ctx, buffer_bytes: i64, iters: i32, taps_per_second: *mut f64, taps: *mut f64, err: *mut *mut c_char) -> c_int;
    pub fn cr_hogbom_noalloc(ctx: *mut cr_ctx, model: *mut f32, residual: *mut f32, psf: *const f32, mask: *const u8, nx: i32, ny: i32, gain: f32, threshold: f32, cycle_threshold: f32, nsigma_threshold: f32, cycle_niter: i64, inclusive: i32, comp_x: *mut i32, comp_y: *mut i32, comp_peak: *mut f32, comp_flux: *mut f32, actual: *mut i64, reported: *mut i64, stop_reason: *mut i32, err: *mut *mut c_char) -> c_int;
}
