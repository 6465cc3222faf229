/*
 * casars_cuda.h -- C ABI of the GB300 (sm_103a) imaging hot path.
 *
 * One shared library, libcasars_cuda.so, that a casa-imaging host (the Rust
 * crate, Python through ctypes, or C++) calls at the seams where casa-imaging
 * selects a backend today.  Each entry point names the reference function or
 * seam it replaces (paths relative to the casa-rs repository;
 * `lib.rs` = crates/casa-imaging/src/lib.rs, `gridder.rs`, `weighting.rs`,
 * `fft.rs` likewise).
 *
 * Conventions (the reference's, gridder_interop.rs:40-80 and
 * casacore_cpp_gridder_shim.cpp:24-121):
 *   - every call returns int status: CR_OK (0) or an error code; on error a
 *     heap string is stored in *err (if err is non-NULL) and must be released
 *     with cr_free_error();
 *   - arrays are x-major: grids flat = x * grid_ny + y, images flat =
 *     x * ny + y; complex values are interleaved (re, im) float32;
 *   - caller-owned buffers are host or device memory as the call's
 *     `location` argument says (CR_HOST / CR_DEVICE); the library owns its
 *     device workspaces, which live in the context;
 *   - a context is one CUDA stream; calls on one context are serialised by
 *     the caller; distinct contexts may be used from distinct threads.
 */
#ifndef CASARS_CUDA_H
#define CASARS_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes: 1-3 as the reference's C shims, 4-6 added for the device */
#define CR_OK 0
#define CR_INVALID 1          /* invalid arguments (ImagingError::InvalidRequest) */
#define CR_NO_SAMPLES 2       /* no usable samples (ImagingError::NoUsableSamples) */
#define CR_BUFFER_SMALL 3     /* a caller buffer is too small */
#define CR_CUDA 4             /* CUDA runtime / cuFFT failure */
#define CR_NORMALIZATION 5    /* zero or non-finite peak (ImagingError::Normalization) */
#define CR_TIMEOUT 6          /* a device-side bounded wait gave up */

#define CR_HOST 0
#define CR_DEVICE 1

/* weighting modes (types.rs:145-180) */
#define CR_WEIGHT_NATURAL 0
#define CR_WEIGHT_UNIFORM 1
#define CR_WEIGHT_BRIGGS 2

/* Hogbom stop reasons (CleanStopReason, lib.rs:74653-74676) */
#define CR_STOP_NONE 0
#define CR_STOP_GLOBAL_THRESHOLD 1
#define CR_STOP_CYCLE_THRESHOLD 2
#define CR_STOP_NSIGMA_THRESHOLD 3
#define CR_STOP_NO_CLEANABLE_PIXELS 4

typedef struct cr_ctx cr_ctx;
typedef struct cr_gridder cr_gridder;
typedef struct cr_wproj cr_wproj;
typedef struct cr_plan cr_plan;
typedef struct cr_cube_plan cr_cube_plan;
typedef struct cr_accumulator cr_accumulator;
typedef struct cr_multiscale cr_multiscale;

/* ImageGeometry (types.rs:885-930). */
typedef struct {
    int32_t nx, ny;
    double cell_x_rad, cell_y_rad;
} cr_geometry;

/* Grid shape chosen by casa_composite_padded_len (gridder.rs:371-443). */
typedef struct {
    int64_t grid_nx, grid_ny;
    int64_t blc_x, blc_y;
    double du, dv;            /* grid spacing in wavelengths */
    int32_t oversampling;
} cr_grid_info;

/* WProjector summary (gridder.rs:3391-3586). */
typedef struct {
    int32_t planes;
    int32_t sampling;
    double w_scale;
    int32_t max_support;
    int32_t kernel_width;     /* common cropped width */
    int64_t cube_elements;    /* complex elements of the per-plane residue cubes */
} cr_wproj_info;

/* VisibilityBatch (types.rs:1376-1405), structure of arrays.
 * w may be NULL for the standard gridder; sumwt_factor NULL means 1;
 * gridable NULL means every sample is gridable. */
typedef struct {
    int64_t n;
    const double* u;
    const double* v;
    const double* w;
    const float* weight;
    const float* sumwt_factor;
    const uint8_t* gridable;
    const float* vis;         /* complex64 interleaved */
    int32_t location;         /* CR_HOST or CR_DEVICE */
} cr_vis_batch;

/* Row-shaped visibilities (StandardMfsVisibilityRow, types.rs:1639-1662):
 * per row its uvw in metres and [channels][correlations] DATA, FLAG and
 * (optional) WEIGHT_SPECTRUM, plus [correlations] WEIGHT and an optional
 * per-row gridable flag.  lambda_scale[c] = channel frequency / c is host
 * memory; the other arrays are at `location`.  Arrays are row-major:
 * data[(row * channels + channel) * correlations + corr]. */
typedef struct {
    int64_t rows;
    int32_t channels;
    int32_t correlations;
    const double* uvw_m;            /* [rows][3] */
    const double* lambda_scale;     /* host [channels] */
    const float* data;              /* complex64 [rows][channels][correlations] */
    const uint8_t* flag;            /* [rows][channels][correlations] or NULL */
    const float* weight;            /* [rows][correlations] (unused with a spectrum) */
    const float* weight_spectrum;   /* [rows][channels][correlations] or NULL */
    const uint8_t* gridable;        /* [rows] or NULL */
    int32_t location;
} cr_row_runs;

/* StandardMfsVisibilityPolarization (types.rs:1612-1632): mode 0 = one
 * explicit correlation corr0; mode 1 = the pair (corr0, corr1) collapsed by
 * `transform` (StandardMfsPairCollapseTransform, types.rs:1582-1608): 0 half
 * sum, 1 half difference, 2 (a - b) * (0, 1/2), 3 (a - b) * (0, -1/2). */
typedef struct {
    int32_t mode;
    int32_t corr0, corr1;
    int32_t transform;
    float sumwt_factor;
} cr_polarization;

/* WProjectGridAccumulation / DirtyGridAccumulation (lib.rs:70973-70988). */
typedef struct {
    double normalization_sumwt;
    double reported_sumwt;
    int64_t gridded;
    int64_t skipped;
    int64_t unique_records;   /* distinct (cell, offset, plane, sign) keys gridded */
    int64_t taps;             /* kernel taps one grid pass applies: sum over records of the
                                 footprint (2S+1)^2 (49 for the standard gridder) */
} cr_sums;

/* PsfState essentials (lib.rs:64680-64690). */
typedef struct {
    float psf_peak;
    float normalization_sumwt;
    float reported_sumwt;
} cr_psf_state;

/* Per-stage device times of the last call, milliseconds (CUDA events);
 * grid_kernel_ms / degrid_kernel_ms bracket the gridding / degridding kernel
 * launch alone (0 when the call launched none). */
typedef struct {
    float plan_ms, grid_ms, degrid_ms, fft_ms, other_ms;
    float grid_kernel_ms, degrid_kernel_ms;
} cr_timings;

/* ---- context -------------------------------------------------------------
 * New; the reference has no device context.  Thread-safe per context.      */
int cr_ctx_create(int32_t device, cr_ctx** out, char** err);
void cr_ctx_destroy(cr_ctx* ctx);
void cr_free_error(char* err);
/* Use an external cudaStream_t (e.g. torch's current stream); NULL restores
 * the context's own stream (non-blocking: not ordered with the legacy
 * default stream).  To run on the legacy default stream (torch's default
 * stream, whose handle is 0) pass cudaStreamLegacy ((void*)1). */
int cr_ctx_set_stream(cr_ctx* ctx, void* stream, char** err);
void* cr_ctx_stream(cr_ctx* ctx);
int cr_ctx_synchronize(cr_ctx* ctx, char** err);
int cr_ctx_last_timings(cr_ctx* ctx, cr_timings* out);
/* Number of this library's kernel launches since the context was created. */
int64_t cr_ctx_launch_count(cr_ctx* ctx);
/* Bytes of device workspace the context holds (its grow-only buffers). */
int64_t cr_ctx_workspace_bytes(cr_ctx* ctx);
/* Bounds of the device-side waits, for tests of the timeout paths.  The
 * reference has no device waits; its counterpart is the error taxonomy of
 * ImagingError (crates/casa-imaging/src/error.rs:7-24).  barrier_polls bounds
 * each wait of the Hogbom grid barrier (polls ~64 ns apart; default 2^24,
 * about a second), mbar_polls the first wait on each bulk copy of the cube
 * kernels (default 2^22 polls).  0 gives up at once: a call whose wait gives
 * up returns CR_TIMEOUT and leaves its outputs undefined; the context stays
 * usable.  A negative value restores the default.  Waits that let a block's
 * copies in flight land after a timeout always keep the default bound.
 * Changing a limit retires the context's captured cube pipelines. */
int cr_ctx_set_wait_limits(cr_ctx* ctx, int64_t barrier_polls, int64_t mbar_polls);
/* Precision of the image-stage FFTs (grid correction, fftshift, 2-D FFT) of
 * the single-plane calls: 0 (Auto) or 64 = FP64, the default; 32 = FP32.
 * Replaces the precision field of DirtyProductFftPolicy
 * (crates/casa-imaging/src/lib.rs:1280-1312; FftPrecisionChoice at
 * crates/casa-imaging/src/fft_backend.rs:61-68). Cube plans carry their own
 * setting (cr_cube_plan_set_fft_precision). */
int cr_ctx_set_image_fft_precision(cr_ctx* ctx, int32_t bits);
/* How the FP64-grade image transforms of the single-plane calls run:
 * 0 (the default) = float-pair kernels (values as a sum of two floats, about
 * 48 significant bits, on the float32 pipes) for grids whose sides are even,
 * 5-smooth and at most 13824, cuFFT FP64 otherwise; 1 = always cuFFT FP64.
 * New; no counterpart in the reference (whose host FFT has no such
 * choice).  Returns CR_INVALID for other values. */
int cr_ctx_set_image_fft_engine(cr_ctx* ctx, int32_t engine);
/* For tests of the failure paths: a budget in bytes for the context's
 * workspaces (0, the default, lifts it).  A call that would grow them past
 * the budget fails with CR_CUDA, as a failed device allocation does, before
 * any work; the context stays usable.  New; no counterpart in the reference
 * (its allocation failures come from the host allocator).  CR_INVALID for a
 * negative budget. */
int cr_ctx_set_alloc_limit(cr_ctx* ctx, int64_t bytes);
/* Per-call stage and kernel timings (cr_ctx_last_timings) on (nonzero, the
 * default) or off.  Collecting them makes every call wait for its events;
 * with them off, cr_ctx_last_timings reports zeros and a call whose outputs
 * all stay in device memory returns once its work is queued on the
 * context's stream (calls that return host values still wait for them).
 * Such a call may still be copying its host inputs when it returns: keep
 * them unchanged until the stream has passed the call (cr_ctx_synchronize,
 * or an event on the stream).  New; no counterpart in the reference
 * (ImagingStageTimings is always filled there). */
int cr_ctx_set_timings(cr_ctx* ctx, int32_t enable);
const char* cr_version(void);

/* ---- gridders ------------------------------------------------------------
 * cr_gridder_create replaces StandardGridder::new_with_padding_factor
 * (gridder.rs:393-443); oversampling 100 is the reference default. */
int cr_gridder_create(cr_ctx* ctx, const cr_geometry* geom, double padding,
                      int32_t oversampling, cr_gridder** out, cr_grid_info* info, char** err);
void cr_gridder_destroy(cr_gridder* g);
/* Copies the normalised tap rows [(2*(os/2)+1) x 7] and the two correction
 * axes (float32) to host buffers; any pointer may be NULL. */
int cr_gridder_tables(cr_gridder* g, float* taps, float* corr_x, float* corr_y, char** err);

/* WProjector::new (gridder.rs:3403-3586).  planes <= 0 chooses the count
 * from max_abs_w (choose_w_project_plane_count, gridder.rs:3801-3806);
 * sampling <= 0 keeps the reference rule (4 when planes > 1, else 1).
 * support_min > 0 selects the law S_p = support_min +
 * round((support_max - support_min) * p / (planes - 1)); support_min <= 0
 * keeps the reference's threshold search (gridder.rs:3832-3855). */
int cr_wproj_create(cr_ctx* ctx, cr_gridder* g, double max_abs_w, int32_t planes,
                    int32_t sampling, int32_t support_min, int32_t support_max,
                    cr_wproj** out, cr_wproj_info* info, char** err);
void cr_wproj_destroy(cr_wproj* wp);
/* Copies supports [planes], cropped kernels [planes][width][width] complex64
 * and the normalisation table [planes][2r+1][2r+1] float32 to host. */
int cr_wproj_tables(cr_wproj* wp, int32_t* support, float* kernels, float* norm, char** err);

/* ---- gridding / degridding ---------------------------------------------
 * cr_grid_dirty replaces accumulate_dirty_psf_and_residual_standard_streaming_grid
 * (lib.rs:68306-68500) when wp is NULL, and accumulate_w_project_dirty_grids_streaming
 * (lib.rs:71091-71138) when wp is given.  Outputs two grid_nx*grid_ny
 * complex64 grids (PSF, dirty) at `out_location`. */
int cr_grid_dirty(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                  float* psf_grid, float* dirty_grid, int32_t out_location, cr_sums* sums,
                  char** err);
/* degrid_sample_taps_planned_normalized (gridder.rs:1278-1312) /
 * degrid_sample_planned (gridder.rs:3726-3747) for every sample of the batch:
 * model_grid is grid_nx*grid_ny complex64 at `grid_location`, pred receives
 * n complex64 at `out_location` (0 for samples that do not plan). */
int cr_degrid(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
              const float* model_grid, int32_t grid_location, float* pred,
              int32_t out_location, char** err);
/* Fused residual refresh: degrid_model_and_grid_residual_taps_planned_f64
 * (gridder.rs:1315-1396) / accumulate_w_project_residual_streaming_sample
 * (lib.rs:71514-71541): residual_grid = G((vis - D(model_grid)) * weight). */
int cr_grid_residual(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                     const float* model_grid, int32_t grid_location, float* residual_grid,
                     int32_t out_location, cr_sums* sums, char** err);

/* ---- materialised plans -------------------------------------------------
 * The device form of the reference's planned taps (plan_sample,
 * gridder.rs:3588-3624; the materialised tap plans of
 * StandardMfsCpuExecutor, execution.rs:53-160): FP64 index selection, sort
 * and deduplication of one batch, done once and reused by any number of
 * gridding, degridding and residual calls while the batch's coordinates,
 * weights and visibilities stay unchanged (a major-cycle loop).  The plan
 * keeps no pointer to the batch. */
int cr_plan_create(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                   cr_plan** out, cr_sums* sums, char** err);
void cr_plan_destroy(cr_plan* plan);
int cr_plan_grid_dirty(cr_ctx* ctx, cr_plan* plan, float* psf_grid, float* dirty_grid,
                       int32_t out_location, char** err);
int cr_plan_degrid(cr_ctx* ctx, cr_plan* plan, const float* model_grid, int32_t grid_location,
                   float* pred, int32_t out_location, char** err);
int cr_plan_grid_residual(cr_ctx* ctx, cr_plan* plan, const float* model_grid,
                          int32_t grid_location, float* residual_grid, int32_t out_location,
                          char** err);
/* The major-cycle residual refresh of run_hogbom_cotton_schwab
 * (lib.rs:59354-59636 calls it through refresh_residual; the refresh is
 * compute_residual, lib.rs:68560-68620 standard, 70592-70644 W-projection):
 * model image -> apodise + centred forward FFT -> degrid -> residual
 * gridding -> centred inverse FFT + correction -> x k/sumwt (k = 2 for
 * W-projection) -> / psf_peak, over the plan's materialised records. */
int cr_plan_residual_image(cr_ctx* ctx, cr_plan* plan, const float* model,
                           int32_t model_location, const cr_psf_state* state,
                           float* residual_out, int32_t out_location, char** err);

/* ---- FFT, correction, normalisation ------------------------------------
 * Centred inverse FFT (fft.rs:600-630) of a grid then crop x correction:
 * corrected_image_from_grid_f64 (gridder.rs:1646-1657), or the W-projection
 * correction (gridder.rs:1685-1715) when wp is given; the result is scaled
 * by `scale` (float32 multiply).  cuFFT performs the bare transform only. */
int cr_grid_to_image(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float* grid,
                     int32_t grid_location, float scale, float* image, int32_t out_location,
                     char** err);
/* apodize_model / apodize_w_project_model (gridder.rs:1554-1592) then the
 * centred unscaled forward FFT (fft.rs:34): model image -> model grid. */
int cr_image_to_grid(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float* model,
                     int32_t model_location, float* grid, int32_t out_location, char** err);

/* ---- whole stages (the run_imaging seams) --------------------------------
 * compute_dirty_psf_and_residual_standard_streaming (lib.rs:68137-68185) with
 * dirty_grids_to_psf_and_residual_owned (lib.rs:48987-49130), or
 * compute_dirty_psf_and_residual_w_project_streaming (lib.rs:70539-70590).
 * Writes the normalised PSF and residual images (nx*ny float32). */
int cr_dirty_image(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                   float* psf, float* residual, int32_t out_location, cr_psf_state* state,
                   cr_sums* sums, char** err);
/* compute_residual (lib.rs:68560-68620 / lib.rs:70592-70644): model image ->
 * residual image normalised by the given PSF state. */
int cr_residual_image(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                      const float* model, int32_t model_location, const cr_psf_state* state,
                      float* residual, int32_t out_location, cr_sums* sums, char** err);
/* Forward operator A of the forward/adjoint pair: model image -> model
 * visibilities (apodize, centred FFT, degrid). */
int cr_predict(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
               const float* model, int32_t model_location, float* pred,
               int32_t out_location, char** err);
/* Adjoint A^H: visibilities (the batch's vis, weighted) -> image, without
 * normalisation: grid, centred inverse FFT scaled by Nx*Ny, crop, correct. */
int cr_adjoint(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
               float* image, int32_t out_location, char** err);

/* ---- streaming dirty accumulation ----------------------------------------
 * StandardMfsDirtyAccumulator (lib.rs:3259-3380): natural-weighted batches
 * (weights already final) gridded one after another into one pair of
 * device-resident PSF and dirty grids with the standard gridder, so a caller
 * can load a MeasurementSet chunk by chunk and release each; finish forms
 * the normalised PSF and residual images (dirty_grids_to_psf_and_residual_
 * owned) from the accumulated grids and sums, CR_NO_SAMPLES when nothing
 * usable was added.  The accumulator can finish more than once. */
int cr_accumulator_create(cr_ctx* ctx, cr_gridder* g, cr_accumulator** out, char** err);
void cr_accumulator_destroy(cr_accumulator* acc);
int cr_accumulator_add(cr_ctx* ctx, cr_accumulator* acc, const cr_vis_batch* batch,
                       cr_sums* batch_sums, char** err);
int cr_accumulator_finish(cr_ctx* ctx, cr_accumulator* acc, float* psf, float* residual,
                          int32_t out_location, cr_psf_state* state, cr_sums* total, char** err);

/* ---- batched spectral cube ------------------------------------------------
 * Channel c's batch is the unflagged samples of rows r = 0..rows-1 with
 * u_lambda = u_m[r] * lambda_scale[c], v_lambda = v_m[r] * lambda_scale[c]
 * (the cube batch assembly of casars-imager/src/lib.rs:49571-49576:
 * lambda_scale = channel frequency / speed of light; flagged samples are left
 * out of the channel batch).  vis, weight and flags are channel-major
 * [channels][rows]; lambda_scale is host memory, the other arrays are at
 * `location`.  Weighting is per channel with the PerPlane density of cube
 * imaging (weighting.rs:1055-1180 with weighting.rs:1455-1483: the density
 * at the rounded cell, Hermitian mirror included); gridding is the standard
 * PSWF gridder (support 3) of every channel.  All channels are planned and
 * gridded by one fixed sequence of launches (it does not grow with the
 * number of channels).  channels * rows must stay below 2^32. */
typedef struct {
    int64_t rows;
    int32_t channels;
    const double* u_m;            /* [rows] metres */
    const double* v_m;            /* [rows] metres */
    const double* lambda_scale;   /* [channels], host memory */
    const float* vis;             /* [channels][rows] complex64 */
    const float* weight;          /* [channels][rows] or NULL (all 1) */
    const uint8_t* flags;         /* [channels][rows], nonzero = flagged, or NULL */
    int32_t location;
} cr_cube_batch;

/* psf_grids [channels][gnx][gny] float32 (real part of each channel's PSF
 * grid), dirty_grids [channels][gnx][gny] complex64, sums[channels]. */
/* Calls whose arrays are all device memory are captured into a CUDA graph
 * on their second occurrence with the same pointers and parameters and
 * replayed afterwards (cr_timings.grid_ms then times the whole pipeline);
 * this switches that off (0) or on (nonzero, the default). */
int cr_ctx_set_cube_graphs(cr_ctx* ctx, int32_t enable);
/* Records per work item of the cube gridding pass.  0 (the default): the
 * first call of each cube shape times 1024, 2048 and 4096 and keeps the
 * fastest for the context; one of those values: that size, no timing.
 * Returns CR_INVALID for any other value.  New; no counterpart in the
 * reference (its CPU cube path has no work items). */
int cr_ctx_set_cube_grid_chunk(cr_ctx* ctx, int32_t chunk);
int cr_cube_grid_dirty(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch,
                       int32_t weighting, float robust, float* psf_grids, float* dirty_grids,
                       int32_t out_location, cr_sums* sums, char** err);
/* pred [channels][rows] complex64 = degridded model_grids [channels][gnx][gny]
 * complex64 (degrid_sample_taps_planned_normalized, gridder.rs:1278-1312);
 * 0 for samples the gridder skips. */
int cr_cube_degrid(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch, int32_t weighting,
                   float robust, const float* model_grids, int32_t grid_location, float* pred,
                   int32_t out_location, char** err);
/* Both from one plan of the batch (one grid + degrid pass of the cube). */
int cr_cube_grid_degrid(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch,
                        int32_t weighting, float robust, float* psf_grids, float* dirty_grids,
                        const float* model_grids, int32_t grid_location, float* pred,
                        int32_t out_location, cr_sums* sums, char** err);
/* The per-sample plan of every channel ([channels][rows] int32 / float32):
 * start cell and tap row per axis (sample_tap_span, gridder.rs:1976-1995)
 * and the imaging weight; -1 and 0 for samples that are not gridded. */
int cr_cube_sample_taps(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch,
                        int32_t weighting, float robust, int32_t* start_x, int32_t* start_y,
                        int32_t* row_x, int32_t* row_y, float* imaging_weight,
                        int32_t out_location, char** err);

/* ---- persistent cube plans -------------------------------------------------
 * The cube's weighting and records made once (cr_cube_plan_create, the
 * weighting and planning of cr_cube_grid_dirty) and reused by gridding,
 * degridding and residual calls: the planned-sample replay that
 * run_standard_mfs_cube_clean (casa-imaging lib.rs:3026-3210) drives once per
 * plane and major cycle.  The plan copies what it needs (weighted
 * visibilities in record order); the batch may be released afterwards.
 * `sums` receives one cr_sums per channel.
 *
 * planes (host, [channels], NULL = all) selects the planes a residual call
 * refreshes; the others' outputs are left as they are.  The image calls
 * use the single-plane normalisation per channel (cr_dirty_image /
 * cr_plan_residual_image); a plane without usable samples gets zero images
 * and a zero cr_psf_state instead of an error. */
int cr_cube_plan_create(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch,
                        int32_t weighting, float robust, cr_cube_plan** out, cr_sums* sums,
                        char** err);
void cr_cube_plan_destroy(cr_cube_plan* plan);
int32_t cr_cube_plan_channels(const cr_cube_plan* plan);
/* Transforms of the image calls: 32 = float32 C2C (the default; FP64 runs
 * at a small fraction of the float32 rate on this GPU), 64 = FP64 Z2Z as in
 * the single-plane calls.  Returns CR_INVALID for other values. */
int cr_cube_plan_set_fft_precision(cr_cube_plan* plan, int32_t bits);
int cr_cube_plan_grid_dirty(cr_ctx* ctx, cr_cube_plan* plan, float* psf_grids,
                            float* dirty_grids, int32_t out_location, char** err);
int cr_cube_plan_degrid(cr_ctx* ctx, cr_cube_plan* plan, const float* model_grids,
                        int32_t grid_location, float* pred, int32_t out_location, char** err);
/* Residual grids: degrid the model grids, (vis - pred) weighted, gridded. */
int cr_cube_plan_grid_residual(cr_ctx* ctx, cr_cube_plan* plan, const float* model_grids,
                               int32_t grid_location, const uint8_t* planes,
                               float* residual_grids, int32_t out_location, char** err);
/* Normalised PSF and residual images [channels][nx][ny] with each plane's
 * PSF state. */
int cr_cube_plan_dirty_images(cr_ctx* ctx, cr_cube_plan* plan, float* psf_images,
                              float* residual_images, int32_t out_location,
                              cr_psf_state* states, char** err);
/* Model images [channels][nx][ny] -> residual images of the selected
 * planes (the major-cycle refresh of each plane). */
int cr_cube_plan_residual_images(cr_ctx* ctx, cr_cube_plan* plan, const float* models,
                                 int32_t model_location, const uint8_t* planes,
                                 const cr_psf_state* states, float* residual_images,
                                 int32_t out_location, char** err);

/* ---- row runs ---------------------------------------------------------------
 * The row path's sample preparation on the device
 * (routed_weighted_grid_sample_from_run, lib.rs:880-1062): every kept
 * (row, channel) sample, in that order, as a visibility batch -- u, v, w in
 * wavelengths (uvw_m * lambda_scale, FP64), the natural weight, the plane's
 * sumwt factor, the row's gridable flag, the (collapsed) visibility -- plus
 * the VisImagingWeight density coordinates of the row path
 * (casa_vis_imaging_weight_uv_lambda, weighting.rs:748-756:
 * float32(u_m * float32(f/c))).  A sample is dropped when a used correlation
 * is flagged, its visibility is not finite, a hand's weight or the natural
 * weight is not finite and positive, or the sumwt factor is not.  Outputs
 * hold rows * channels entries at out_location; *n_out receives the count.
 * vis is complex64 interleaved. */
int cr_row_runs_prepare(cr_ctx* ctx, const cr_row_runs* runs, const cr_polarization* pol,
                        double* u, double* v, double* w, float* weight, float* sumwt_factor,
                        uint8_t* gridable, float* vis, double* density_u, double* density_v,
                        int32_t out_location, int64_t* n_out, char** err);
/* PlaneStokes::derive_pair_selection and paired_sumwt_factor
 * (types.rs:62-138): the polarization of plane 0 I, 1 Q, 2 U, 3 V (a pair of
 * CASA correlation codes RR=5, RL=6, LR=7, LL=8, XX=9, XY=10, YX=11, YY=12,
 * collapsed; sumwt factor 2 for I, 1 otherwise) or of the raw planes 4 XX,
 * 5 YY, 6 RR, 7 LL (that correlation, explicit, sumwt factor 1).
 * CR_INVALID when the correlations cannot form the plane. */
int cr_polarization_for_plane(int32_t plane, const int32_t* corr_types, int32_t correlations,
                              cr_polarization* out, char** err);
/* Weighting of a row-path batch: the density is built at the density
 * coordinates (density_u, density_v, at the batch's location) and looked up
 * at the batch's u, v, as the streaming weighting plan does
 * (accumulate_standard_mfs_density_row_with_accessors, weighting.rs:646-746;
 * weight_sample, weighting.rs:333-380). */
int cr_apply_weighting_rows(cr_ctx* ctx, cr_gridder* g, const cr_vis_batch* batch,
                            const double* density_u, const double* density_v, int32_t mode,
                            float robust, float* out_weight, int32_t out_location, float* f2,
                            char** err);

/* ---- row-block read-ahead feed ---------------------------------------------
 * The device side of stream_imaging_source_read_ahead_blocks
 * (casars-imager/src/lib.rs:36608-36760): a bounded read-ahead pipeline of
 * MeasurementSet row blocks.  The caller's reader (the producer) fills one
 * page-locked staging slot at a time with a row block's UVW, DATA, FLAG,
 * WEIGHT or WEIGHT_SPECTRUM and FLAG_ROW columns in the layout of
 * cr_row_runs and submits it; the slot is uploaded on the feed's own copy
 * stream while the previous block is prepared and gridded, and a worker
 * thread of the feed (the consumer) runs cr_row_runs_prepare and
 * cr_accumulator_add on the context's stream for each block in submission
 * order.  At most max_live_row_blocks blocks are live (acquired and not yet
 * consumed; the reference's default read-ahead depth is 2,
 * imaging_source_read_ahead_max_live_row_blocks, lib.rs:36542-36544);
 * acquire waits for a slot when all are live, which is the reference's
 * producer back-pressure.  Weights are used as given (natural weighting, as
 * for cr_accumulator_*).  While a feed is between create and finish its
 * context belongs to the feed's worker: the caller makes no other call on
 * that context until finish returns. */
typedef struct cr_row_feed cr_row_feed;
typedef struct {
    int32_t max_live_row_blocks;    /* staging slots, >= 1 */
    int64_t row_block_rows;         /* rows per slot, >= 1 */
    int32_t channels;               /* of the one spectral window fed */
    int32_t correlations;
    const double* lambda_scale;     /* host [channels]: CHAN_FREQ / c, copied */
    cr_polarization polarization;   /* the plane's collapse (cr_polarization_for_plane) */
    int32_t has_flag;               /* FLAG present */
    int32_t has_weight_spectrum;    /* WEIGHT_SPECTRUM instead of WEIGHT */
    int32_t has_gridable;           /* per-row gridable (not FLAG_ROW) present */
} cr_row_feed_config;
/* A staging slot: page-locked host arrays of max_rows rows in the layout of
 * cr_row_runs; the absent columns are NULL. */
typedef struct {
    int32_t slot;
    int64_t max_rows;
    double* uvw_m;                  /* [rows][3] */
    float* data;                    /* complex64 [rows][channels][correlations] */
    uint8_t* flag;                  /* [rows][channels][correlations] */
    float* weight;                  /* [rows][correlations] */
    float* weight_spectrum;         /* [rows][channels][correlations] */
    uint8_t* gridable;              /* [rows] */
} cr_row_block;
/* ImagingSourceReadAheadSummary (casars-imager/src/lib.rs:36324-36335):
 * blocks consumed, samples prepared (kept), host bytes uploaded, the most
 * blocks live at once, and wall times: acquire waiting for a free slot
 * (producer_send_blocked), the worker waiting for a block
 * (consumer_recv_blocked), the worker busy (consumer_elapsed), and the time
 * a block was being filled while the worker was busy
 * (producer_consumer_overlap). */
typedef struct {
    int64_t row_blocks;
    int64_t streamed_samples;
    int64_t source_bytes;
    int32_t live_row_block_high_water;
    double producer_send_blocked_s;
    double consumer_recv_blocked_s;
    double consumer_elapsed_s;
    double producer_consumer_overlap_s;
} cr_row_feed_summary;
int cr_row_feed_create(cr_ctx* ctx, cr_gridder* g, const cr_row_feed_config* config,
                       cr_row_feed** out, char** err);
/* Stops the worker (blocks still queued are dropped) and frees the slots. */
void cr_row_feed_destroy(cr_row_feed* feed);
/* The next free slot (waits while max_live_row_blocks blocks are live).  A
 * failure of an earlier block is reported here, by submit and by finish. */
int cr_row_feed_acquire(cr_row_feed* feed, cr_row_block* block, char** err);
/* Queues the acquired slot's first `rows` rows (0 <= rows <= max_rows);
 * rows = 0 hands the slot back unused (not counted as a row block). */
int cr_row_feed_submit(cr_row_feed* feed, int32_t slot, int64_t rows, char** err);
/* Waits for every submitted block, then forms the normalised PSF and residual
 * images from the accumulated grids (cr_accumulator_finish); CR_NO_SAMPLES
 * when nothing usable was fed.  The feed can take more blocks afterwards. */
int cr_row_feed_finish(cr_row_feed* feed, float* psf, float* residual, int32_t out_location,
                       cr_psf_state* state, cr_sums* total, cr_row_feed_summary* summary,
                       char** err);

/* ---- restoring beam ---------------------------------------------------------
 * fit_beam_from_psf (beam.rs:27-103): the main lobe above `cutoff` (clamped
 * to [0.01, 0.99], lowered by 1.5x per failed attempt, at most 50 attempts),
 * resampled bicubically and fitted by Levenberg-Marquardt; FWHM and position
 * angle in radians, quantised through float32 arcsec / degrees.  *fitted is
 * 0 when no attempt converged.  The fit runs on the host (a device PSF is
 * copied back first; ctx may be NULL for a host PSF). */
typedef struct {
    double major_fwhm_rad, minor_fwhm_rad, position_angle_rad;
} cr_beam;
int cr_fit_beam(cr_ctx* ctx, const float* psf, int32_t nx, int32_t ny, int32_t location,
                double cell_x_rad, double cell_y_rad, float cutoff, cr_beam* beam,
                int32_t* fitted, int32_t* attempts, float* cutoff_used, char** err);
/* restore_model (beam.rs:105-120) plus the residual: restored = model (*)
 * Gaussian (the analytic beam of make_casa_gaussian_psf_image, full-plane
 * circular FFT convolution) + residual (NULL: model only).  Even sides. */
int cr_restore(cr_ctx* ctx, const float* model, const float* residual, int32_t nx, int32_t ny,
               int32_t location, double cell_x_rad, double cell_y_rad, const cr_beam* beam,
               float* restored, int32_t out_location, char** err);
/* estimate_psf_sidelobe_level_with_beam (beam.rs:319-328):
 * max(|min psf|, |max(psf - Gaussian)|); 0 for an unusable beam. */
int cr_psf_sidelobe(cr_ctx* ctx, const float* psf, int32_t nx, int32_t ny, int32_t location,
                    double cell_x_rad, double cell_y_rad, const cr_beam* beam, float* level,
                    char** err);

/* ---- weighting -----------------------------------------------------------
 * apply_weighting_with_density_source, Combined density
 * (weighting.rs:1055-1180): natural passes weights through; uniform and
 * Briggs build the density grid with the Hermitian mirror and reweight.
 * out_weight receives n float32 at `out_location`; f2 (Briggs) is returned. */
int cr_apply_weighting(cr_ctx* ctx, cr_gridder* g, const cr_vis_batch* batch, int32_t mode,
                       float robust, float* out_weight, int32_t out_location, float* f2,
                       char** err);
/* The same with the PerPlane density of cube imaging, one channel's batch
 * (density_build_cell_convention / density_cell_convention with
 * WeightDensityMode::PerPlane, weighting.rs:1455-1483: rounded FP64 cells). */
int cr_apply_weighting_plane(cr_ctx* ctx, cr_gridder* g, const cr_vis_batch* batch,
                             int32_t mode, float robust, float* out_weight,
                             int32_t out_location, float* f2, char** err);

/* ---- Hogbom minor cycle --------------------------------------------------
 * run_hogbom_minor_cycle_cpu_with_progress (lib.rs:59748-59883): one
 * persistent device loop of peak search (ties to the smallest y*nx+x),
 * threshold tests, model update and shifted-PSF subtraction.  model,
 * residual, psf (nx*ny float32) and mask (nx*ny uint8 or NULL) are at
 * `location`; model and residual are updated in place.  Component arrays
 * (capacity cycle_niter + 1) are host memory and may be NULL. */
int cr_hogbom(cr_ctx* ctx, float* model, float* residual, const float* psf,
              const uint8_t* mask, int32_t nx, int32_t ny, int32_t location, float gain,
              float threshold, float cycle_threshold, float nsigma_threshold,
              int64_t cycle_niter, int32_t inclusive, int32_t* comp_x, int32_t* comp_y,
              float* comp_peak, float* comp_flux, int64_t* actual, int64_t* reported,
              int32_t* stop_reason, char** err);

/* run_hogbom_plane_minor_cycle (crates/casa-imaging/src/lib.rs:64630-64680;
 * HogbomPlaneMinorCycleControl, lib.rs:64555-64580): the finite peak with a
 * relative tolerance (finite_peak_location_masked_with_relative_tolerance,
 * lib.rs:73998-74026: y-major scan, a value replaces the peak only if
 * |v| > |peak| * (1 + tol)), stop when |peak| <= threshold or <= the cycle
 * threshold, model += gain * peak, subtract_shifted_psf.  Arrays as
 * cr_hogbom; tolerance 0 runs the same persistent loop as cr_hogbom, a
 * positive tolerance an exact single-block replay of the scan. */
int cr_hogbom_plane(cr_ctx* ctx, float* model, float* residual, const float* psf,
                    const uint8_t* mask, int32_t nx, int32_t ny, int32_t location, float gain,
                    float threshold, float cycle_threshold, float peak_relative_tolerance,
                    int64_t cycle_limit, int32_t inclusive, int32_t* comp_x, int32_t* comp_y,
                    float* comp_peak, float* comp_flux, int64_t* actual, int64_t* reported,
                    char** err);

/* The Hogbom minor cycles of several planes in one launch: model, residual,
 * psf (and mask, or NULL) are DEVICE arrays [nplanes][nx][ny]; the n planes
 * listed in `planes` (host) each run run_hogbom_minor_cycle_cpu_with_progress
 * with the same gain, thresholds and budget, as cr_hogbom would one by one
 * (each plane's blocks only touch that plane).  nsigma_thresholds (host [n],
 * or NULL for nsigma_threshold on every plane) gives each listed plane its
 * own n-sigma threshold, as the cube's per-plane controllers compute them
 * (lib.rs:46395-46396).  actual, reported and stop_reason are host [n]; the
 * component arrays (host, or NULL) hold [n][cycle_niter + 1] entries, plane
 * s's first actual[s] of them valid. */
int cr_hogbom_planes(cr_ctx* ctx, float* model, float* residual, const float* psf,
                     const uint8_t* mask, int32_t nplanes, int32_t nx, int32_t ny,
                     const int32_t* planes, int32_t n, float gain, float threshold,
                     float cycle_threshold, float nsigma_threshold,
                     const float* nsigma_thresholds, int64_t cycle_niter, int32_t inclusive,
                     int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
                     int64_t* actual, int64_t* reported, int32_t* stop_reason, char** err);

/* ---- Clark minor cycle ------------------------------------------------------
 * run_clark_minor_cycle_cpu (lib.rs:62129-62355): subcycles over the active
 * pixels (|residual| >= max(peak x max exterior PSF x factor, cycle
 * threshold)) with a (3 ncent + 1)^2 PSF patch about the centre
 * (build_clark_psf_patch, lib.rs:64422-64456; ncent = max(4, ceil(major /
 * cell), ceil(minor / cell)) of the fitted beam), then the residual update by
 * the PSF convolution of the subcycle's components (fft_convolve_real,
 * lib.rs:64415-64420).  model and residual are
 * updated in place at `location`; component arrays (host, capacity
 * cycle_niter) may be NULL; *max_exterior_abs receives the patch's exterior
 * PSF peak. */
int cr_clark(cr_ctx* ctx, float* model, float* residual, const float* psf, const uint8_t* mask,
             int32_t nx, int32_t ny, int32_t location, int32_t ncent, float gain,
             float threshold, float cycle_threshold, float nsigma_threshold, int64_t cycle_niter,
             int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
             int64_t* actual, int32_t* stop_reason, float* max_exterior_abs, char** err);

/* ---- multiscale CLEAN ------------------------------------------------------
 * run_multiscale_cotton_schwab's deconvolver state and minor cycle
 * (crates/casa-imaging/src/lib.rs:63543-64405).  cr_multiscale_create builds
 * the state of build_multiscale_state (lib.rs:64172-64230) from the PSF
 * (nx x ny float32 at `location`), an optional clean mask (nonzero =
 * cleanable; it then gives each scale its mask, lib.rs:64232-64261), the
 * scale sizes in pixels (host array; none = the single scale 0,
 * lib.rs:64164-64170; at most 16) and the small-scale bias.  The state
 * lives on the device: the scale images, the PSF convolved with scale k
 * then scale l, and the residual convolved with every scale.
 * cr_multiscale_set_residual refreshes the convolved residuals after a major
 * cycle (refresh_multiscale_dirty_conv_scales, lib.rs:63261-63267);
 * cr_multiscale_residual copies out the residual convolved with scale 0 (the
 * deconvolver's residual); cr_multiscale_peak reports whether any scale has
 * a candidate and the masked peak |value| of that residual.
 * cr_multiscale_minor_cycle runs one minor cycle (lib.rs:63700-63800) on the
 * device: at most cycle_niter components, each gain * strength of the
 * scale-biased best candidate, added to `model` (nx x ny float32 at
 * `location`, updated in place) over the scale image's support and
 * subtracted from every convolved residual inside the component's window.
 * Component arrays (host, capacity cycle_niter, or all NULL) receive
 * position, scale index, strength and flux; *stop_reason is a CR_STOP_*
 * code, or -1 for the divergence rule (DivergenceDetected, lib.rs:64011-64023). */
int cr_multiscale_create(cr_ctx* ctx, const float* psf, const uint8_t* mask, int32_t nx,
                         int32_t ny, int32_t location, const float* scales, int32_t nscales,
                         float small_scale_bias, cr_multiscale** out, char** err);
void cr_multiscale_destroy(cr_multiscale* ms);
int cr_multiscale_set_residual(cr_multiscale* ms, const float* residual, int32_t location,
                               char** err);
int cr_multiscale_residual(cr_multiscale* ms, float* out, int32_t location, char** err);
int cr_multiscale_peak(cr_multiscale* ms, int32_t* has_candidate, float* peak0, char** err);
int cr_multiscale_minor_cycle(cr_multiscale* ms, float* model, int32_t location, float gain,
                              float threshold, float cycle_threshold, float nsigma_threshold,
                              int64_t cycle_niter, int32_t* comp_x, int32_t* comp_y,
                              int32_t* comp_scale, float* comp_strength, float* comp_flux,
                              int64_t* actual, int64_t* reported, int32_t* stop_reason,
                              char** err);

/* Robust RMS of residual images for the n-sigma threshold:
 * robust_rms_jy_per_beam (crates/casa-imaging/src/lib.rs:74130-74183), the
 * threshold being nsigma * rms (nsigma_threshold_jy_per_beam,
 * lib.rs:74474-74484).  images [nimages][nx][ny] float32 and optional clean
 * masks [nimages][nx][ny] (nonzero = cleanable) at `location`; for each of
 * the nplanes listed planes (host array of image indices):
 *   values = the finite pixels (only those outside the clean mask when the
 *            plane's mask is not all true), Chauvenet-clipped (automatic z,
 *            at most 5 iterations, lib.rs:74512-74622) when not restricted
 *            by a mask;
 *   rms[k] = f32(MADFM(values)) * 1.4826f, 0 when no value remains.
 * Optional host outputs: madfm[k] (FP64) and counts[k] (values the MADFM was
 * taken over).  The MADFM is an exact selection (bit-identical to sorting);
 * the clipping windows come from FP64 sums in another order than the
 * reference's sequential sums. */
int cr_robust_rms(cr_ctx* ctx, const float* images, const uint8_t* masks, int32_t nimages,
                  int32_t nx, int32_t ny, int32_t location, const int32_t* planes,
                  int32_t nplanes, float* rms, double* madfm, int64_t* counts, char** err);

/* Measurement, not imaging (no counterpart in the reference): the tap-rate
 * ceiling of the W-projection gridding loop.  Runs only the irreducible work
 * of a tap -- one float2 read from an L2-resident buffer of buffer_bytes
 * (rows of 32 consecutive values at scattered addresses, as the kernel cube
 * is read) and three paired FP32 FMAs into register accumulators -- for
 * `iters` iterations of 8 rows per thread on every resident thread, and
 * returns the taps per second of one timed launch and the taps it made. */
int cr_probe_tap_rate(cr_ctx* ctx, int64_t buffer_bytes, int32_t iters,
                      double* taps_per_second, double* taps, char** err);

/* ---- allocation-free Hogbom minor cycle ----------------------------------
 * No counterpart in the reference.  The same minor cycle as cr_hogbom for
 * callers that may not allocate device memory once they run: for example a
 * host that reserved a fixed device-memory budget at start-up and forbids
 * further allocation, or a process in which another allocator holds nearly
 * all device memory, so a cudaMalloc could fail or stall the device in the
 * middle of a deconvolution loop.  It calls no cudaMalloc, cudaFree or
 * allocating library routine.  model, residual, psf and mask are DEVICE
 * buffers (model and residual updated in place); the component arrays are
 * host memory, as in cr_hogbom.
 *
 * Its scratch (barrier words, per-block peak candidates and the component
 * list) is one fixed 295,168-byte array in the library's device memory, which
 * every GPU that loads the library holds until the process exits.  Limit:
 * at most 16384 components per call (cycle_niter, plus one when inclusive);
 * a larger budget is rejected with CR_INVALID.  The array's memory is
 * committed when a context is created on the device: cr_ctx_create looks up
 * its device address (once per device, with that device current), which
 * loads the module that holds it, so this call does no set-up of its own;
 * create the context before any stream capture.  Every call on a device
 * shares the one array: calls that overlap on the GPU (other streams,
 * contexts or threads) race and must be serialised by the caller.  Like the
 * library's other calls, it makes the context's device current
 * (cudaSetDevice) and leaves it current. */
int cr_hogbom_noalloc(cr_ctx* ctx, float* model, float* residual, const float* psf,
                      const uint8_t* mask, int32_t nx, int32_t ny, float gain, float threshold,
                      float cycle_threshold, float nsigma_threshold, int64_t cycle_niter,
                      int32_t inclusive, int32_t* comp_x, int32_t* comp_y, float* comp_peak,
                      float* comp_flux, int64_t* actual, int64_t* reported,
                      int32_t* stop_reason, char** err);

#ifdef __cplusplus
}
#endif
#endif
