/*
 * casa_oracle.h -- FP64 CPU restatement of the casa-imaging hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker that the CUDA path
 * is compared against, and the CPU baseline that bench.py times beside it.
 * It is never linked into, loaded by, or called from the product library
 * (casa-rs_gb300/) and the product has no CPU fallback that routes here.
 *
 * Every function restates one reference function; the citation is the
 * reference file and line (paths relative to the casa-rs repository, `lib.rs`
 * meaning crates/casa-imaging/src/lib.rs, `gridder.rs` meaning
 * crates/casa-imaging/src/gridder.rs, `weighting.rs` likewise).
 *
 * Conventions shared with the product ABI:
 *   grids   complex, interleaved (re, im), x-major: flat = x * gny + y
 *   images  float32 x-major: flat = x * ny + y
 *   vis     complex64 interleaved (re, im)
 * Compiled with -ffp-contract=off so every float multiply and add rounds
 * separately, as the reference (and CASA) do.
 */
#ifndef CASA_ORACLE_H
#define CASA_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- grid geometry and PSWF tables -------------------------------------- */
int64_t oc_casa_composite_padded_len(int64_t image_len, double padding);
void oc_image_blc(int64_t grid_len, int64_t image_len, int64_t* blc);
double oc_grdsf(double nu);
float oc_spheroidal_kernel(double distance, double support);
void oc_std_kernel_table(int32_t oversampling, int32_t support, float* out);
int32_t oc_std_tap_rows(int32_t oversampling);
void oc_std_normalized_taps(const float* table, int32_t table_len, int32_t oversampling,
                            int32_t support, float* out);
void oc_correction_axis(int64_t size, float* out);
void oc_gridder_correction_axis(int64_t size, float* out);
void oc_sinc_axis(int64_t size, int64_t conv_sampling, float* out);

/* ---- standard (PSWF) gridder -------------------------------------------- */
typedef struct {
    int64_t gnx, gny;          /* grid shape */
    int32_t oversampling;      /* taps per cell */
    int32_t support;           /* 3 -> 7 taps */
    double du, dv;             /* grid spacing in wavelengths */
    const float* taps;         /* [tap_rows][2*support+1] normalised rows */
    int32_t tap_rows;
} oc_std_gridder;

typedef struct {
    double normalization_sumwt;
    double reported_sumwt;
    int64_t gridded;
    int64_t skipped;
} oc_accum;

int oc_std_tap_span(const oc_std_gridder* g, double coordinate, int64_t size,
                    int64_t* start, int64_t* weight_index);
int oc_std_plan(const oc_std_gridder* g, double u, double v, int64_t* x0, int64_t* y0,
                int64_t* wx, int64_t* wy);
void oc_std_plan_many(const oc_std_gridder* g, int64_t n, const double* u, const double* v,
                      int32_t* x0, int32_t* y0, int32_t* wx, int32_t* wy);
void oc_std_grid_dirty(const oc_std_gridder* g, int64_t n, const double* u, const double* v,
                       const float* weight, const float* sumwt_factor, const uint8_t* gridable,
                       const float* vis, double* psf_grid, double* dirty_grid, oc_accum* acc,
                       int32_t nthreads);
void oc_std_degrid(const oc_std_gridder* g, const double* model_grid, int64_t n,
                   const double* u, const double* v, double* pred);
void oc_std_residual(const oc_std_gridder* g, const double* model_grid, int64_t n,
                     const double* u, const double* v, const float* weight,
                     const float* sumwt_factor, const uint8_t* gridable, const float* vis,
                     double* residual_grid, double* pred, oc_accum* acc, int32_t nthreads);

/* ---- W-projection ------------------------------------------------------- */
typedef struct {
    int64_t gnx, gny;
    double du, dv;
    int32_t planes;
    int32_t sampling;
    double w_scale;
    int32_t width;             /* common (padded) kernel width */
    const int32_t* support;    /* [planes] */
    const double* kernels;     /* [planes][width][width] complex, (kx, ky) x-major */
    int32_t norm_radius;       /* (sampling + 1) / 2 */
    const double* norm_table;  /* [planes][2r+1][2r+1] */
} oc_wproj;

int64_t oc_wproj_suggested_planes(int64_t nx, int64_t ny, double cell_x, double cell_y,
                                  double max_abs_w);
double oc_wproj_max_uvw(double cell_x, double max_abs_w, int explicit_planes);
int32_t oc_wproj_find_support(const double* axis_x, const double* axis_y, int64_t conv_size,
                              double peak, int32_t sampling);
int oc_wproj_build(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t gnx,
                   int64_t gny, double max_abs_w, int32_t planes, int explicit_planes,
                   int32_t sampling, int32_t support_min, int32_t support_max,
                   int32_t max_width, int32_t nthreads, double* w_scale_out,
                   int32_t* support_out, int32_t* width_out, double* kernels_out,
                   double* norm_out);
int32_t oc_wproj_plane_index(const oc_wproj* p, double w);
int oc_wproj_plan(const oc_wproj* p, double u, double v, double w, int64_t* loc_x,
                  int64_t* loc_y, int64_t* off_x, int64_t* off_y, int32_t* plane,
                  int32_t* conj, double* normalization);
void oc_wproj_grid_dirty(const oc_wproj* p, int64_t n, const double* u, const double* v,
                         const double* w, const float* weight, const float* sumwt_factor,
                         const uint8_t* gridable, const float* vis, double* psf_grid,
                         double* dirty_grid, oc_accum* acc, int32_t nthreads);
void oc_wproj_degrid(const oc_wproj* p, const double* model_grid, int64_t n, const double* u,
                     const double* v, const double* w, double* pred, int32_t nthreads);
void oc_wproj_residual(const oc_wproj* p, const double* model_grid, int64_t n,
                       const double* u, const double* v, const double* w, const float* weight,
                       const float* sumwt_factor, const uint8_t* gridable, const float* vis,
                       double* residual_grid, oc_accum* acc, int32_t nthreads);

/* ---- weighting ---------------------------------------------------------- */
int oc_density_cell(int64_t nx, int64_t ny, double cell_x, double cell_y, double u, double v,
                    int convention, int64_t* cx, int64_t* cy);
void oc_density_grid(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t n,
                     const double* u, const double* v, const float* weight, float* density);
void oc_density_grid_conv(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t n,
                          const double* u, const double* v, const float* weight, int convention,
                          float* density);
float oc_briggs_f2(const float* density, int64_t cells, float robust);
float oc_briggs_denominator(float density, float f2);
void oc_reweight(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t n,
                 const double* u, const double* v, const float* weight, const float* density,
                 int mode, float f2, float* out_weight);
void oc_reweight_conv(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t n,
                      const double* u, const double* v, const float* weight,
                      const float* density, int mode, float f2, int convention,
                      float* out_weight);

/* ---- Hogbom ------------------------------------------------------------- */
int oc_peak_location(const float* image, const uint8_t* mask, int64_t nx, int64_t ny,
                     int64_t* px, int64_t* py, float* value);
int oc_minor_cycle_stop_reason(float peak_abs, float threshold, float cycle_threshold,
                               float nsigma_threshold);
int64_t oc_hogbom(float* model, float* residual, const float* psf, const uint8_t* mask,
                  int64_t nx, int64_t ny, float gain, float threshold, float cycle_threshold,
                  float nsigma_threshold, int64_t cycle_niter, int inclusive,
                  int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
                  int32_t* stop_reason, int64_t* reported);
int oc_peak_relative(const float* image, const uint8_t* mask, int64_t nx, int64_t ny,
                     float tol, int64_t* px, int64_t* py, float* value);
int64_t oc_hogbom_plane(float* model, float* residual, const float* psf, const uint8_t* mask,
                        int64_t nx, int64_t ny, float gain, float threshold,
                        float cycle_threshold, float tol, int64_t cycle_limit, int inclusive,
                        int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
                        int64_t* reported);
void oc_subtract_shifted_psf(float* residual, const float* psf, int64_t nx, int64_t ny,
                             int64_t px, int64_t py, float component);

/* W-projection grid / degrid in the reference's Complex32 precision (the
 * timed CPU baseline; gridder.rs:3680-3747); kernels32 is the FP64 kernel
 * array of `p` rounded to float32, grids are float32 complex */
void oc_wproj_grid_dirty_f32(const oc_wproj* p, const float* kernels32, int64_t n,
                             const double* u, const double* v, const double* w,
                             const float* weight, const float* sumwt_factor,
                             const uint8_t* gridable, const float* vis, float* psf_grid,
                             float* dirty_grid, oc_accum* acc, int32_t nthreads);
void oc_wproj_degrid_f32(const oc_wproj* p, const float* kernels32, const float* model_grid,
                         int64_t n, const double* u, const double* v, const double* w,
                         float* pred, int32_t nthreads);

/* robust RMS of the n-sigma threshold (lib.rs:74130-74626) */
void oc_mean_stddev(const float* v, int64_t n, double* mean_out, double* std_out);
double oc_chauvenet_max_zscore(uint64_t npts);
int64_t oc_chauvenet_clip(float* v, int64_t n, double zscore, int32_t max_iterations);
double oc_madfm(const float* v, int64_t n, double* median_out);
float oc_robust_rms(const float* residual, const uint8_t* mask, int64_t n, double* madfm_out,
                    int64_t* count_out);

#ifdef __cplusplus
}
#endif
#endif
