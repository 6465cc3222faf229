/*
 * casa_oracle.c -- FP64 CPU restatement of the casa-imaging hot path.
 *
 * TEST INFRASTRUCTURE ONLY: the checker for the CUDA path and the timed CPU
 * baseline.  Nothing in the product library links or loads this file.
 *
 * The reference (bglenden/casa-rs, Rust) cannot be built here: no cargo or
 * rustc exists on either machine.  This file restates its arithmetic from the
 * source; each function names the reference function and lines it follows.
 * Float32 steps that the reference takes deliberately (tap products, density
 * cells, Briggs denominators, Hogbom updates) are kept in float32; the bulk
 * accumulations that the reference performs in float64 (standard grids,
 * sums of weights) are float64; W-projection accumulates in float64 as well,
 * so that this library is the FP64 ideal the GPU is measured against.
 *
 * Build: gcc -O2 -ffp-contract=off -fPIC -shared -pthread (see oracle/build.py).
 */
#include "casa_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* small parallel-for over contiguous chunks                                 */
/* ------------------------------------------------------------------------ */
typedef void (*oc_chunk_fn)(void* ctx, int64_t begin, int64_t end, int32_t worker);

typedef struct {
    oc_chunk_fn fn;
    void* ctx;
    int64_t begin, end;
    int32_t worker;
} oc_task;

static void* oc_task_main(void* arg) {
    oc_task* t = (oc_task*)arg;
    t->fn(t->ctx, t->begin, t->end, t->worker);
    return NULL;
}

/* Splits [0, n) into `workers` contiguous chunks in order, like the
 * reference's `div_ceil` chunking (lib.rs:71219-71224). */
static int32_t oc_parallel_chunks(int64_t n, int32_t workers, oc_chunk_fn fn, void* ctx) {
    if (workers < 1) workers = 1;
    if ((int64_t)workers > n) workers = (int32_t)(n > 0 ? n : 1);
    int64_t chunk = (n + workers - 1) / workers;
    if (workers == 1) {
        fn(ctx, 0, n, 0);
        return 1;
    }
    pthread_t* th = (pthread_t*)calloc((size_t)workers, sizeof(pthread_t));
    oc_task* tasks = (oc_task*)calloc((size_t)workers, sizeof(oc_task));
    int32_t used = 0;
    for (int32_t i = 0; i < workers; ++i) {
        int64_t b = (int64_t)i * chunk;
        int64_t e = b + chunk < n ? b + chunk : n;
        if (b >= e) break;
        tasks[i].fn = fn;
        tasks[i].ctx = ctx;
        tasks[i].begin = b;
        tasks[i].end = e;
        tasks[i].worker = i;
        pthread_create(&th[i], NULL, oc_task_main, &tasks[i]);
        used++;
    }
    for (int32_t i = 0; i < used; ++i) pthread_join(th[i], NULL);
    free(th);
    free(tasks);
    return used;
}

/* ------------------------------------------------------------------------ */
/* geometry                                                                  */
/* ------------------------------------------------------------------------ */

/* padded_len + casa_composite_padded_len + is_casa_composite_len
 * (gridder.rs:4152-4173). */
static int oc_is_composite(int64_t value) {
    const int64_t f[3] = {2, 3, 5};
    for (int i = 0; i < 3; ++i)
        while (value > 1 && value % f[i] == 0) value /= f[i];
    return value == 1;
}

int64_t oc_casa_composite_padded_len(int64_t image_len, double padding) {
    int64_t padded = (int64_t)floor(padding * (double)image_len - 0.5);
    if (padded < image_len) padded = image_len;
    if (padded % 2 != 0) padded += 1;
    while (!oc_is_composite(padded)) padded += 2;
    return padded;
}

/* image_blc (gridder.rs:401-404). */
void oc_image_blc(int64_t grid_len, int64_t image_len, int64_t* blc) {
    *blc = (grid_len - image_len + (grid_len % 2 == 0 ? 1 : 0)) / 2;
}

/* grdsf (gridder.rs:4230-4265): CASA's rational approximation of the
 * zero-order prolate spheroidal function.  `powi` is evaluated by repeated
 * squaring, as LLVM lowers it. */
double oc_grdsf(double nu) {
    static const double P0[5] = {8.203343e-2, -3.644705e-1, 6.278660e-1, -5.335581e-1,
                                 2.312756e-1};
    static const double P1[5] = {4.028559e-3, -3.697768e-2, 1.021332e-1, -1.201436e-1,
                                 6.412774e-2};
    static const double Q0[3] = {1.0, 8.212018e-1, 2.078043e-1};
    static const double Q1[3] = {1.0, 9.599102e-1, 2.918724e-1};
    if (!(nu >= 0.0 && nu <= 1.0)) return 0.0;
    const double* p;
    const double* q;
    double nu_end;
    if (nu < 0.75) {
        p = P0;
        q = Q0;
        nu_end = 0.75;
    } else {
        p = P1;
        q = Q1;
        nu_end = 1.0;
    }
    double d = nu * nu - nu_end * nu_end;
    double d2 = d * d;
    double pw[5] = {1.0, d, d2, d2 * d, d2 * d2};
    double num = 0.0, den = 0.0;
    for (int k = 0; k < 5; ++k) num = num + p[k] * pw[k];
    for (int k = 0; k < 3; ++k) den = den + q[k] * pw[k];
    return den == 0.0 ? 0.0 : num / den;
}

/* spheroidal_kernel (gridder.rs:4200-4209). */
float oc_spheroidal_kernel(double distance, double support) {
    if (!(isfinite(distance) && distance <= support)) return 0.0f;
    double nu = distance / support;
    if (nu > 1.0) return 0.0f;
    return (float)((1.0 - nu * nu) * oc_grdsf(nu));
}

/* Kernel table of StandardGridder::new_with_padding_factor
 * (gridder.rs:407-416): os*(S+1) entries, the first os*S filled. */
void oc_std_kernel_table(int32_t os, int32_t support, float* out) {
    int64_t len = (int64_t)os * (support + 1);
    for (int64_t i = 0; i < len; ++i) out[i] = 0.0f;
    for (int64_t i = 0; i < (int64_t)os * support; ++i) {
        double distance = (double)i / ((double)support * (double)os);
        out[i] = oc_spheroidal_kernel(distance * (double)support, (double)support);
    }
}

int32_t oc_std_tap_rows(int32_t os) { return 2 * (os / 2) + 1; }

/* build_normalized_tap_weights (gridder.rs:2026-2051): one row per offset in
 * [-os/2, os/2], each normalised by its float32 sum. */
void oc_std_normalized_taps(const float* table, int32_t table_len, int32_t os, int32_t support,
                            float* out) {
    int32_t half = os / 2;
    int32_t taps = 2 * support + 1;
    for (int32_t offset = -half; offset <= half; ++offset) {
        float* row = out + (int64_t)(offset + half) * taps;
        float norm = 0.0f;
        for (int32_t t = 0; t < taps; ++t) {
            int64_t delta = t - support;
            int64_t lookup = delta * os + offset;
            if (lookup < 0) lookup = -lookup;
            float wgt = lookup < table_len ? table[lookup] : 0.0f;
            row[t] = wgt;
            norm = norm + wgt;
        }
        if (norm > 0.0f)
            for (int32_t t = 0; t < taps; ++t) row[t] = row[t] / norm;
    }
}

/* build_correction_axis (gridder.rs:4175-4188). */
void oc_correction_axis(int64_t size, float* out) {
    double center = (double)size / 2.0;
    for (int64_t i = 0; i < size; ++i) {
        double nu = fabs((double)i - center) / center;
        if (nu < 0.0) nu = 0.0;
        if (nu > 1.0) nu = 1.0;
        double v = oc_grdsf(nu);
        out[i] = v > 1.0e-6 ? (float)(1.0 / v) : 0.0f;
    }
}

/* build_gridder_correction_axis (gridder.rs:4190-4198). */
void oc_gridder_correction_axis(int64_t size, float* out) {
    double center = (double)size / 2.0;
    for (int64_t i = 0; i < size; ++i) {
        double nu = fabs((double)i - center) / center;
        if (nu < 0.0) nu = 0.0;
        if (nu > 1.0) nu = 1.0;
        out[i] = (float)oc_grdsf(nu);
    }
}

/* build_sinc_axis (gridder.rs:4211-4228): float32 argument and float32 sin. */
void oc_sinc_axis(int64_t size, int64_t conv_sampling, float* out) {
    for (int64_t i = 0; i < size; ++i) {
        float offset = (float)(i - size / 2);
        float denom = (float)size * (float)conv_sampling;
        float arg = (float)(3.14159265358979323846 * (double)offset / (double)denom);
        out[i] = (i == size / 2) ? 1.0f : sinf(arg) / arg;
    }
}

/* ------------------------------------------------------------------------ */
/* standard gridder                                                          */
/* ------------------------------------------------------------------------ */

/* sample_tap_span + normalized_tap_weight_index (gridder.rs:1958-1995).
 * Rust f64::round is half-away-from-zero, which is C round(). */
int oc_std_tap_span(const oc_std_gridder* g, double coordinate, int64_t size, int64_t* start,
                    int64_t* weight_index) {
    if (!isfinite(coordinate)) return 0;
    if (!(fabs(coordinate) < 9.0e15)) return 0;
    int64_t anchor = (int64_t)round(coordinate);
    int64_t offset = (int64_t)round(((double)anchor - coordinate) * (double)g->oversampling);
    int64_t s = anchor - g->support;
    int64_t e = anchor + g->support;
    if (s < 0 || e >= size) return 0;
    int64_t idx = offset + g->oversampling / 2;
    if (idx < 0 || idx >= g->tap_rows) return 0;
    *start = s;
    *weight_index = idx;
    return 1;
}

/* plan_positive_taps with grid_coordinate_x/y (gridder.rs:540-566,
 * gridder.rs:1877-1886): x = u/du + Nx/2, y = -v/dv + Ny/2. */
int oc_std_plan(const oc_std_gridder* g, double u, double v, int64_t* x0, int64_t* y0,
                int64_t* wx, int64_t* wy) {
    double x = u / g->du + (double)g->gnx / 2.0;
    double y = -v / g->dv + (double)g->gny / 2.0;
    if (!oc_std_tap_span(g, x, g->gnx, x0, wx)) return 0;
    if (!oc_std_tap_span(g, y, g->gny, y0, wy)) return 0;
    return 1;
}

/* oc_std_plan over arrays: start cells and tap rows, -1 when rejected. */
void oc_std_plan_many(const oc_std_gridder* g, int64_t n, const double* u, const double* v,
                      int32_t* x0, int32_t* y0, int32_t* wx, int32_t* wy) {
    for (int64_t i = 0; i < n; ++i) {
        int64_t a, b, c, d;
        if (oc_std_plan(g, u[i], v[i], &a, &b, &c, &d)) {
            x0[i] = (int32_t)a;
            y0[i] = (int32_t)b;
            wx[i] = (int32_t)c;
            wy[i] = (int32_t)d;
        } else {
            x0[i] = y0[i] = wx[i] = wy[i] = -1;
        }
    }
}

static int oc_finite_f(float a) { return isfinite(a); }

typedef struct {
    const oc_std_gridder* g;
    const double *u, *v;
    const float *weight, *sumwt_factor, *vis;
    const uint8_t* gridable;
    double** psf;
    double** dirty;
    oc_accum* acc;
    const double* model;
    double* pred;
} oc_std_job;

/* accumulate_dirty_psf_and_residual_standard_streaming_grid_serial
 * (lib.rs:68433-68500) with grid_sample_taps_real_complex_pair_planned_f64
 * (gridder.rs:1021-1071): the tap product wx*wy is float32, promoted. */
static void oc_std_grid_chunk(void* vctx, int64_t b, int64_t e, int32_t worker) {
    oc_std_job* j = (oc_std_job*)vctx;
    const oc_std_gridder* g = j->g;
    const int32_t taps = 2 * g->support + 1;
    double* psf = j->psf[worker];
    double* dirty = j->dirty[worker];
    oc_accum* acc = &j->acc[worker];
    for (int64_t i = b; i < e; ++i) {
        if (j->gridable && !j->gridable[i]) {
            acc->skipped++;
            continue;
        }
        float w = j->weight[i];
        float f = j->sumwt_factor ? j->sumwt_factor[i] : 1.0f;
        if (!(oc_finite_f(w) && w > 0.0f && oc_finite_f(f) && f > 0.0f)) {
            acc->skipped++;
            continue;
        }
        int64_t x0, y0, wxi, wyi;
        if (!oc_std_plan(g, j->u[i], j->v[i], &x0, &y0, &wxi, &wyi)) {
            acc->skipped++;
            continue;
        }
        double gw = (double)(w * f);
        acc->normalization_sumwt += gw;
        acc->reported_sumwt += gw;
        acc->gridded++;
        float vr = j->vis[2 * i], vi = j->vis[2 * i + 1];
        int finite_vis = oc_finite_f(vr) && oc_finite_f(vi);
        double rr = (double)vr * gw, ri = (double)vi * gw;
        const float* xw = g->taps + wxi * taps;
        const float* yw = g->taps + wyi * taps;
        for (int32_t tx = 0; tx < taps; ++tx) {
            int64_t row = (x0 + tx) * g->gny;
            for (int32_t ty = 0; ty < taps; ++ty) {
                double wgt = (double)(xw[tx] * yw[ty]);
                int64_t cell = row + y0 + ty;
                psf[2 * cell] += gw * wgt;
                if (finite_vis) {
                    dirty[2 * cell] += rr * wgt;
                    dirty[2 * cell + 1] += ri * wgt;
                }
            }
        }
    }
}

static void oc_merge_grids(double* target, double** parts, int32_t nparts, int64_t len) {
    for (int32_t p = 0; p < nparts; ++p)
        for (int64_t k = 0; k < len; ++k) target[k] += parts[p][k];
}

void oc_std_grid_dirty(const oc_std_gridder* g, int64_t n, const double* u, const double* v,
                       const float* weight, const float* sumwt_factor, const uint8_t* gridable,
                       const float* vis, double* psf_grid, double* dirty_grid, oc_accum* acc,
                       int32_t nthreads) {
    if (nthreads < 1) nthreads = 1;
    if ((int64_t)nthreads > n) nthreads = (int32_t)(n > 0 ? n : 1);
    int64_t len = 2 * g->gnx * g->gny;
    oc_std_job j = {g, u, v, weight, sumwt_factor, vis, gridable, NULL, NULL, NULL, NULL, NULL};
    j.psf = (double**)calloc((size_t)nthreads, sizeof(double*));
    j.dirty = (double**)calloc((size_t)nthreads, sizeof(double*));
    j.acc = (oc_accum*)calloc((size_t)nthreads, sizeof(oc_accum));
    for (int32_t t = 0; t < nthreads; ++t) {
        if (nthreads == 1) {
            j.psf[t] = psf_grid;
            j.dirty[t] = dirty_grid;
        } else {
            j.psf[t] = (double*)calloc((size_t)len, sizeof(double));
            j.dirty[t] = (double*)calloc((size_t)len, sizeof(double));
        }
    }
    int32_t used = oc_parallel_chunks(n, nthreads, oc_std_grid_chunk, &j);
    memset(acc, 0, sizeof(*acc));
    for (int32_t t = 0; t < used; ++t) {
        acc->normalization_sumwt += j.acc[t].normalization_sumwt;
        acc->reported_sumwt += j.acc[t].reported_sumwt;
        acc->gridded += j.acc[t].gridded;
        acc->skipped += j.acc[t].skipped;
    }
    if (nthreads > 1) {
        oc_merge_grids(psf_grid, j.psf, used, len);
        oc_merge_grids(dirty_grid, j.dirty, used, len);
        for (int32_t t = 0; t < nthreads; ++t) {
            free(j.psf[t]);
            free(j.dirty[t]);
        }
    }
    free(j.psf);
    free(j.dirty);
    free(j.acc);
}

/* degrid_sample_taps_planned_normalized (gridder.rs:1278-1312), FP64 sum. */
void oc_std_degrid(const oc_std_gridder* g, const double* model, int64_t n, const double* u,
                   const double* v, double* pred) {
    const int32_t taps = 2 * g->support + 1;
    for (int64_t i = 0; i < n; ++i) {
        int64_t x0, y0, wxi, wyi;
        pred[2 * i] = 0.0;
        pred[2 * i + 1] = 0.0;
        if (!oc_std_plan(g, u[i], v[i], &x0, &y0, &wxi, &wyi)) continue;
        const float* xw = g->taps + wxi * taps;
        const float* yw = g->taps + wyi * taps;
        double re = 0.0, im = 0.0;
        for (int32_t tx = 0; tx < taps; ++tx) {
            int64_t row = (x0 + tx) * g->gny;
            for (int32_t ty = 0; ty < taps; ++ty) {
                double wgt = (double)(xw[tx] * yw[ty]);
                int64_t cell = row + y0 + ty;
                re += model[2 * cell] * wgt;
                im += model[2 * cell + 1] * wgt;
            }
        }
        pred[2 * i] = re;
        pred[2 * i + 1] = im;
    }
}

/* degrid_model_and_grid_residual_taps_planned_f64 (gridder.rs:1315-1396) as
 * driven by the standard residual refresh: residual = (vis - pred) * gw. */
static void oc_std_residual_chunk(void* vctx, int64_t b, int64_t e, int32_t worker) {
    oc_std_job* j = (oc_std_job*)vctx;
    const oc_std_gridder* g = j->g;
    const int32_t taps = 2 * g->support + 1;
    double* res = j->dirty[worker];
    oc_accum* acc = &j->acc[worker];
    for (int64_t i = b; i < e; ++i) {
        if (j->pred) {
            j->pred[2 * i] = 0.0;
            j->pred[2 * i + 1] = 0.0;
        }
        if (j->gridable && !j->gridable[i]) {
            acc->skipped++;
            continue;
        }
        float w = j->weight[i];
        float f = j->sumwt_factor ? j->sumwt_factor[i] : 1.0f;
        float vr = j->vis[2 * i], vi = j->vis[2 * i + 1];
        if (!(oc_finite_f(w) && w > 0.0f && oc_finite_f(f) && f > 0.0f &&
              oc_finite_f(vr) && oc_finite_f(vi))) {
            acc->skipped++;
            continue;
        }
        int64_t x0, y0, wxi, wyi;
        if (!oc_std_plan(g, j->u[i], j->v[i], &x0, &y0, &wxi, &wyi)) {
            acc->skipped++;
            continue;
        }
        double gw = (double)(w * f);
        acc->normalization_sumwt += gw;
        acc->reported_sumwt += gw;
        acc->gridded++;
        const float* xw = g->taps + wxi * taps;
        const float* yw = g->taps + wyi * taps;
        double pr = 0.0, pi = 0.0;
        if (j->model) {
            for (int32_t tx = 0; tx < taps; ++tx) {
                int64_t row = (x0 + tx) * g->gny;
                for (int32_t ty = 0; ty < taps; ++ty) {
                    double wgt = (double)(xw[tx] * yw[ty]);
                    int64_t cell = row + y0 + ty;
                    pr += j->model[2 * cell] * wgt;
                    pi += j->model[2 * cell + 1] * wgt;
                }
            }
        }
        if (j->pred) {
            j->pred[2 * i] = pr;
            j->pred[2 * i + 1] = pi;
        }
        double rr = ((double)vr - pr) * gw, ri = ((double)vi - pi) * gw;
        for (int32_t tx = 0; tx < taps; ++tx) {
            int64_t row = (x0 + tx) * g->gny;
            for (int32_t ty = 0; ty < taps; ++ty) {
                double wgt = (double)(xw[tx] * yw[ty]);
                int64_t cell = row + y0 + ty;
                res[2 * cell] += rr * wgt;
                res[2 * cell + 1] += ri * wgt;
            }
        }
    }
}

void oc_std_residual(const oc_std_gridder* g, const double* model_grid, int64_t n,
                     const double* u, const double* v, const float* weight,
                     const float* sumwt_factor, const uint8_t* gridable, const float* vis,
                     double* residual_grid, double* pred, oc_accum* acc, int32_t nthreads) {
    if (nthreads < 1) nthreads = 1;
    if ((int64_t)nthreads > n) nthreads = (int32_t)(n > 0 ? n : 1);
    int64_t len = 2 * g->gnx * g->gny;
    oc_std_job j = {g, u, v, weight, sumwt_factor, vis, gridable, NULL, NULL, NULL,
                    model_grid, pred};
    j.dirty = (double**)calloc((size_t)nthreads, sizeof(double*));
    j.acc = (oc_accum*)calloc((size_t)nthreads, sizeof(oc_accum));
    for (int32_t t = 0; t < nthreads; ++t)
        j.dirty[t] = nthreads == 1 ? residual_grid : (double*)calloc((size_t)len, sizeof(double));
    int32_t used = oc_parallel_chunks(n, nthreads, oc_std_residual_chunk, &j);
    memset(acc, 0, sizeof(*acc));
    for (int32_t t = 0; t < used; ++t) {
        acc->normalization_sumwt += j.acc[t].normalization_sumwt;
        acc->reported_sumwt += j.acc[t].reported_sumwt;
        acc->gridded += j.acc[t].gridded;
        acc->skipped += j.acc[t].skipped;
    }
    if (nthreads > 1) {
        oc_merge_grids(residual_grid, j.dirty, used, len);
        for (int32_t t = 0; t < nthreads; ++t) free(j.dirty[t]);
    }
    free(j.dirty);
    free(j.acc);
}

/* ------------------------------------------------------------------------ */
/* W-projection                                                              */
/* ------------------------------------------------------------------------ */

/* suggested_w_project_plane_count (gridder.rs:3822-3830). */
int64_t oc_wproj_suggested_planes(int64_t nx, int64_t ny, double cell_x, double cell_y,
                                  double max_abs_w) {
    if (!(isfinite(max_abs_w) && max_abs_w > 0.0)) return 1;
    double a = (double)nx * fabs(cell_x);
    double b = (double)ny * fabs(cell_y);
    double half = (a > b ? a : b) / 2.0;
    return (int64_t)(1.05 * max_abs_w * fabs(sin(half)));
}

/* w_project_max_uvw_lambda (gridder.rs:3808-3820). */
double oc_wproj_max_uvw(double cell_x, double max_abs_w, int explicit_planes) {
    return explicit_planes ? 0.25 / fabs(cell_x) : 1.05 * max_abs_w;
}

/* find_w_project_support_from_transformed (gridder.rs:3832-3855).  The
 * axis arrays hold |T(c,0)|/peak and |T(0,c)|/peak for c in [0, conv/2-1). */
int32_t oc_wproj_find_support(const double* axis_x, const double* axis_y, int64_t conv_size,
                              double peak, int32_t sampling) {
    (void)peak;
    int64_t quarter = conv_size / 2 - 1;
    int64_t trial = 0;
    int found = 0;
    for (int64_t c = quarter - 1; c >= 1; --c) {
        if (axis_x[c] > 1.0e-3 || axis_y[c] > 1.0e-3) {
            trial = c;
            found = 1;
            break;
        }
    }
    int64_t max_support = quarter / sampling - 1;
    int64_t floor1 = max_support > 1 ? max_support : 1;
    if (!found) return (int32_t)floor1;
    int64_t s = (int64_t)floorf((float)trial / (float)sampling + 0.5f) + 1;
    return (int32_t)(s < floor1 ? s : floor1);
}

typedef struct {
    int64_t conv, inner, half;
    double s0, s1, w_scale;
    int32_t planes, sampling;
    const double* corr;       /* [inner] */
    const double* tw_re;      /* [conv] */
    const double* tw_im;
    int32_t width_stride;     /* row stride of T_out */
    int32_t* crop;            /* [planes] columns needed per plane */
    int32_t axis_len;         /* entries of the support-search axes */
    double* out;              /* [planes][width_stride][width_stride] complex */
    double* axis_x;           /* [planes][axis_len] |T(c,0)| (unnormalised) */
    double* axis_y;
} oc_wk_job;

/* Screen of WProjector::new (gridder.rs:3437-3471) transformed by the forward
 * DFT of `fft2` (fft.rs:27-32), evaluated directly (FP64) only at the output
 * samples that the crop keeps.  T(x,y) = sum_ix sum_iy s(ix,iy)
 * exp(-2 pi i (x ix + y iy)/conv), separably. */
static void oc_wk_plane_chunk(void* vctx, int64_t b, int64_t e, int32_t worker) {
    (void)worker;
    oc_wk_job* j = (oc_wk_job*)vctx;
    const int64_t inner = j->inner, half = j->half, conv = j->conv;
    for (int64_t plane = b; plane < e; ++plane) {
        double w = j->planes > 1 ? (double)(plane * plane) / j->w_scale : 0.0;
        int64_t cw = j->crop[plane];
        int64_t alen = j->axis_len;
        int64_t ylen = cw > alen ? cw : alen;
        /* screen row by row; A[ix][y] = sum_iy s(ix,iy) tw(y*iy) */
        double* sre = (double*)calloc((size_t)inner, sizeof(double));
        double* sim = (double*)calloc((size_t)inner, sizeof(double));
        double* are = (double*)calloc((size_t)(inner * ylen), sizeof(double));
        double* aim = (double*)calloc((size_t)(inner * ylen), sizeof(double));
        double* colsum_re = (double*)calloc((size_t)inner, sizeof(double));
        double* colsum_im = (double*)calloc((size_t)inner, sizeof(double));
        for (int64_t ixi = 0; ixi < inner; ++ixi) {
            int64_t ix = ixi - half;
            double l = j->s0 * (double)ix;
            for (int64_t iyi = 0; iyi < inner; ++iyi) {
                int64_t iy = iyi - half;
                double m = j->s1 * (double)iy;
                double rsq = l * l + m * m;
                if (rsq >= 1.0) {
                    sre[iyi] = 0.0;
                    sim[iyi] = 0.0;
                    continue;
                }
                double phase = 6.283185307179586476925 * w * (sqrt(1.0 - rsq) - 1.0);
                double c = j->corr[ixi] * j->corr[iyi];
                sre[iyi] = c * cos(phase);
                sim[iyi] = c * sin(phase);
            }
            double csr = 0.0, csi = 0.0;
            for (int64_t iyi = 0; iyi < inner; ++iyi) {
                csr += sre[iyi];
                csi += sim[iyi];
            }
            colsum_re[ixi] = csr;
            colsum_im[ixi] = csi;
            for (int64_t y = 0; y < ylen; ++y) {
                double accr = 0.0, acci = 0.0;
                /* twiddle index (y * iy) mod conv, advanced by y per step */
                int64_t k = ((y * (-half)) % conv + conv) % conv;
                const int64_t step = y % conv;
                for (int64_t iyi = 0; iyi < inner; ++iyi) {
                    double tr = j->tw_re[k], ti = j->tw_im[k];
                    accr += sre[iyi] * tr - sim[iyi] * ti;
                    acci += sre[iyi] * ti + sim[iyi] * tr;
                    k += step;
                    if (k >= conv) k -= conv;
                }
                are[ixi * ylen + y] = accr;
                aim[ixi * ylen + y] = acci;
            }
        }
        /* T[x][y] = sum_ix tw(x*ix) A[ix][y] for x, y < cw */
        double* out = j->out + (size_t)plane * j->width_stride * j->width_stride * 2;
        double* tr_row = (double*)malloc((size_t)inner * sizeof(double));
        double* ti_row = (double*)malloc((size_t)inner * sizeof(double));
        double* accr = (double*)malloc((size_t)ylen * sizeof(double));
        double* acci = (double*)malloc((size_t)ylen * sizeof(double));
        for (int64_t x = 0; x < cw; ++x) {
            int64_t k = ((x * (-half)) % conv + conv) % conv;
            const int64_t step = x % conv;
            for (int64_t ixi = 0; ixi < inner; ++ixi) {
                tr_row[ixi] = j->tw_re[k];
                ti_row[ixi] = j->tw_im[k];
                k += step;
                if (k >= conv) k -= conv;
            }
            for (int64_t y = 0; y < cw; ++y) accr[y] = acci[y] = 0.0;
            for (int64_t ixi = 0; ixi < inner; ++ixi) {
                const double tr = tr_row[ixi], ti = ti_row[ixi];
                const double* ar = are + ixi * ylen;
                const double* ai = aim + ixi * ylen;
                for (int64_t y = 0; y < cw; ++y) {
                    accr[y] += ar[y] * tr - ai[y] * ti;
                    acci[y] += ar[y] * ti + ai[y] * tr;
                }
            }
            for (int64_t y = 0; y < cw; ++y) {
                out[2 * (x * j->width_stride + y)] = accr[y];
                out[2 * (x * j->width_stride + y) + 1] = acci[y];
            }
        }
        free(tr_row);
        free(ti_row);
        free(accr);
        free(acci);
        /* support-search axes: T(c,0) = sum_ix tw(c*ix) colsum(ix);
         * T(0,c) = sum_ix A[ix][c] */
        for (int64_t c = 0; c < alen; ++c) {
            double accr = 0.0, acci = 0.0, br = 0.0, bi = 0.0;
            for (int64_t ixi = 0; ixi < inner; ++ixi) {
                int64_t ix = ixi - half;
                int64_t k = ((c * ix) % conv + conv) % conv;
                double tr = j->tw_re[k], ti = j->tw_im[k];
                accr += colsum_re[ixi] * tr - colsum_im[ixi] * ti;
                acci += colsum_re[ixi] * ti + colsum_im[ixi] * tr;
                br += are[ixi * ylen + c];
                bi += aim[ixi * ylen + c];
            }
            j->axis_x[plane * alen + c] = sqrt(accr * accr + acci * acci);
            j->axis_y[plane * alen + c] = sqrt(br * br + bi * bi);
        }
        free(sre);
        free(sim);
        free(are);
        free(aim);
        free(colsum_re);
        free(colsum_im);
    }
}

static void oc_wk_run(oc_wk_job* j, int32_t nthreads) {
    oc_parallel_chunks(j->planes, nthreads, oc_wk_plane_chunk, j);
}

/* w_project_plane_sum (gridder.rs:3991-4002). */
static double oc_plane_sum(const double* k, int32_t width, int32_t support, int32_t sampling) {
    double sum = 0.0;
    for (int32_t iy = -support; iy <= support; ++iy) {
        int64_t ky = llabs((int64_t)iy * sampling);
        for (int32_t ix = -support; ix <= support; ++ix) {
            int64_t kx = llabs((int64_t)ix * sampling);
            sum += k[2 * (kx * width + ky)];
        }
    }
    return sum;
}

/* compute_w_project_sample_normalization (gridder.rs:3782-3799). */
static int oc_sample_norm(const double* k, int32_t width, int32_t support, int32_t sampling,
                          int64_t off_x, int64_t off_y, double* out) {
    double n = 0.0;
    for (int32_t iy = -support; iy <= support; ++iy) {
        int64_t ky = llabs((int64_t)iy * sampling + off_y);
        for (int32_t ix = -support; ix <= support; ++ix) {
            int64_t kx = llabs((int64_t)ix * sampling + off_x);
            if (kx >= width || ky >= width) return 0;
            n += k[2 * (kx * width + ky)];
        }
    }
    *out = n;
    return 1;
}

/* WProjector::new (gridder.rs:3403-3586).  support_min > 0 selects the
 * support law S_p = support_min + round((support_max - support_min) p/(P-1));
 * support_min <= 0 selects the reference's threshold search.  Kernels are
 * written at the common width [planes][width][width] (complex, x-major),
 * divided by the plane-zero peak and by the plane-zero integral, and the
 * per-(plane, off_x, off_y) normalisation table is filled.  Returns 0 on
 * success, 1 for invalid arguments, 2 for a zero plane-zero peak or integral,
 * 3 when the widest kernel exceeds max_width. */
int oc_wproj_build(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t gnx,
                   int64_t gny, double max_abs_w, int32_t planes, int explicit_planes,
                   int32_t sampling, int32_t support_min, int32_t support_max,
                   int32_t max_width, int32_t nthreads, double* w_scale_out,
                   int32_t* support_out, int32_t* width_out, double* kernels_out,
                   double* norm_out) {
    (void)nx;
    (void)ny;
    if (planes < 1 || sampling < 1) return 1;
    int64_t conv = gnx > gny ? gnx : gny;
    int64_t inner = conv / sampling;
    if (inner < 2) inner = 2;
    int64_t half = inner / 2;
    int64_t quarter = conv / 2 - 1;
    int32_t r = (sampling + 1) / 2;
    double* corr = (double*)calloc((size_t)inner, sizeof(double));
    {
        double center = (double)inner / 2.0;
        for (int64_t i = 0; i < inner; ++i) {
            double nu = fabs((double)i - center) / center;
            if (nu > 1.0) nu = 1.0;
            corr[i] = (double)(float)oc_grdsf(nu);
        }
    }
    double s0 = fabs(cell_x) * (double)sampling * (double)gnx / (double)conv;
    double s1 = fabs(cell_y) * (double)sampling * (double)gny / (double)conv;
    double eff = oc_wproj_max_uvw(cell_x, max_abs_w, explicit_planes);
    double w_scale = (planes > 1 && isfinite(eff) && eff > 0.0)
                         ? (double)((int64_t)(planes - 1) * (planes - 1)) / eff
                         : 1.0;
    *w_scale_out = w_scale;

    /* output crop widths */
    int32_t* crop = (int32_t*)calloc((size_t)planes, sizeof(int32_t));
    int law = support_min > 0;
    if (law) {
        for (int32_t p = 0; p < planes; ++p) {
            double frac = planes > 1 ? (double)p / (double)(planes - 1) : 0.0;
            int32_t s = support_min + (int32_t)llround((double)(support_max - support_min) * frac);
            support_out[p] = s;
            int64_t cw = (int64_t)s * sampling + r + 1;
            if (cw > quarter) {
                free(corr);
                free(crop);
                return 1;
            }
            crop[p] = (int32_t)cw;
        }
    } else {
        /* the threshold search needs the full axes; the crop is bounded by the
         * largest support the search can return */
        int64_t max_support = quarter / sampling - 1;
        if (max_support < 1) max_support = 1;
        int64_t cw = max_support * sampling + r + 1;
        if (cw > quarter) cw = quarter;
        if (cw < 1) cw = 1;
        for (int32_t p = 0; p < planes; ++p) crop[p] = (int32_t)cw;
    }
    int32_t stride = 0;
    for (int32_t p = 0; p < planes; ++p)
        if (crop[p] > stride) stride = crop[p];
    double* tw_re = (double*)malloc((size_t)conv * sizeof(double));
    double* tw_im = (double*)malloc((size_t)conv * sizeof(double));
    for (int64_t k = 0; k < conv; ++k) {
        double a = 6.283185307179586476925 * (double)k / (double)conv;
        tw_re[k] = cos(a);
        tw_im[k] = -sin(a);
    }
    int32_t axis_len = law ? 1 : (int32_t)(quarter > 1 ? quarter : 1);
    double* raw = (double*)calloc((size_t)planes * stride * stride * 2, sizeof(double));
    double* axis_x = (double*)calloc((size_t)planes * axis_len, sizeof(double));
    double* axis_y = (double*)calloc((size_t)planes * axis_len, sizeof(double));
    oc_wk_job job = {conv, inner, half, s0, s1, w_scale, planes, sampling, corr, tw_re,
                     tw_im, stride, crop, axis_len, raw, axis_x, axis_y};
    oc_wk_run(&job, nthreads);

    int rc = 0;
    double peak = hypot(raw[0], raw[1]);
    if (!(peak > 0.0)) rc = 2;
    int32_t width = 0;
    if (rc == 0) {
        for (int32_t p = 0; p < planes; ++p) {
            if (!law) {
                double* ax = axis_x + (size_t)p * axis_len;
                double* ay = axis_y + (size_t)p * axis_len;
                for (int32_t c = 0; c < axis_len; ++c) {
                    ax[c] /= peak;
                    ay[c] /= peak;
                }
                support_out[p] = oc_wproj_find_support(ax, ay, conv, peak, sampling);
                int64_t cw = (int64_t)support_out[p] * sampling + r + 1;
                if (cw > quarter) cw = quarter;
                if (cw < 1) cw = 1;
                crop[p] = (int32_t)cw;
            }
            if (crop[p] > width) width = crop[p];
        }
        if (width > max_width) rc = 3;
    }
    if (rc == 0) {
        *width_out = width;
        memset(kernels_out, 0, (size_t)planes * width * width * 2 * sizeof(double));
        for (int32_t p = 0; p < planes; ++p) {
            const double* src = raw + (size_t)p * stride * stride * 2;
            double* dst = kernels_out + (size_t)p * width * width * 2;
            for (int32_t x = 0; x < crop[p]; ++x)
                for (int32_t y = 0; y < crop[p]; ++y) {
                    dst[2 * (x * width + y)] = src[2 * (x * stride + y)] / peak;
                    dst[2 * (x * width + y) + 1] = src[2 * (x * stride + y) + 1] / peak;
                }
        }
        double pb = oc_plane_sum(kernels_out, width, support_out[0], sampling);
        if (!(isfinite(pb) && pb > 0.0)) rc = 2;
        if (rc == 0) {
            size_t total = (size_t)planes * width * width * 2;
            for (size_t k = 0; k < total; ++k) kernels_out[k] /= pb;
            int32_t L = 2 * r + 1;
            for (int32_t p = 0; p < planes; ++p) {
                const double* kp = kernels_out + (size_t)p * width * width * 2;
                for (int32_t ox = -r; ox <= r; ++ox)
                    for (int32_t oy = -r; oy <= r; ++oy) {
                        double nrm = 0.0;
                        if (!oc_sample_norm(kp, width, support_out[p], sampling, ox, oy, &nrm))
                            nrm = 0.0;
                        norm_out[(size_t)p * L * L + (size_t)(ox + r) * L + (oy + r)] = nrm;
                    }
            }
        }
    }
    free(corr);
    free(crop);
    free(tw_re);
    free(tw_im);
    free(raw);
    free(axis_x);
    free(axis_y);
    return rc;
}

/* w_plane_index (gridder.rs:3759-3767). */
int32_t oc_wproj_plane_index(const oc_wproj* p, double w) {
    if (p->planes <= 1) return 0;
    double c = p->w_scale * fabs(w);
    if (c < 0.0) c = 0.0;
    c = sqrt(c);
    double r = round(c);
    if (r < 0.0) r = 0.0;
    if (r > (double)(p->planes - 1)) r = (double)(p->planes - 1);
    return (int32_t)r;
}

/* WProjector::plan_sample (gridder.rs:3588-3624). */
int oc_wproj_plan(const oc_wproj* p, double u, double v, double w, int64_t* loc_x,
                  int64_t* loc_y, int64_t* off_x, int64_t* off_y, int32_t* plane,
                  int32_t* conj, double* normalization) {
    double px = u / p->du + (double)p->gnx / 2.0;
    double py = -v / p->dv + (double)p->gny / 2.0;
    if (!(isfinite(px) && isfinite(py) && isfinite(w))) return 0;
    if (!(fabs(px) < 9.0e15 && fabs(py) < 9.0e15)) return 0;
    int64_t lx = (int64_t)round(px), ly = (int64_t)round(py);
    int64_t ox = (int64_t)round(((double)lx - px) * (double)p->sampling);
    int64_t oy = (int64_t)round(((double)ly - py) * (double)p->sampling);
    int32_t pl = oc_wproj_plane_index(p, w);
    int64_t s = p->support[pl];
    if (s <= 0 || lx - s < 0 || ly - s < 0 || lx + s >= p->gnx || ly + s >= p->gny) return 0;
    double nrm;
    int32_t r = p->norm_radius;
    if (llabs(ox) <= r && llabs(oy) <= r) {
        int32_t L = 2 * r + 1;
        nrm = p->norm_table[(size_t)pl * L * L + (size_t)(ox + r) * L + (oy + r)];
    } else {
        const double* kp = p->kernels + (size_t)pl * p->width * p->width * 2;
        if (!oc_sample_norm(kp, p->width, (int32_t)s, p->sampling, ox, oy, &nrm)) return 0;
    }
    *loc_x = lx;
    *loc_y = ly;
    *off_x = ox;
    *off_y = oy;
    *plane = pl;
    *conj = w > 0.0;
    *normalization = nrm;
    return 1;
}

/* raw_w_project_sample_is_valid (lib.rs:73666-73676) plus the gridable flag. */
static int oc_wproj_sample_valid(const uint8_t* gridable, int64_t i, float w, float f, float vr,
                                 float vi, double u, double v, double ww) {
    if (gridable && !gridable[i]) return 0;
    return isfinite(w) && w > 0.0f && isfinite(f) && f > 0.0f && isfinite(vr) &&
           isfinite(vi) && isfinite(u) && isfinite(v) && isfinite(ww);
}

typedef struct {
    const oc_wproj* p;
    const double *u, *v, *w;
    const float *weight, *sumwt_factor, *vis;
    const uint8_t* gridable;
    double** psf;
    double** dirty;
    oc_accum* acc;
    const double* model;
    double* pred;
} oc_wp_job;

/* accumulate_w_project_dirty_streaming_sample (lib.rs:71487-71512) with
 * grid_sample_planned_pair (gridder.rs:3701-3724), FP64 accumulation. */
static void oc_wp_grid_chunk(void* vctx, int64_t b, int64_t e, int32_t worker) {
    oc_wp_job* j = (oc_wp_job*)vctx;
    const oc_wproj* p = j->p;
    double* psf = j->psf[worker];
    double* dirty = j->dirty[worker];
    oc_accum* acc = &j->acc[worker];
    for (int64_t i = b; i < e; ++i) {
        float wt = j->weight[i];
        float f = j->sumwt_factor ? j->sumwt_factor[i] : 1.0f;
        float vr = j->vis[2 * i], vi = j->vis[2 * i + 1];
        if (!oc_wproj_sample_valid(j->gridable, i, wt, f, vr, vi, j->u[i], j->v[i], j->w[i])) {
            acc->skipped++;
            continue;
        }
        int64_t lx, ly, ox, oy;
        int32_t pl, cj;
        double nrm;
        if (!oc_wproj_plan(p, j->u[i], j->v[i], j->w[i], &lx, &ly, &ox, &oy, &pl, &cj, &nrm)) {
            acc->skipped++;
            continue;
        }
        acc->normalization_sumwt += 2.0 * (double)wt * nrm;
        acc->reported_sumwt += (double)wt * (double)f;
        acc->gridded++;
        double pw = (double)wt;
        double dr = (double)vr * (double)wt, di = (double)vi * (double)wt;
        const double* k = p->kernels + (size_t)pl * p->width * p->width * 2;
        int32_t s = p->support[pl];
        double sg = cj ? -1.0 : 1.0;
        for (int32_t iy = -s; iy <= s; ++iy) {
            int64_t ky = llabs((int64_t)iy * p->sampling + oy);
            for (int32_t ix = -s; ix <= s; ++ix) {
                int64_t kx = llabs((int64_t)ix * p->sampling + ox);
                double kr = k[2 * (kx * p->width + ky)];
                double ki = sg * k[2 * (kx * p->width + ky) + 1];
                int64_t cell = (lx + ix) * p->gny + (ly + iy);
                psf[2 * cell] += pw * kr;
                psf[2 * cell + 1] += pw * ki;
                dirty[2 * cell] += dr * kr - di * ki;
                dirty[2 * cell + 1] += dr * ki + di * kr;
            }
        }
    }
}

void oc_wproj_grid_dirty(const oc_wproj* p, int64_t n, const double* u, const double* v,
                         const double* w, const float* weight, const float* sumwt_factor,
                         const uint8_t* gridable, const float* vis, double* psf_grid,
                         double* dirty_grid, oc_accum* acc, int32_t nthreads) {
    if (nthreads < 1) nthreads = 1;
    if ((int64_t)nthreads > n) nthreads = (int32_t)(n > 0 ? n : 1);
    int64_t len = 2 * p->gnx * p->gny;
    oc_wp_job j = {p, u, v, w, weight, sumwt_factor, vis, gridable, NULL, NULL, NULL, NULL,
                   NULL};
    j.psf = (double**)calloc((size_t)nthreads, sizeof(double*));
    j.dirty = (double**)calloc((size_t)nthreads, sizeof(double*));
    j.acc = (oc_accum*)calloc((size_t)nthreads, sizeof(oc_accum));
    for (int32_t t = 0; t < nthreads; ++t) {
        j.psf[t] = nthreads == 1 ? psf_grid : (double*)calloc((size_t)len, sizeof(double));
        j.dirty[t] = nthreads == 1 ? dirty_grid : (double*)calloc((size_t)len, sizeof(double));
    }
    int32_t used = oc_parallel_chunks(n, nthreads, oc_wp_grid_chunk, &j);
    memset(acc, 0, sizeof(*acc));
    for (int32_t t = 0; t < used; ++t) {
        acc->normalization_sumwt += j.acc[t].normalization_sumwt;
        acc->reported_sumwt += j.acc[t].reported_sumwt;
        acc->gridded += j.acc[t].gridded;
        acc->skipped += j.acc[t].skipped;
    }
    if (nthreads > 1) {
        oc_merge_grids(psf_grid, j.psf, used, len);
        oc_merge_grids(dirty_grid, j.dirty, used, len);
        for (int32_t t = 0; t < nthreads; ++t) {
            free(j.psf[t]);
            free(j.dirty[t]);
        }
    }
    free(j.psf);
    free(j.dirty);
    free(j.acc);
}

/* degrid_sample_planned (gridder.rs:3726-3747): sum conj(cwt) * grid. */
static void oc_wp_degrid_one(const oc_wproj* p, const double* g, int64_t lx, int64_t ly,
                             int64_t ox, int64_t oy, int32_t pl, int32_t cj, double* pr,
                             double* pi) {
    const double* k = p->kernels + (size_t)pl * p->width * p->width * 2;
    int32_t s = p->support[pl];
    double sg = cj ? -1.0 : 1.0;
    double re = 0.0, im = 0.0;
    for (int32_t iy = -s; iy <= s; ++iy) {
        int64_t ky = llabs((int64_t)iy * p->sampling + oy);
        for (int32_t ix = -s; ix <= s; ++ix) {
            int64_t kx = llabs((int64_t)ix * p->sampling + ox);
            double kr = k[2 * (kx * p->width + ky)];
            double ki = -sg * k[2 * (kx * p->width + ky) + 1]; /* conj(cwt) */
            int64_t cell = (lx + ix) * p->gny + (ly + iy);
            double gr = g[2 * cell], gi = g[2 * cell + 1];
            re += kr * gr - ki * gi;
            im += kr * gi + ki * gr;
        }
    }
    *pr = re;
    *pi = im;
}

static void oc_wp_degrid_chunk(void* vctx, int64_t b, int64_t e, int32_t worker) {
    (void)worker;
    oc_wp_job* j = (oc_wp_job*)vctx;
    for (int64_t i = b; i < e; ++i) {
        int64_t lx, ly, ox, oy;
        int32_t pl, cj;
        double nrm;
        j->pred[2 * i] = 0.0;
        j->pred[2 * i + 1] = 0.0;
        if (!oc_wproj_plan(j->p, j->u[i], j->v[i], j->w[i], &lx, &ly, &ox, &oy, &pl, &cj, &nrm))
            continue;
        oc_wp_degrid_one(j->p, j->model, lx, ly, ox, oy, pl, cj, &j->pred[2 * i],
                         &j->pred[2 * i + 1]);
    }
}

void oc_wproj_degrid(const oc_wproj* p, const double* model_grid, int64_t n, const double* u,
                     const double* v, const double* w, double* pred, int32_t nthreads) {
    oc_wp_job j = {p, u, v, w, NULL, NULL, NULL, NULL, NULL, NULL, NULL, model_grid, pred};
    oc_parallel_chunks(n, nthreads, oc_wp_degrid_chunk, &j);
}

/* accumulate_w_project_residual_streaming_sample (lib.rs:71514-71541):
 * residual = (vis - pred) * weight, gridded with the same kernel. */
static void oc_wp_residual_chunk(void* vctx, int64_t b, int64_t e, int32_t worker) {
    oc_wp_job* j = (oc_wp_job*)vctx;
    const oc_wproj* p = j->p;
    double* res = j->dirty[worker];
    oc_accum* acc = &j->acc[worker];
    for (int64_t i = b; i < e; ++i) {
        float wt = j->weight[i];
        float f = j->sumwt_factor ? j->sumwt_factor[i] : 1.0f;
        float vr = j->vis[2 * i], vi = j->vis[2 * i + 1];
        if (!oc_wproj_sample_valid(j->gridable, i, wt, f, vr, vi, j->u[i], j->v[i], j->w[i])) {
            acc->skipped++;
            continue;
        }
        int64_t lx, ly, ox, oy;
        int32_t pl, cj;
        double nrm;
        if (!oc_wproj_plan(p, j->u[i], j->v[i], j->w[i], &lx, &ly, &ox, &oy, &pl, &cj, &nrm)) {
            acc->skipped++;
            continue;
        }
        acc->normalization_sumwt += 2.0 * (double)wt * nrm;
        acc->reported_sumwt += (double)wt * (double)f;
        acc->gridded++;
        double pr = 0.0, pi = 0.0;
        if (j->model) oc_wp_degrid_one(p, j->model, lx, ly, ox, oy, pl, cj, &pr, &pi);
        double rr = ((double)vr - pr) * (double)wt, ri = ((double)vi - pi) * (double)wt;
        const double* k = p->kernels + (size_t)pl * p->width * p->width * 2;
        int32_t s = p->support[pl];
        double sg = cj ? -1.0 : 1.0;
        for (int32_t iy = -s; iy <= s; ++iy) {
            int64_t ky = llabs((int64_t)iy * p->sampling + oy);
            for (int32_t ix = -s; ix <= s; ++ix) {
                int64_t kx = llabs((int64_t)ix * p->sampling + ox);
                double kr = k[2 * (kx * p->width + ky)];
                double ki = sg * k[2 * (kx * p->width + ky) + 1];
                int64_t cell = (lx + ix) * p->gny + (ly + iy);
                res[2 * cell] += rr * kr - ri * ki;
                res[2 * cell + 1] += rr * ki + ri * kr;
            }
        }
    }
}

void oc_wproj_residual(const oc_wproj* p, const double* model_grid, int64_t n,
                       const double* u, const double* v, const double* w, const float* weight,
                       const float* sumwt_factor, const uint8_t* gridable, const float* vis,
                       double* residual_grid, oc_accum* acc, int32_t nthreads) {
    if (nthreads < 1) nthreads = 1;
    if ((int64_t)nthreads > n) nthreads = (int32_t)(n > 0 ? n : 1);
    int64_t len = 2 * p->gnx * p->gny;
    oc_wp_job j = {p, u, v, w, weight, sumwt_factor, vis, gridable, NULL, NULL, NULL,
                   model_grid, NULL};
    j.dirty = (double**)calloc((size_t)nthreads, sizeof(double*));
    j.acc = (oc_accum*)calloc((size_t)nthreads, sizeof(oc_accum));
    for (int32_t t = 0; t < nthreads; ++t)
        j.dirty[t] = nthreads == 1 ? residual_grid : (double*)calloc((size_t)len, sizeof(double));
    int32_t used = oc_parallel_chunks(n, nthreads, oc_wp_residual_chunk, &j);
    memset(acc, 0, sizeof(*acc));
    for (int32_t t = 0; t < used; ++t) {
        acc->normalization_sumwt += j.acc[t].normalization_sumwt;
        acc->reported_sumwt += j.acc[t].reported_sumwt;
        acc->gridded += j.acc[t].gridded;
        acc->skipped += j.acc[t].skipped;
    }
    if (nthreads > 1) {
        oc_merge_grids(residual_grid, j.dirty, used, len);
        for (int32_t t = 0; t < nthreads; ++t) free(j.dirty[t]);
    }
    free(j.dirty);
    free(j.acc);
}

/* ------------------------------------------------------------------------ */
/* weighting                                                                 */
/* ------------------------------------------------------------------------ */

/* weight_density_cell_anchor (gridder.rs:1888-1934).  convention 0 is
 * VisImagingWeight (float32 u, v, scale and origin; separate multiply and
 * add; truncation), convention 1 the cube Briggs rounding. */
int oc_density_cell(int64_t nx, int64_t ny, double cell_x, double cell_y, double u, double v,
                    int convention, int64_t* cx, int64_t* cy) {
    double cxd = (double)nx / 2.0, cyd = (double)ny / 2.0;
    double us = (double)nx * cell_x, vs = (double)ny * cell_y;
    double x, y;
    if (convention == 0) {
        float uf = (float)u, vf = (float)v;
        float xs = (-uf) * (float)us;
        float ys = vf * (float)vs;
        float xf = xs + (float)cxd;
        float yf = ys + (float)cyd;
        x = (double)xf;
        y = (double)yf;
    } else {
        x = u * us + cxd;
        y = -v * vs + cyd;
    }
    if (!(isfinite(x) && isfinite(y))) return 0;
    if (convention == 0) {
        /* trunc(x) in (0, nx)  <=>  1 <= x < nx */
        if (!(x >= 1.0 && x < (double)nx && y >= 1.0 && y < (double)ny)) return 0;
        *cx = (int64_t)x;
        *cy = (int64_t)y;
    } else {
        double rx = round(x), ry = round(y);
        if (!(rx >= 1.0 && rx < (double)nx && ry >= 1.0 && ry < (double)ny)) return 0;
        *cx = (int64_t)rx;
        *cy = (int64_t)ry;
    }
    return 1;
}

/* build_density_grid_serial / accumulate_density_sample_serial
 * (weighting.rs:1747-1854) with the Hermitian mirror, at the cells of
 * `convention` (0 VisImagingWeight, 1 the cube PerPlane rounding of
 * density_build_cell_convention, weighting.rs:1470-1483). */
void oc_density_grid_conv(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t n,
                          const double* u, const double* v, const float* weight, int convention,
                          float* density) {
    memset(density, 0, (size_t)(nx * ny) * sizeof(float));
    for (int64_t i = 0; i < n; ++i) {
        float w = weight[i];
        if (!(isfinite(w) && w > 0.0f)) continue;
        int64_t x, y;
        if (oc_density_cell(nx, ny, cell_x, cell_y, u[i], v[i], convention, &x, &y))
            density[x * ny + y] = density[x * ny + y] + w;
        if (oc_density_cell(nx, ny, cell_x, cell_y, -u[i], -v[i], convention, &x, &y))
            density[x * ny + y] = density[x * ny + y] + w;
    }
}

void oc_density_grid(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t n,
                     const double* u, const double* v, const float* weight, float* density) {
    oc_density_grid_conv(nx, ny, cell_x, cell_y, n, u, v, weight, 0, density);
}

/* Briggs f2 of apply_weighting_with_density_source (weighting.rs:1108-1121):
 * f2 = (5 * 10^-robust)^2 / (sum d^2 / sum d) with FP64 sums in array order. */
float oc_briggs_f2(const float* density, int64_t cells, float robust) {
    double total = 0.0, sumsq = 0.0;
    for (int64_t k = 0; k < cells; ++k) total += (double)density[k];
    for (int64_t k = 0; k < cells; ++k)
        if (density[k] > 0.0f) sumsq += (double)density[k] * (double)density[k];
    if (!(sumsq > 0.0 && total > 0.0)) return 0.0f;
    double a = 5.0 * pow(10.0, -(double)robust);
    return (float)(a * a / (sumsq / total));
}

/* casa_briggs_denominator (weighting.rs:2440-2443): separate float ops. */
float oc_briggs_denominator(float density, float f2) {
    float product = density * f2;
    return product + 1.0f;
}

/* reweight_batch (weighting.rs:2094-2150): mode 0 natural, 1 uniform,
 * 2 Briggs; density looked up at the cells of `convention`. */
void oc_reweight_conv(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t n,
                      const double* u, const double* v, const float* weight,
                      const float* density, int mode, float f2, int convention,
                      float* out_weight) {
    for (int64_t i = 0; i < n; ++i) {
        float w = weight[i];
        if (mode == 0) {
            out_weight[i] = w;
            continue;
        }
        int64_t x, y;
        if (!oc_density_cell(nx, ny, cell_x, cell_y, u[i], v[i], convention, &x, &y)) {
            out_weight[i] = 0.0f;
            continue;
        }
        float d = density[x * ny + y];
        if (!(isfinite(w) && w > 0.0f && isfinite(d) && d > 0.0f)) {
            out_weight[i] = 0.0f;
            continue;
        }
        out_weight[i] = mode == 1 ? w / d : w / oc_briggs_denominator(d, f2);
    }
}

void oc_reweight(int64_t nx, int64_t ny, double cell_x, double cell_y, int64_t n,
                 const double* u, const double* v, const float* weight, const float* density,
                 int mode, float f2, float* out_weight) {
    oc_reweight_conv(nx, ny, cell_x, cell_y, n, u, v, weight, density, mode, f2, 0, out_weight);
}

/* ------------------------------------------------------------------------ */
/* Hogbom                                                                    */
/* ------------------------------------------------------------------------ */

/* peak_location_masked_in_bounds_zero_tolerance (lib.rs:74064-74118) over
 * the full image: largest |value|, ties to the smallest y*nx + x. */
int oc_peak_location(const float* image, const uint8_t* mask, int64_t nx, int64_t ny,
                     int64_t* px, int64_t* py, float* value) {
    int have = 0;
    float best = 0.0f;
    int64_t bx = 0, by = 0, bkey = 0;
    for (int64_t x = 0; x < nx; ++x) {
        for (int64_t y = 0; y < ny; ++y) {
            if (mask && !mask[x * ny + y]) continue;
            float val = image[x * ny + y];
            int64_t key = y * nx + x;
            if (!have) {
                have = 1;
                best = val;
                bx = x;
                by = y;
                bkey = key;
            } else if (fabsf(val) > fabsf(best) || (fabsf(val) == fabsf(best) && key < bkey)) {
                best = val;
                bx = x;
                by = y;
                bkey = key;
            }
        }
    }
    if (!have) return 0;
    *px = bx;
    *py = by;
    *value = best;
    return 1;
}

static int oc_threshold_reached(float peak, float thr) {
    if (thr <= 0.0f) return peak <= thr;
    float tol = 0.01f * thr;
    if (tol < 2.0e-8f) tol = 2.0e-8f;
    return peak <= thr || fabsf(peak - thr) <= tol;
}

/* minor_cycle_stop_reason (lib.rs:74653-74676).  Returns 0 for none,
 * 1 global threshold, 2 cycle threshold, 3 nsigma threshold. */
int oc_minor_cycle_stop_reason(float peak_abs, float threshold, float cycle_threshold,
                               float nsigma_threshold) {
    int floor_active = threshold > 0.0f && (0.01f * threshold) < 2.0e-8f &&
                       cycle_threshold <= threshold;
    if (peak_abs < threshold || (floor_active && oc_threshold_reached(peak_abs, threshold)))
        return 1;
    if (cycle_threshold >= nsigma_threshold) return peak_abs < cycle_threshold ? 2 : 0;
    if (nsigma_threshold > threshold) return peak_abs < nsigma_threshold ? 3 : 0;
    return 0;
}

/* subtract_shifted_kernel_in_window over the full image (lib.rs:74805-74870):
 * residual(x,y) -= component * psf(x - px + cx, y - py + cy), float32. */
void oc_subtract_shifted_psf(float* residual, const float* psf, int64_t nx, int64_t ny,
                             int64_t px, int64_t py, float component) {
    int64_t kcx = nx / 2, kcy = ny / 2;
    int64_t kx0 = px - kcx, ky0 = py - kcy;
    int64_t x0 = kx0 > 0 ? kx0 : 0, y0 = ky0 > 0 ? ky0 : 0;
    int64_t x1 = kx0 + nx - 1 < nx - 1 ? kx0 + nx - 1 : nx - 1;
    int64_t y1 = ky0 + ny - 1 < ny - 1 ? ky0 + ny - 1 : ny - 1;
    for (int64_t x = x0; x <= x1; ++x)
        for (int64_t y = y0; y <= y1; ++y) {
            float prod = component * psf[(x - kx0) * ny + (y - ky0)];
            residual[x * ny + y] = residual[x * ny + y] - prod;
        }
}

/* finite_peak_location_masked_with_relative_tolerance (lib.rs:73998-74026):
 * a y-major scan (x fastest) over finite unmasked values; a value replaces
 * the current peak only if |v| > |peak| * (1 + tol) in float32. */
int oc_peak_relative(const float* image, const uint8_t* mask, int64_t nx, int64_t ny,
                     float tol, int64_t* px, int64_t* py, float* value) {
    const float k1 = 1.0f + tol;
    int have = 0;
    float best = 0.0f;
    int64_t bx = 0, by = 0;
    for (int64_t y = 0; y < ny; ++y)
        for (int64_t x = 0; x < nx; ++x) {
            if (mask && !mask[x * ny + y]) continue;
            float v = image[x * ny + y];
            if (!isfinite(v)) continue;
            if (!have || fabsf(v) > fabsf(best) * k1) {
                have = 1;
                best = v;
                bx = x;
                by = y;
            }
        }
    if (!have) return 0;
    *px = bx;
    *py = by;
    *value = best;
    return 1;
}

/* run_hogbom_plane_minor_cycle (lib.rs:64630-64680): budget as
 * hogbom_component_budget, stop when |peak| <= threshold or <= the cycle
 * threshold; reported = min(actual, cycle_limit) (CasaInclusive). */
int64_t oc_hogbom_plane(float* model, float* residual, const float* psf, const uint8_t* mask,
                        int64_t nx, int64_t ny, float gain, float threshold,
                        float cycle_threshold, float tol, int64_t cycle_limit, int inclusive,
                        int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
                        int64_t* reported) {
    int64_t budget = inclusive ? cycle_limit + 1 : cycle_limit;
    int64_t updates = 0;
    while (updates < budget) {
        int64_t px, py;
        float pv;
        if (!oc_peak_relative(residual, mask, nx, ny, tol, &px, &py, &pv)) break;
        float pabs = fabsf(pv);
        if (pabs <= threshold || pabs <= cycle_threshold) break;
        float comp = gain * pv;
        model[px * ny + py] = model[px * ny + py] + comp;
        oc_subtract_shifted_psf(residual, psf, nx, ny, px, py, comp);
        if (comp_x) {
            comp_x[updates] = (int32_t)px;
            comp_y[updates] = (int32_t)py;
            comp_peak[updates] = pv;
            comp_flux[updates] = comp;
        }
        updates++;
    }
    *reported = updates < cycle_limit ? updates : cycle_limit;
    return updates;
}

/* run_hogbom_minor_cycle_cpu_with_progress (lib.rs:59748-59883) with
 * hogbom_component_budget (lib.rs:64541-64552).  Returns the number of
 * components; stop_reason 0 budget exhausted, 1 global, 2 cycle, 3 nsigma
 * threshold, 4 no cleanable pixels. */
int64_t oc_hogbom(float* model, float* residual, const float* psf, const uint8_t* mask,
                  int64_t nx, int64_t ny, float gain, float threshold, float cycle_threshold,
                  float nsigma_threshold, int64_t cycle_niter, int inclusive,
                  int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
                  int32_t* stop_reason, int64_t* reported) {
    int64_t budget = inclusive ? cycle_niter + 1 : cycle_niter;
    int64_t updates = 0;
    int32_t stop = 0;
    while (updates < budget) {
        int64_t px, py;
        float pv;
        if (!oc_peak_location(residual, mask, nx, ny, &px, &py, &pv)) {
            stop = 4;
            break;
        }
        int reason = oc_minor_cycle_stop_reason(fabsf(pv), threshold, cycle_threshold,
                                                nsigma_threshold);
        if (reason) {
            stop = reason;
            break;
        }
        float comp = gain * pv;
        model[px * ny + py] = model[px * ny + py] + comp;
        oc_subtract_shifted_psf(residual, psf, nx, ny, px, py, comp);
        if (comp_x) {
            comp_x[updates] = (int32_t)px;
            comp_y[updates] = (int32_t)py;
            comp_peak[updates] = pv;
            comp_flux[updates] = comp;
        }
        updates++;
    }
    *stop_reason = stop;
    *reported = updates < cycle_niter ? updates : cycle_niter;
    return updates;
}

/* ------------------------------------------------------------------------ */
/* robust RMS for the n-sigma threshold                                      */
/* ------------------------------------------------------------------------ */
/* mean_stddev (lib.rs:74560-74576): sequential FP64 sums, sample variance. */
void oc_mean_stddev(const float* v, int64_t n, double* mean_out, double* std_out) {
    double nn = (double)n;
    double s = 0.0;
    for (int64_t i = 0; i < n; ++i) s += (double)v[i];
    double mean = s / nn;
    double sq = 0.0;
    for (int64_t i = 0; i < n; ++i) {
        double d = (double)v[i] - mean;
        sq += d * d;
    }
    double var = n > 1 ? sq / (nn - 1.0) : 0.0;
    *mean_out = mean;
    *std_out = sqrt(var);
}

/* `(0.5 / erfc(z / sqrt 2)) as u64` (lib.rs:74624-74626) with Rust's
 * saturating float-to-integer cast. */
static uint64_t oc_chauvenet_npts(double z) {
    double x = 0.5 / erfc(z / 1.4142135623730951);
    if (!(x >= 0.0)) return 0;               /* NaN or negative */
    if (x >= 18446744073709551615.0) return UINT64_MAX;
    return (uint64_t)x;
}

/* chauvenet_max_zscore (lib.rs:74578-74622). */
double oc_chauvenet_max_zscore(uint64_t npts) {
    static const uint64_t cnt[14] = {0, 1, 3, 10, 40, 185, 1074, 7893, 73579, 872138,
                                     13165126ull, 253398672ull, 6225098696ull,
                                     195341107722ull};
    static const double zs[14] = {0.5, 1.0, 1.5, 2.0, 2.5, 3.0, 3.5,
                                  4.0, 4.5, 5.0, 5.5, 6.0, 6.5, 7.0};
    const int L = 14;
    for (int i = 0; i < L; ++i)
        if (cnt[i] == npts) return zs[i];
    int lo = 0, hi = 1;
    if (npts > cnt[L - 1]) {
        double z = zs[L - 1] + 0.5;
        for (;;) {
            if (oc_chauvenet_npts(z) >= npts) {
                lo = L - 2;
                hi = L - 1;
                break;
            }
            z += 0.5;
        }
    } else {
        while (hi < L && cnt[hi] < npts) {
            ++lo;
            ++hi;
        }
    }
    double low_z = zs[lo], high_z = zs[hi];
    double z = (low_z + high_z) / 2.0;
    for (;;) {
        uint64_t m = oc_chauvenet_npts(z);
        if (m == npts || fabs(high_z - low_z) <= 1e-12) return z;
        if (m > npts)
            high_z = z;
        else
            low_z = z;
        z = (low_z + high_z) / 2.0;
    }
}

/* apply_chauvenet_clipping (lib.rs:74512-74558): values are compacted in
 * place keeping their order; returns the new count. */
int64_t oc_chauvenet_clip(float* v, int64_t n, double zscore, int32_t max_iterations) {
    if (n == 0) return 0;
    uint64_t max_i = max_iterations >= 0 ? (uint64_t)max_iterations : 1000u;
    int64_t prev = 0;
    uint64_t it = 0;
    while (it <= max_i && n > 0) {
        int64_t cur = n;
        if (it > 0 && cur == prev) break;
        double mean, sd;
        oc_mean_stddev(v, n, &mean, &sd);
        if (!isfinite(mean) || !isfinite(sd) || sd <= 0.0) break;
        double z = zscore >= 0.0 ? zscore : oc_chauvenet_max_zscore((uint64_t)cur);
        double low = mean - z * sd, high = mean + z * sd;
        int64_t k = 0;
        for (int64_t i = 0; i < n; ++i) {
            double x = (double)v[i];
            if (x >= low && x <= high) v[k++] = v[i];
        }
        n = k;
        prev = cur;
        ++it;
    }
    return n;
}

static int oc_cmp_f64(const void* a, const void* b) {
    double x = *(const double*)a, y = *(const double*)b;
    return x < y ? -1 : (x > y ? 1 : 0);
}

/* casacore_median / casacore_madfm (casa-lattices statistics.rs:1346-1379)
 * over FP64 copies of the values; sorts `w` (n doubles) in place. */
static double oc_sorted_median(double* w, int64_t n) {
    qsort(w, (size_t)n, sizeof(double), oc_cmp_f64);
    int64_t n2 = (n - 1) / 2;
    return (n % 2 == 0) ? (w[n2] + w[n2 + 1]) / 2.0 : w[n2];
}

double oc_madfm(const float* v, int64_t n, double* median_out) {
    if (n <= 0) {
        if (median_out) *median_out = 0.0;
        return 0.0;
    }
    double* w = (double*)malloc((size_t)n * sizeof(double));
    for (int64_t i = 0; i < n; ++i) w[i] = (double)v[i];
    double med = oc_sorted_median(w, n);
    for (int64_t i = 0; i < n; ++i) w[i] = fabs((double)v[i] - med);
    double mad = oc_sorted_median(w, n);
    free(w);
    if (median_out) *median_out = med;
    return mad;
}

/* robust_rms_jy_per_beam (lib.rs:74130-74183), the default (sorted MADFM)
 * path: the finite values (all of them when the mask is absent or all true;
 * else those outside the clean mask), Chauvenet clipping (automatic z, at
 * most 5 iterations) for the full mask only, then f32(madfm) * 1.4826f. */
float oc_robust_rms(const float* residual, const uint8_t* mask, int64_t n, double* madfm_out,
                    int64_t* count_out) {
    int full = 1;
    if (mask)
        for (int64_t i = 0; i < n; ++i)
            if (!mask[i]) {
                full = 0;
                break;
            }
    float* vals = (float*)malloc((size_t)(n > 0 ? n : 1) * sizeof(float));
    int64_t m = 0;
    for (int64_t i = 0; i < n; ++i) {
        float x = residual[i];
        if (!isfinite(x)) continue;
        if (!full && mask[i]) continue;
        vals[m++] = x;
    }
    if (m > 0 && full) m = oc_chauvenet_clip(vals, m, -1.0, 5);
    double mad = m > 0 ? oc_madfm(vals, m, NULL) : 0.0;
    free(vals);
    if (madfm_out) *madfm_out = mad;
    if (count_out) *count_out = m;
    if (m == 0) return 0.0f;
    return (float)mad * 1.4826f;
}

/* ------------------------------------------------------------------------ */
/* W-projection in the reference's own precision (timed CPU baseline)        */
/* ------------------------------------------------------------------------ */
/* grid_sample_planned_pair / degrid_sample_planned (gridder.rs:3680-3747)
 * as the reference runs them: Complex32 kernels and grids, float32 complex
 * products, iy outer and ix inner.  Per-thread private grids merged in order
 * (lib.rs:71428-71540).  The FP64 functions above stay the checker; these
 * are what the CPU baseline times. */
typedef struct {
    const oc_wproj* p;
    const float* k32;
    const double *u, *v, *w;
    const float *weight, *sumwt_factor, *vis;
    const uint8_t* gridable;
    float** psf;
    float** dirty;
    oc_accum* acc;
    const float* model;
    float* pred;
} oc_wp32_job;

static void oc_wp32_grid_chunk(void* vctx, int64_t b, int64_t e, int32_t worker) {
    oc_wp32_job* j = (oc_wp32_job*)vctx;
    const oc_wproj* p = j->p;
    float* psf = j->psf[worker];
    float* dirty = j->dirty[worker];
    oc_accum* acc = &j->acc[worker];
    for (int64_t i = b; i < e; ++i) {
        float wt = j->weight[i];
        float f = j->sumwt_factor ? j->sumwt_factor[i] : 1.0f;
        float vr = j->vis[2 * i], vi = j->vis[2 * i + 1];
        if (!oc_wproj_sample_valid(j->gridable, i, wt, f, vr, vi, j->u[i], j->v[i], j->w[i])) {
            acc->skipped++;
            continue;
        }
        int64_t lx, ly, ox, oy;
        int32_t pl, cj;
        double nrm;
        if (!oc_wproj_plan(p, j->u[i], j->v[i], j->w[i], &lx, &ly, &ox, &oy, &pl, &cj, &nrm)) {
            acc->skipped++;
            continue;
        }
        acc->normalization_sumwt += 2.0 * (double)wt * nrm;
        acc->reported_sumwt += (double)wt * (double)f;
        acc->gridded++;
        const float dr = vr * wt, di = vi * wt;
        const float* k = j->k32 + (size_t)pl * p->width * p->width * 2;
        const int32_t s = p->support[pl];
        const float sg = cj ? -1.0f : 1.0f;
        for (int32_t iy = -s; iy <= s; ++iy) {
            const int64_t ky = llabs((int64_t)iy * p->sampling + oy);
            for (int32_t ix = -s; ix <= s; ++ix) {
                const int64_t kx = llabs((int64_t)ix * p->sampling + ox);
                const float kr = k[2 * (kx * p->width + ky)];
                const float ki = sg * k[2 * (kx * p->width + ky) + 1];
                const int64_t cell = (lx + ix) * p->gny + (ly + iy);
                psf[2 * cell] += wt * kr;
                psf[2 * cell + 1] += wt * ki;
                dirty[2 * cell] += dr * kr - di * ki;
                dirty[2 * cell + 1] += dr * ki + di * kr;
            }
        }
    }
}

void oc_wproj_grid_dirty_f32(const oc_wproj* p, const float* kernels32, int64_t n,
                             const double* u, const double* v, const double* w,
                             const float* weight, const float* sumwt_factor,
                             const uint8_t* gridable, const float* vis, float* psf_grid,
                             float* dirty_grid, oc_accum* acc, int32_t nthreads) {
    if (nthreads < 1) nthreads = 1;
    if ((int64_t)nthreads > n) nthreads = (int32_t)(n > 0 ? n : 1);
    const int64_t len = 2 * p->gnx * p->gny;
    oc_wp32_job j = {p, kernels32, u, v, w, weight, sumwt_factor, vis, gridable,
                     NULL, NULL, NULL, NULL, NULL};
    j.psf = (float**)calloc((size_t)nthreads, sizeof(float*));
    j.dirty = (float**)calloc((size_t)nthreads, sizeof(float*));
    j.acc = (oc_accum*)calloc((size_t)nthreads, sizeof(oc_accum));
    for (int32_t t = 0; t < nthreads; ++t) {
        j.psf[t] = nthreads == 1 ? psf_grid : (float*)calloc((size_t)len, sizeof(float));
        j.dirty[t] = nthreads == 1 ? dirty_grid : (float*)calloc((size_t)len, sizeof(float));
    }
    const int32_t used = oc_parallel_chunks(n, nthreads, oc_wp32_grid_chunk, &j);
    memset(acc, 0, sizeof(*acc));
    for (int32_t t = 0; t < used; ++t) {
        acc->normalization_sumwt += j.acc[t].normalization_sumwt;
        acc->reported_sumwt += j.acc[t].reported_sumwt;
        acc->gridded += j.acc[t].gridded;
        acc->skipped += j.acc[t].skipped;
    }
    if (nthreads > 1) {
        for (int32_t t = 0; t < used; ++t)
            for (int64_t c = 0; c < len; ++c) {
                psf_grid[c] += j.psf[t][c];
                dirty_grid[c] += j.dirty[t][c];
            }
        for (int32_t t = 0; t < nthreads; ++t) {
            free(j.psf[t]);
            free(j.dirty[t]);
        }
    }
    free(j.psf);
    free(j.dirty);
    free(j.acc);
}

static void oc_wp32_degrid_chunk(void* vctx, int64_t b, int64_t e, int32_t worker) {
    (void)worker;
    oc_wp32_job* j = (oc_wp32_job*)vctx;
    const oc_wproj* p = j->p;
    for (int64_t i = b; i < e; ++i) {
        int64_t lx, ly, ox, oy;
        int32_t pl, cj;
        double nrm;
        j->pred[2 * i] = 0.0f;
        j->pred[2 * i + 1] = 0.0f;
        if (!oc_wproj_plan(p, j->u[i], j->v[i], j->w[i], &lx, &ly, &ox, &oy, &pl, &cj, &nrm))
            continue;
        const float* k = j->k32 + (size_t)pl * p->width * p->width * 2;
        const int32_t s = p->support[pl];
        const float sg = cj ? -1.0f : 1.0f;
        float re = 0.0f, im = 0.0f;
        for (int32_t iy = -s; iy <= s; ++iy) {
            const int64_t ky = llabs((int64_t)iy * p->sampling + oy);
            for (int32_t ix = -s; ix <= s; ++ix) {
                const int64_t kx = llabs((int64_t)ix * p->sampling + ox);
                const float kr = k[2 * (kx * p->width + ky)];
                const float ki = -sg * k[2 * (kx * p->width + ky) + 1];
                const int64_t cell = (lx + ix) * p->gny + (ly + iy);
                const float gr = j->model[2 * cell], gi = j->model[2 * cell + 1];
                re += kr * gr - ki * gi;
                im += kr * gi + ki * gr;
            }
        }
        j->pred[2 * i] = re;
        j->pred[2 * i + 1] = im;
    }
}

void oc_wproj_degrid_f32(const oc_wproj* p, const float* kernels32, const float* model_grid,
                         int64_t n, const double* u, const double* v, const double* w,
                         float* pred, int32_t nthreads) {
    oc_wp32_job j = {p, kernels32, u, v, w, NULL, NULL, NULL, NULL, NULL, NULL, NULL,
                     model_grid, pred};
    oc_parallel_chunks(n, nthreads, oc_wp32_degrid_chunk, &j);
}
