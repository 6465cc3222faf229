// cr_internal.cuh -- shared internals of libcasars_cuda (not part of the ABI).
#pragma once

#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "casars_cuda.h"

namespace cr {

// Error carried from any internal function to the C-ABI boundary, where it
// becomes a status code plus a heap message.
struct Error : std::runtime_error {
    int code;
    Error(int c, const std::string& m) : std::runtime_error(m), code(c) {}
};

[[noreturn]] void fail(int code, const std::string& msg);
void check_cuda(cudaError_t e, const char* what);
void check_cufft(cufftResult r, const char* what);

#define CR_CUDA_CHECK(call) ::cr::check_cuda((call), #call)

// The C-ABI convention: *err receives a heap copy of the message (freed by
// cr_free_error), the call returns the error's status code.
inline void set_err(char** err, const std::string& msg) {
    if (!err) return;
    char* s = (char*)std::malloc(msg.size() + 1);
    if (s) std::memcpy(s, msg.c_str(), msg.size() + 1);
    *err = s;
}

template <class F>
int guarded(char** err, F&& f) {
    if (err) *err = nullptr;
    try {
        f();
        return CR_OK;
    } catch (const Error& e) {
        set_err(err, e.what());
        return e.code;
    } catch (const std::exception& e) {
        set_err(err, e.what());
        return CR_INVALID;
    } catch (...) {
        set_err(err, "unknown error");
        return CR_INVALID;
    }
}

inline void need(bool c, const char* what) {
    if (!c) fail(CR_INVALID, what);
}

struct DevBuf {
    void* ptr = nullptr;
    size_t bytes = 0;
};

// A named set of grow-only device buffers.
using Pool = std::map<std::string, DevBuf>;

struct CubeGraph;   // a captured cube pipeline (cr_cube.cu)
struct DfPlan;      // a float-pair transform plan for one line length (cr_dfft.cu)

// Default bounds of the device-side waits: polls of a grid barrier (each
// followed by a 64 ns sleep: about a second) and of an mbarrier (try_wait
// polls: milliseconds).  cr_ctx_set_wait_limits lowers them for tests.
constexpr long long kBarrierPollsDefault = 1ll << 24;
constexpr long long kMbarPollsDefault = 1ll << 22;
// pieces of a staged host batch upload (StagedBatch)
constexpr int kStageChunks = 4;

}  // namespace cr

// A context: one device, one stream, grow-only device workspaces, cached
// cuFFT plans and a launch counter.
struct cr_ctx {
    int device = 0;
    int sms = 0;           // multiprocessors of the device (grid sizing)
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    // a second stream for work that runs beside the main stream's inside one
    // call, forked from and joined back to `stream` by these events
    cudaStream_t aux_stream = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    // one per chunk of a host batch uploaded on aux_stream (StagedBatch)
    cudaEvent_t stage_ev[cr::kStageChunks] = {};
    cr::Pool ws;
    std::map<std::pair<int64_t, int64_t>, cufftHandle> fft_plans;
    std::map<std::pair<int64_t, int64_t>, cufftHandle> fft_plans_c2c;
    // real-to-complex and complex-to-real plans, by cufftType
    std::map<int, std::map<std::pair<int64_t, int64_t>, cufftHandle>> fft_plans_real;
    // batched real transforms over cube planes, by (type, batch)
    std::map<std::pair<int, int>, std::map<std::pair<int64_t, int64_t>, cufftHandle>>
        fft_plans_many;
    cudaEvent_t ev[8] = {};
    // [0,1] bracket the last gridding kernel, [2,3] the last degridding kernel
    cudaEvent_t kev[4] = {};
    int kev_used = 0;
    cr_timings timings = {};
    int64_t launches = 0;
    // cube path: tuned gridding chunk per cube shape, captured pipelines per
    // call signature; ws_epoch changes whenever a workspace is (re)allocated,
    // which retires the captured graphs (they hold workspace addresses)
    std::map<std::string, uint32_t> cube_chunk;
    uint32_t cube_chunk_forced = 0;   // nonzero: this chunk instead of the tuner's
    std::map<std::string, std::shared_ptr<cr::CubeGraph>> cube_graphs;
    bool cube_graphs_enabled = true;
    // Precision of the image-stage FFTs of single-plane calls: 64 (default)
    // or 32.
    int image_fft_bits = 64;
    // How the FP64-grade image transforms run: 0 float-pair kernels where
    // the grid allows (cr_dfft.cu), else cuFFT FP64; 1 always cuFFT FP64.
    int image_fft_engine = 0;
    std::map<int64_t, std::shared_ptr<cr::DfPlan>> df_plans;
    bool capturing = false;
    uint64_t ws_epoch = 0;
    // small pinned host buffer for device->host scalars
    void* pinned = nullptr;
    // mapped host word that kernels set (CR_TIMEOUT) when a bounded wait
    // gives up; read after the stream synchronises
    int* status_h = nullptr;
    int* status_d = nullptr;
    // bounds of the first wait of a grid barrier (Hogbom) and of a
    // bulk-copy mbarrier (cube kernels); the drain waits after a timeout
    // keep the defaults
    // test hook: a budget (bytes) for the context's workspaces, 0 = none; a
    // call that would grow them past it fails as an allocation failure would
    int64_t alloc_limit = 0;
    // per-call stage and kernel timings (cr_ctx_last_timings); off, calls
    // record no events and do not wait for them
    bool timings_enabled = true;
    long long barrier_polls = cr::kBarrierPollsDefault;
    long long mbar_polls = cr::kMbarPollsDefault;
};

// Standard (PSWF) gridder state.
struct cr_gridder {
    cr_ctx* ctx = nullptr;
    cr_geometry geom = {};
    cr_grid_info info = {};
    int32_t tap_rows = 0;
    std::vector<float> taps_h, corr_x_h, corr_y_h;
    float* taps_d = nullptr;     // [tap_rows][7], zero-padded to taps_bytes
    uint32_t taps_bytes = 0;     // tap_rows * 7 * 4 rounded up to 16 (bulk copies)
    float* taps8_d = nullptr;    // [tap_rows][8]: rows padded with a zero to 32 bytes
    float* corr_x_d = nullptr;   // [grid_nx]
    float* corr_y_d = nullptr;   // [grid_ny]
};

// W-projection state: cropped kernels, normalisation table and the
// residue cubes the gridder and degridder read.
struct cr_wproj {
    cr_ctx* ctx = nullptr;
    cr_gridder* g = nullptr;
    cr_wproj_info info = {};
    int32_t radius = 0;          // (sampling + 1) / 2: offsets lie in [-radius, radius]
    int32_t axis = 0;            // 2 * radius + 1
    std::vector<int32_t> support_h;
    std::vector<int64_t> cube_off_h;  // [planes] start of each plane's residue cube
    std::vector<int32_t> cube_q_h;    // [planes] residue extent Q of each cube
    int32_t* support_d = nullptr;
    int64_t* cube_off_d = nullptr;
    int32_t* cube_q_d = nullptr;
    float2* kernels_d = nullptr;      // [planes][width][width]
    float* norm_d = nullptr;          // [planes][axis][axis]
    float2* cube_d = nullptr;         // per plane [s][s][Q][Q]: K[qx s + rx, qy s + ry]
    float* sinc_x_d = nullptr;        // sinc axis for the image correction (max(g) long)
    float* sinc_gx_d = nullptr;       // sinc axes for the model apodisation
    float* sinc_gy_d = nullptr;
    int32_t* first_plane_d = nullptr;  // [max support + 1] first plane with support >= S
    bool support_monotone = false;     // supports non-decreasing in the plane index
};

namespace cr {

// ---- context helpers -------------------------------------------------------
void* workspace(cr_ctx* ctx, const std::string& name, size_t bytes);
// Looks up the allocation-free Hogbom's static scratch on `device` (which the
// caller has made current), loading the module that holds it.
void noalloc_prepare(int device);
// the same from another pool (stream-ordered on ctx's stream)
void* pool_alloc(cr_ctx* ctx, Pool& pool, const std::string& name, size_t bytes);
void pool_free(cr_ctx* ctx, Pool& pool);
void note_launch(cr_ctx* ctx, const char* what);
// After the stream has synchronised: a status that a kernel set (a bounded
// wait that gave up) becomes an error, and the word is cleared.
void check_device_status(cr_ctx* ctx);
// Event pair around one gridding (which = 0) or degridding (which = 1) kernel.
void kernel_mark(cr_ctx* ctx, int which, bool end);
cufftHandle fft_plan(cr_ctx* ctx, int64_t nx, int64_t ny);
cufftHandle fft_plan_c2c(cr_ctx* ctx, int64_t nx, int64_t ny);
cufftHandle fft_plan_type(cr_ctx* ctx, int64_t nx, int64_t ny, cufftType type);
cufftHandle fft_plan_many(cr_ctx* ctx, int64_t nx, int64_t ny, cufftType type, int batch);

// ---- host-side tables (restated from gridder.rs) ----------------------------
int64_t casa_composite_padded_len(int64_t image_len, double padding);
int64_t image_blc(int64_t grid_len, int64_t image_len);
double grdsf(double nu);
std::vector<float> std_normalized_taps(int32_t oversampling, int32_t support);
std::vector<float> correction_axis(int64_t size);
std::vector<float> gridder_correction_axis(int64_t size);
std::vector<float> sinc_axis(int64_t size, int64_t conv_sampling);

// ---- device primitives -------------------------------------------------------
// Exclusive scan of n uint32 values into out (may alias in); *total_dev (if
// non-null, device pointer) receives the sum as uint64.
void exclusive_scan_u32(cr_ctx* ctx, const uint32_t* in, uint32_t* out, int64_t n,
                        unsigned long long* total_dev);
// Stable LSD radix sort of (key, value) pairs on the low `bits` bits.
// Sorted output ends in keys/vals.
void radix_sort_pairs(cr_ctx* ctx, uint64_t* keys, uint32_t* vals, int64_t n, int bits);

// ---- batch upload ------------------------------------------------------------
struct DeviceBatch {
    int64_t n = 0;
    const double* u = nullptr;
    const double* v = nullptr;
    const double* w = nullptr;
    const float* weight = nullptr;
    const float* sumwt_factor = nullptr;
    const uint8_t* gridable = nullptr;
    const float2* vis = nullptr;
    // staged uploads (StagedBatch): piece k, samples [chunk_end[k - 1],
    // chunk_end[k]), is on the device once stage_ev[k] has completed
    int nchunks = 0;
    int64_t chunk_end[kStageChunks] = {};
    const cudaEvent_t* stage_ev = nullptr;
};
DeviceBatch device_batch(cr_ctx* ctx, const cr_vis_batch* b, bool need_w);

// A batch for the calls that plan it straight away.  A large host batch is
// uploaded in kStageChunks pieces on the auxiliary stream, each followed by
// one of ctx->stage_ev, so that the plan kernel starts on the first piece
// while the others are still copying (plan_wproj / plan_standard wait for
// each piece before planning it).  Otherwise it is device_batch's.  When the
// batch goes out of scope the main stream waits for the last piece, so no
// copy outlives the call whatever path it takes.
struct StagedBatch : DeviceBatch {
    cr_ctx* ctx = nullptr;
    StagedBatch(cr_ctx* c, const cr_vis_batch* b, bool need_w);
    StagedBatch(const StagedBatch&) = delete;
    StagedBatch& operator=(const StagedBatch&) = delete;
    ~StagedBatch();
};

// Host or device source -> device pointer (copies host data into a named
// workspace).
const void* device_input(cr_ctx* ctx, const void* p, size_t bytes, int32_t location,
                         const char* name);
void copy_out(cr_ctx* ctx, void* dst, const void* src_dev, size_t bytes, int32_t location);

// ---- row runs -------------------------------------------------------------------
struct RowsOut {
    double *u, *v, *w, *du, *dv;
    float* weight;
    float* sumwt_factor;
    uint8_t* gridable;
    float2* vis;
};
// Kept samples of the row runs into `out` (device arrays of rows x channels
// entries); returns their count (synchronises).
int64_t prepare_rows(cr_ctx* ctx, const cr_row_runs* rr, const cr_polarization* pol,
                     const RowsOut& out);

// ---- records: the deduplicated sample plan ------------------------------------
// Samples with identical (cell, kernel offset, w-plane, conjugation) get
// identical taps; they are summed into one record before gridding.
struct Records {
    int64_t n_samples = 0;
    uint64_t* keys = nullptr;        // sorted keys [n]
    uint32_t* order = nullptr;       // sorted sample indices [n]
    int32_t* sample_rec = nullptr;   // [n] record of each sample, -1 when skipped
    int32_t* rec_x = nullptr;        // anchor / start cell x   [n]
    int32_t* rec_y = nullptr;        // [n]
    int32_t* rec_a = nullptr;        // plane (wproj) or x tap row (standard)  [n]
    int32_t* rec_b = nullptr;        // offset index (wproj) or y tap row      [n]
    int32_t* rec_conj = nullptr;     // [n]
    double2* rec_vsum = nullptr;     // sum vis * weight  [n]
    double* rec_wsum = nullptr;      // sum weight        [n]
    float2* rec_pred = nullptr;      // degridded value   [n]
    uint32_t* tile_start = nullptr;  // [ntiles + 1] first record of each home tile
    int64_t ntx = 0, nty = 0;        // home tiles (32 x 32 cells)
    // device scalars: [0] gridded, [1] skipped, [2] unique records
    unsigned long long* counts = nullptr;
    double* sums = nullptr;          // [0] normalisation sumwt, [1] reported sumwt
};

constexpr int kTile = 32;            // home/output tile edge in grid cells

// The records live in `pool` (the context's workspaces when null).
Records plan_wproj(cr_ctx* ctx, cr_wproj* wp, const DeviceBatch& b, Pool* pool = nullptr);
Records plan_standard(cr_ctx* ctx, cr_gridder* g, const DeviceBatch& b, Pool* pool = nullptr);
void read_sums(cr_ctx* ctx, const Records& r, cr_sums* out);

// ---- gridding kernels ----------------------------------------------------------
// mode 0: PSF + dirty from the record sums; mode 1: residual
// (vsum - pred * wsum) into `dirty` only.
void wproj_grid(cr_ctx* ctx, cr_wproj* wp, const Records& r, float2* psf, float2* dirty,
                int mode);
void wproj_degrid(cr_ctx* ctx, cr_wproj* wp, const Records& r, const float2* grid);
void std_grid(cr_ctx* ctx, cr_gridder* g, const Records& r, float2* psf, float2* dirty,
              int mode);
void std_degrid(cr_ctx* ctx, cr_gridder* g, const Records& r, const float2* grid);
void broadcast_pred(cr_ctx* ctx, const Records& r, float2* pred);

// the cube gridding chunk sizes the tuner chooses from
bool cube_grid_chunk_valid(uint32_t chunk);

// ---- multiscale CLEAN (cr_msclean.cu) ----------------------------------------------
void multiscale_create(cr_multiscale* ms, const float* psf, const uint8_t* mask,
                       float small_scale_bias);
void multiscale_set_residual(cr_multiscale* ms, const float* residual);

// ---- robust RMS (n-sigma threshold) ----------------------------------------------
// robust_rms_jy_per_beam of the listed planes of device images [P][npix]
// (masks [P][npix] or null); rms / madfm / counts per listed plane (host).
void robust_rms(cr_ctx* ctx, const float* images, const uint8_t* masks, int64_t npix,
                const std::vector<int>& planes, float* rms, double* madfm, int64_t* counts);
double chauvenet_max_zscore(uint64_t npts);

// ---- FFT stage -------------------------------------------------------------------
// grid (device, modified in place) -> image * scale (device)
// single: float32 C2C transforms instead of FP64 Z2Z (the cube image stage)
void grid_to_image(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, float2* grid, float scale,
                   float* image, bool single = false);
// the exact adjoint of image_to_grid's image-side factor (no sinc division)
// The image stage over planes of a cube, batched: grids (complex, or the
// PSF's real parts) [C][gnx][gny] -> images [C][nx][ny] for the listed
// planes, plane k scaled by scales[k] as grid_to_image scales; and models
// [C][nx][ny] -> model grids for the listed planes.
void grid_to_image_planes(cr_ctx* ctx, cr_gridder* g, const float2* grids,
                          const float* real_grids, const std::vector<int>& planes,
                          const std::vector<float>& scales, float* images, bool single);
void image_to_grid_planes(cr_ctx* ctx, cr_gridder* g, const float* models,
                          const std::vector<int>& planes, float2* grids, bool single);
// abs_peak and scale_image over the listed planes of images [C][n]: peaks
// indexed by plane; plane k scaled by scales[k] (then divided by its peak
// when peaks is given).
void abs_peak_planes(cr_ctx* ctx, const float* images, int64_t n,
                     const std::vector<int>& planes, unsigned int* peaks);
void scale_image_planes(cr_ctx* ctx, float* images, int64_t n, const std::vector<int>& planes,
                        const std::vector<float>& scales, const unsigned int* peaks);
void grid_to_image_adjoint(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, float2* grid, float scale,
                           float* image, bool single = false);
// model image (device) -> centred model grid (device)
void image_to_grid(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float* model, float2* grid,
                   bool single = false);
// grid_to_image of a real grid (the real part of a PSF grid), standard gridder
void grid_to_image_real(cr_ctx* ctx, cr_gridder* g, const float* grid, float scale,
                        float* image, bool single = false);
// The FP64-grade image transforms in float-pair arithmetic (cr_dfft.cu):
// whether both grid sizes are served; grid (or the PSF's real parts) ->
// image, with crop_correct_body's scale, sinc factors and mode; image ->
// model grid (apodize_body's factors, then the float32 grid).
bool dfft_supported(int64_t gnx, int64_t gny);
void dfft_grid_to_image(cr_ctx* ctx, cr_gridder* g, const float2* grid, const float* real_grid,
                        double scale, const float* sx, const float* sy, int sinc_mode,
                        float* image);
void dfft_image_to_grid(cr_ctx* ctx, cr_gridder* g, const float* model, const float* sinc_x,
                        const float* sinc_y, float2* grid);
// max |image| into *peak_dev (float bits as uint32)
void abs_peak(cr_ctx* ctx, const float* image, int64_t n, unsigned int* peak_dev);
// image *= scale, then / *peak_dev when peak_dev != null
void scale_image(cr_ctx* ctx, float* image, int64_t n, float scale, const unsigned int* peak_dev);

// ---- batched cube (cr_cube.cu) ------------------------------------------------
// Device views of a cube batch: rows' u, v in metres, [C][R] samples;
// lambda_scale is a host array of C values.
struct CubeInput {
    int64_t R = 0;
    int32_t C = 0;
    const double* u = nullptr;
    const double* v = nullptr;
    const double* lambda_scale = nullptr;
    const float2* vis = nullptr;
    const float* weight = nullptr;
    const uint8_t* flags = nullptr;
};
// Records of every channel binned by (channel, home tile).
struct CubeRecords {
    int64_t R = 0;
    int32_t C = 0;
    int64_t ntx = 0, nty = 0, ntiles = 0;
    uint4* rec = nullptr;              // {cell | tap rows, c R + r, w vis}
    float* rec_w = nullptr;
    uint32_t* bin_start = nullptr;     // [C ntiles + 1]
    uint32_t* cell_end = nullptr;      // [C ntiles 1024] end of each (tile, cell) bin
    double* sumwt = nullptr;           // [C]
    unsigned long long* counts = nullptr;  // [C][2] gridded, skipped
    unsigned long long* n_rec = nullptr;
    // work lists: chunks per bin, their scan, (bin, chunk) items, item totals
    uint32_t *grid_chunks = nullptr, *grid_first = nullptr;
    uint32_t *degrid_chunks = nullptr, *degrid_first = nullptr;
    uint2 *grid_items = nullptr, *degrid_items = nullptr;
    unsigned long long* n_items = nullptr;   // [0] gridding, [1] degridding
    uint32_t grid_chunk = 0;                 // records per gridding work item
    bool fill_done = false;                  // set once the work lists are made
    bool lists_masked = false;               // the lists skip some planes
    int64_t n_records = -1;                  // total records, when read back
};
// Per-sample outputs of cube_sample_taps ([C][R], -1 / 0 when not gridded).
struct CubeTaps {
    int32_t *start_x, *start_y, *row_x, *row_y;
    float* weight;
};
// With `taps`, only the weighting and the per-sample plan run.
CubeRecords cube_plan(cr_ctx* ctx, cr_gridder* g, const CubeInput& in, int32_t mode,
                      float robust, const CubeTaps* taps = nullptr, Pool* keep = nullptr);
// psf [C][gnx][gny] float32 (real part), dirty [C][gnx][gny] complex64
void cube_grid(cr_ctx* ctx, cr_gridder* g, CubeRecords& cr, float* psf, float2* dirty);
// pred [C][R] complex64, zero for samples that are not gridded
void cube_degrid(cr_ctx* ctx, cr_gridder* g, CubeRecords& cr, const float2* grid,
                 float2* pred);
// Residual grids of every plane with plane_mask[c] != 0 (device, NULL = all):
// degrid the model grids per record, w vis - w pred, grid that; the psf is
// not formed.  Other planes' grids are left as they are.
void cube_grid_residual(cr_ctx* ctx, cr_gridder* g, CubeRecords& cr, const float2* model,
                        float2* residual, const uint8_t* plane_mask);
void cube_read_sums(cr_ctx* ctx, const CubeRecords& cr, cr_sums* out);
// Host-side constants of the cube plan, uploaded outside any graph capture.
void cube_upload_channels(cr_ctx* ctx, cr_gridder* g, const CubeInput& in);

// One captured planning + gridding (+ degridding) pipeline of the cube.
struct CubeGraph {
    cudaGraphExec_t exec = nullptr;
    uint64_t epoch = 0;
    int eager_runs = 0;
    bool failed = false;     // capture failed: this signature runs eagerly
    int64_t launches = 0;   // kernels in the graph
    CubeRecords cr;
    ~CubeGraph() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

// ---- restoring beam (cr_beam.cu) -------------------------------------------------
bool fit_beam(const float* psf_host, int64_t nx, int64_t ny, double cell_x, double cell_y,
              float cutoff, cr_beam* beam, int32_t* attempts, float* cutoff_used);
void restore(cr_ctx* ctx, const float* model, const float* residual, int32_t nx, int32_t ny,
             double cell_x, double cell_y, const cr_beam& beam, float* out);
float psf_sidelobe(cr_ctx* ctx, const float* psf, int32_t nx, int32_t ny, double cell_x,
                   double cell_y, const cr_beam& beam);

// ---- W-projection build ----------------------------------------------------------
void build_wproj(cr_ctx* ctx, cr_wproj* wp, double max_abs_w, int32_t planes,
                 int32_t sampling, int32_t support_min, int32_t support_max);

// ---- weighting / Hogbom ----------------------------------------------------------
// build_u / build_v (device, optional): where the density is built, when
// that differs from the lookup coordinates u, v (the row path).
void apply_weighting(cr_ctx* ctx, cr_gridder* g, const DeviceBatch& b, int32_t mode,
                     float robust, float* out_weight, float* f2_out, int32_t convention = 0,
                     const double* build_u = nullptr, const double* build_v = nullptr);
void hogbom(cr_ctx* ctx, float* model, float* residual, const float* psf, const uint8_t* mask,
            int32_t nx, int32_t ny, float gain, float threshold, float cycle_threshold,
            float nsigma_threshold, int64_t cycle_niter, int32_t inclusive, int32_t* comp_x,
            int32_t* comp_y, float* comp_peak, float* comp_flux, int64_t* actual,
            int64_t* reported, int32_t* stop_reason, int plane_rules = 0);
// run_hogbom_plane_minor_cycle (lib.rs:64630-64680) on device images: the
// fast loop with its rules when the peak tolerance is 0, a single-block
// replay of the tolerance scan otherwise.
void hogbom_plane(cr_ctx* ctx, float* model, float* residual, const float* psf,
                  const uint8_t* mask, int32_t nx, int32_t ny, float gain, float threshold,
                  float cycle_threshold, float peak_relative_tolerance, int64_t cycle_limit,
                  int32_t inclusive, int32_t* comp_x, int32_t* comp_y, float* comp_peak,
                  float* comp_flux, int64_t* actual, int64_t* reported);
// run_clark_minor_cycle_cpu (lib.rs:62129-62355) on device images; the PSF
// patch is (3 ncent + 1)^2 about the centre (build_clark_psf_patch).
void clark_minor_cycle(cr_ctx* ctx, float* model, float* residual, const float* psf,
                       const uint8_t* mask, int32_t nx, int32_t ny, int32_t ncent, float gain,
                       float threshold, float cycle_threshold, float nsigma_threshold,
                       int64_t cycle_niter, int32_t* comp_x, int32_t* comp_y, float* comp_peak,
                       float* comp_flux, int64_t* actual, int32_t* stop_out,
                       float* max_exterior_out);
// The minor cycles of the listed planes of [nplanes][nx][ny] images in one
// launch (groups of co-resident blocks, one per plane); results per listed
// plane, component arrays [n][cycle_niter + inclusive] (host, or null).
void hogbom_planes(cr_ctx* ctx, float* model, float* residual, const float* psf,
                   const uint8_t* mask, int32_t nx, int32_t ny, int32_t nplanes,
                   const int32_t* planes, int32_t n, float gain, float threshold,
                   float cycle_threshold, float nsigma_threshold,
                   const float* nsigma_per_plane, int64_t cycle_niter, int32_t inclusive,
                   int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
                   int64_t* actual, int64_t* reported, int32_t* stop_reason_out);

inline unsigned int grid_blocks(int64_t n, int threads, int64_t cap = 152 * 32) {
    int64_t b = (n + threads - 1) / threads;
    if (b < 1) b = 1;
    if (b > cap) b = cap;
    return (unsigned int)b;
}

}  // namespace cr

// A materialised plan of one batch (the device form of the reference's
// planned taps): its records outlive the call that made them, in the plan's
// own pool, and serve any number of gridding and degridding calls.
struct cr_accumulator {
    cr_ctx* ctx = nullptr;
    cr_gridder* g = nullptr;
    cr::Pool pool;
    float2* psf = nullptr;
    float2* dirty = nullptr;
    cr_sums sums = {};
    int64_t batches = 0;
};

struct cr_cube_plan {
    cr_ctx* ctx = nullptr;
    cr_gridder* g = nullptr;
    cr::Pool pool;
    cr::CubeRecords rec;
    std::vector<cr_sums> sums;
    int32_t fft_bits = 32;   // image-stage transforms: 32 (C2C) or 64 (Z2Z)
};

struct cr_plan {
    cr_ctx* ctx = nullptr;
    cr_gridder* g = nullptr;
    cr_wproj* wp = nullptr;
    cr::Pool pool;
    cr::Records rec;
    cr_sums sums = {};
};
