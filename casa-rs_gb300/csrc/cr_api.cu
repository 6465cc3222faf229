// cr_api.cu -- the extern "C" boundary of libcasars_cuda.
//
// Every entry point catches internal errors and turns them into the
// reference shims' convention: an int status and a heap message in *err.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "cr_internal.cuh"

using namespace cr;

namespace {

// Work issued between to_aux() and to_main() goes to the context's auxiliary
// stream, which first waits for everything already on the main stream;
// join() makes the main stream wait for that work.  The destructor restores
// the main stream and joins, also when an exception leaves the call early,
// so no auxiliary work outlives the call unordered.
struct AuxFork {
    cr_ctx* ctx;
    cudaStream_t main;
    bool on_aux = false, joined = true;
    explicit AuxFork(cr_ctx* c) : ctx(c), main(c->stream) {}
    void to_aux() {
        CR_CUDA_CHECK(cudaEventRecord(ctx->fork_ev, main));
        CR_CUDA_CHECK(cudaStreamWaitEvent(ctx->aux_stream, ctx->fork_ev, 0));
        ctx->stream = ctx->aux_stream;
        on_aux = true;
        joined = false;
    }
    void to_main() {
        if (!on_aux) return;
        ctx->stream = main;
        on_aux = false;
        CR_CUDA_CHECK(cudaEventRecord(ctx->join_ev, ctx->aux_stream));
    }
    void join() {
        to_main();
        if (!joined) CR_CUDA_CHECK(cudaStreamWaitEvent(main, ctx->join_ev, 0));
        joined = true;
    }
    ~AuxFork() {
        if (on_aux) {
            ctx->stream = main;
            cudaEventRecord(ctx->join_ev, ctx->aux_stream);
        }
        if (!joined) cudaStreamWaitEvent(main, ctx->join_ev, 0);
    }
};

// Stage times of a call from events on its stream.  With the context's
// timings off nothing is recorded and nothing waits for the events.
struct StageTimer {
    cr_ctx* ctx;
    int n = 0;
    explicit StageTimer(cr_ctx* c) : ctx(c) { ctx->kev_used = 0; }
    void mark() {
        if (ctx->timings_enabled && n < 8)
            CR_CUDA_CHECK(cudaEventRecord(ctx->ev[n++], ctx->stream));
    }
    float between(int a, int b) {
        if (b >= n || a >= n) return 0.0f;
        float ms = 0.0f;
        CR_CUDA_CHECK(cudaEventSynchronize(ctx->ev[b]));
        CR_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx->ev[a], ctx->ev[b]));
        return ms;
    }
};

// Stage times of a call plus the bracketed kernel times recorded during it.
void set_timings(cr_ctx* ctx, cr_timings t) {
    if (!ctx->timings_enabled) {
        ctx->kev_used = 0;
        ctx->timings = cr_timings{};
        return;
    }
    for (int k = 0; k < 2; ++k) {
        if (!(ctx->kev_used & (1 << k))) continue;
        float ms = 0.0f;
        CR_CUDA_CHECK(cudaEventSynchronize(ctx->kev[2 * k + 1]));
        CR_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx->kev[2 * k], ctx->kev[2 * k + 1]));
        (k == 0 ? t.grid_kernel_ms : t.degrid_kernel_ms) = ms;
    }
    ctx->kev_used = 0;
    ctx->timings = t;
}

void bind(cr_ctx* ctx) { CR_CUDA_CHECK(cudaSetDevice(ctx->device)); }

Records plan(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const DeviceBatch& b,
             Pool* pool = nullptr) {
    return wp ? plan_wproj(ctx, wp, b, pool) : plan_standard(ctx, g, b, pool);
}

void grid_records(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const Records& r, float2* psf,
                  float2* dirty, int mode) {
    if (wp)
        wproj_grid(ctx, wp, r, psf, dirty, mode);
    else
        std_grid(ctx, g, r, psf, dirty, mode);
}

void degrid_records(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const Records& r,
                    const float2* grid) {
    if (wp)
        wproj_degrid(ctx, wp, r, grid);
    else
        std_degrid(ctx, g, r, grid);
}

size_t grid_bytes(const cr_gridder* g) { return (size_t)g->info.grid_nx * g->info.grid_ny * 8; }
size_t image_pixels(const cr_gridder* g) { return (size_t)g->geom.nx * g->geom.ny; }

// output pointer on the device: the caller's buffer when it is device memory,
// else a named workspace that is copied out afterwards
template <class T>
T* out_ptr(cr_ctx* ctx, void* user, int32_t loc, size_t bytes, const char* name) {
    if (loc == CR_DEVICE) {
        need(user != nullptr, "output pointer is null");
        return (T*)user;
    }
    need(loc == CR_HOST, "location must be CR_HOST or CR_DEVICE");
    return (T*)workspace(ctx, std::string("out_") + name, bytes);
}

void check_wp(cr_gridder* g, cr_wproj* wp) {
    need(g != nullptr, "gridder is null");
    if (wp) need(wp->g == g, "W-projector belongs to another gridder");
}


CubeInput cube_input(cr_ctx* ctx, const cr_cube_batch* b) {
    need(b != nullptr, "cube batch is null");
    need(b->rows >= 0 && b->channels > 0, "cube batch needs rows >= 0 and channels > 0");
    need(b->lambda_scale != nullptr, "lambda_scale is null");
    need(b->rows == 0 || (b->u_m && b->v_m && b->vis), "u_m, v_m and vis are required");
    CubeInput in;
    in.R = b->rows;
    in.C = b->channels;
    const size_t R = (size_t)b->rows, S = (size_t)b->rows * (size_t)b->channels;
    in.lambda_scale = b->lambda_scale;
    in.u = (const double*)device_input(ctx, b->u_m, R * 8, b->location, "cube_u");
    in.v = (const double*)device_input(ctx, b->v_m, R * 8, b->location, "cube_v");
    in.vis = (const float2*)device_input(ctx, b->vis, S * 8, b->location, "cube_vis");
    in.weight = (const float*)device_input(ctx, b->weight, S * 4, b->location, "cube_weight");
    in.flags = (const uint8_t*)device_input(ctx, b->flags, S, b->location, "cube_flags");
    return in;
}

// A call signature of the cube path: every pointer, size and parameter the
// captured pipeline depends on.
std::string cube_key(const cr_gridder* g, const cr_cube_batch* b, int32_t weighting, float robust,
                     const void* psf, const void* dirty, const void* model, const void* pred) {
    std::string k;
    auto put = [&](const void* p, size_t n) { k.append((const char*)p, n); };
    put(&g, sizeof g);
    put(&b->rows, sizeof b->rows);
    put(&b->channels, sizeof b->channels);
    put(&b->u_m, sizeof b->u_m);
    put(&b->v_m, sizeof b->v_m);
    put(&b->vis, sizeof b->vis);
    put(&b->weight, sizeof b->weight);
    put(&b->flags, sizeof b->flags);
    put(&weighting, sizeof weighting);
    put(&robust, sizeof robust);
    put(&psf, sizeof psf);
    put(&dirty, sizeof dirty);
    put(&model, sizeof model);
    put(&pred, sizeof pred);
    put(b->lambda_scale, (size_t)b->channels * sizeof(double));
    return k;
}

// Replays a captured cube pipeline on the context's own stream, ordered
// after and before the caller's stream by events; times it as one stage.
void cube_replay(cr_ctx* ctx, CubeGraph& G, cr_sums* sums) {
    cudaStream_t caller = ctx->stream, own = ctx->own_stream;
    if (caller != own) {
        CR_CUDA_CHECK(cudaEventRecord(ctx->ev[4], caller));
        CR_CUDA_CHECK(cudaStreamWaitEvent(own, ctx->ev[4], 0));
    }
    CR_CUDA_CHECK(cudaEventRecord(ctx->ev[0], own));
    CR_CUDA_CHECK(cudaGraphLaunch(G.exec, own));
    ctx->launches += G.launches;
    CR_CUDA_CHECK(cudaEventRecord(ctx->ev[1], own));
    if (caller != own) {
        CR_CUDA_CHECK(cudaEventRecord(ctx->ev[5], own));
        CR_CUDA_CHECK(cudaStreamWaitEvent(caller, ctx->ev[5], 0));
    }
    ctx->stream = own;
    try {
        cube_read_sums(ctx, G.cr, sums);
        CR_CUDA_CHECK(cudaEventSynchronize(ctx->ev[1]));
        check_device_status(ctx);
    } catch (...) {
        ctx->stream = caller;
        throw;
    }
    ctx->stream = caller;
    float ms = 0.0f;
    CR_CUDA_CHECK(cudaEventElapsedTime(&ms, ctx->ev[0], ctx->ev[1]));
    ctx->kev_used = 0;
    set_timings(ctx, cr_timings{0.f, ms, 0.f, 0.f, 0.f});
}

int cube_run(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch, int32_t weighting,
             float robust, float* psf_grids, float* dirty_grids, const float* model_grids,
             int32_t grid_location, float* pred, int32_t out_location, cr_sums* sums,
             char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && g != nullptr, "null argument");
        bind(ctx);
        // All-device calls are captured into a CUDA graph on their second
        // occurrence (the first runs eagerly: it sizes the workspaces and
        // tunes the gridding chunk) and replayed from then on, until a
        // workspace is reallocated.
        const bool on_device = batch != nullptr && batch->location == CR_DEVICE &&
                               out_location == CR_DEVICE &&
                               (!model_grids || grid_location == CR_DEVICE) &&
                               !psf_grids == !dirty_grids && (!model_grids || pred);
        if (on_device && ctx->cube_graphs_enabled) {
            const std::string key = cube_key(g, batch, weighting, robust, psf_grids,
                                             dirty_grids, model_grids, pred);
            // callers that never repeat a signature must not grow the table
            if (ctx->cube_graphs.size() >= 32 && !ctx->cube_graphs.count(key))
                ctx->cube_graphs.clear();
            auto& slot = ctx->cube_graphs[key];
            if (!slot) slot = std::make_shared<CubeGraph>();
            CubeGraph& G = *slot;
            if (G.exec && G.epoch != ctx->ws_epoch) {
                CR_CUDA_CHECK(cudaGraphExecDestroy(G.exec));
                G.exec = nullptr;
                G.eager_runs = 0;
            }
            if (G.exec) {
                cube_replay(ctx, G, sums);
                return;
            }
            if (G.eager_runs >= 1 && !G.failed) {
                CubeInput in = cube_input(ctx, batch);
                cudaStream_t caller = ctx->stream, own = ctx->own_stream;
                if (caller != own) {
                    CR_CUDA_CHECK(cudaEventRecord(ctx->ev[4], caller));
                    CR_CUDA_CHECK(cudaStreamWaitEvent(own, ctx->ev[4], 0));
                }
                ctx->stream = own;
                try {
                    cube_upload_channels(ctx, g, in);
                } catch (...) {
                    ctx->stream = caller;
                    throw;
                }
                cudaGraph_t graph = nullptr;
                const int64_t launches0 = ctx->launches;
                try {
                    CR_CUDA_CHECK(cudaStreamBeginCapture(own, cudaStreamCaptureModeThreadLocal));
                    ctx->capturing = true;
                    CubeRecords cr = cube_plan(ctx, g, in, weighting, robust);
                    if (psf_grids)
                        cube_grid(ctx, g, cr, psf_grids, (float2*)dirty_grids);
                    if (model_grids)
                        cube_degrid(ctx, g, cr, (const float2*)model_grids, (float2*)pred);
                    ctx->capturing = false;
                    CR_CUDA_CHECK(cudaStreamEndCapture(own, &graph));
                    CR_CUDA_CHECK(cudaGraphInstantiate(&G.exec, graph, 0));
                    CR_CUDA_CHECK(cudaGraphDestroy(graph));
                    G.cr = cr;
                    G.epoch = ctx->ws_epoch;
                    G.launches = ctx->launches - launches0;
                    ctx->launches = launches0;
                } catch (...) {
                    // a call that cannot be captured (say, a workspace that
                    // must grow) runs eagerly, now and from then on
                    if (ctx->capturing) {
                        ctx->capturing = false;
                        graph = nullptr;
                        cudaStreamEndCapture(own, &graph);
                    }
                    if (graph) cudaGraphDestroy(graph);
                    if (G.exec) cudaGraphExecDestroy(G.exec);
                    G.exec = nullptr;
                    cudaGetLastError();
                    ctx->launches = launches0;
                    G.failed = true;
                }
                ctx->stream = caller;
                if (G.exec) {
                    cube_replay(ctx, G, sums);
                    return;
                }
            }
            G.eager_runs++;
        }
        StageTimer tm(ctx);
        tm.mark();
        CubeInput in = cube_input(ctx, batch);
        CubeRecords cr = cube_plan(ctx, g, in, weighting, robust);
        tm.mark();
        const size_t cells = (size_t)g->info.grid_nx * g->info.grid_ny;
        const size_t C = (size_t)in.C;
        float* psf = nullptr;
        float2* dirty = nullptr;
        if (psf_grids || dirty_grids) {
            need(psf_grids && dirty_grids, "psf_grids and dirty_grids go together");
            psf = out_ptr<float>(ctx, psf_grids, out_location, C * cells * 4, "cube_psf");
            dirty = out_ptr<float2>(ctx, dirty_grids, out_location, C * cells * 8, "cube_dirty");
            cube_grid(ctx, g, cr, psf, dirty);
        }
        tm.mark();
        float2* pr = nullptr;
        if (model_grids) {
            need(pred != nullptr, "pred is null");
            const float2* mg = (const float2*)device_input(ctx, model_grids, C * cells * 8,
                                                           grid_location, "cube_model");
            pr = out_ptr<float2>(ctx, pred, out_location, C * (size_t)in.R * 8 + 8, "cube_pred");
            cube_degrid(ctx, g, cr, mg, pr);
        }
        tm.mark();
        if (out_location == CR_HOST) {
            if (psf) {
                copy_out(ctx, psf_grids, psf, C * cells * 4, CR_HOST);
                copy_out(ctx, dirty_grids, dirty, C * cells * 8, CR_HOST);
            }
            if (pr) copy_out(ctx, pred, pr, C * (size_t)in.R * 8, CR_HOST);
        }
        set_timings(ctx, cr_timings{tm.between(0, 1), tm.between(1, 2), tm.between(2, 3), 0.f, 0.f});
        cube_read_sums(ctx, cr, sums);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        check_device_status(ctx);
    });
}

}  // namespace

extern "C" {

const char* cr_version(void) { return "casars_cuda 0.1 (sm_103a)"; }

void cr_free_error(char* err) { std::free(err); }

int cr_ctx_create(int32_t device, cr_ctx** out, char** err) {
    return guarded(err, [&] {
        need(out != nullptr, "out is null");
        *out = nullptr;
        int n = 0;
        CR_CUDA_CHECK(cudaGetDeviceCount(&n));
        need(device >= 0 && device < n, "no such CUDA device");
        CR_CUDA_CHECK(cudaSetDevice(device));
        cr_ctx* c = new cr_ctx();
        c->device = device;
        CR_CUDA_CHECK(cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device));
        // commit the allocation-free Hogbom's static scratch on this device
        // now, so that its calls never load a module (and allocate) later
        cr::noalloc_prepare(device);
        CR_CUDA_CHECK(cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking));
        c->stream = c->own_stream;
        CR_CUDA_CHECK(cudaStreamCreateWithFlags(&c->aux_stream, cudaStreamNonBlocking));
        CR_CUDA_CHECK(cudaEventCreateWithFlags(&c->fork_ev, cudaEventDisableTiming));
        CR_CUDA_CHECK(cudaEventCreateWithFlags(&c->join_ev, cudaEventDisableTiming));
        for (auto& e : c->stage_ev)
            CR_CUDA_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        for (auto& e : c->ev) CR_CUDA_CHECK(cudaEventCreate(&e));
        for (auto& e : c->kev) CR_CUDA_CHECK(cudaEventCreate(&e));
        CR_CUDA_CHECK(cudaMallocHost(&c->pinned, 4096));
        CR_CUDA_CHECK(cudaHostAlloc((void**)&c->status_h, 64, cudaHostAllocMapped));
        *c->status_h = 0;
        CR_CUDA_CHECK(cudaHostGetDevicePointer((void**)&c->status_d, c->status_h, 0));
        *out = c;
    });
}

void cr_ctx_destroy(cr_ctx* ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->ws)
        if (kv.second.ptr) cudaFreeAsync(kv.second.ptr, ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    for (auto& kv : ctx->fft_plans) cufftDestroy(kv.second);
    for (auto& kv : ctx->fft_plans_c2c) cufftDestroy(kv.second);
    for (auto& m : ctx->fft_plans_real)
        for (auto& kv : m.second) cufftDestroy(kv.second);
    for (auto& m : ctx->fft_plans_many)
        for (auto& kv : m.second) cufftDestroy(kv.second);
    for (auto& e : ctx->ev)
        if (e) cudaEventDestroy(e);
    for (auto& e : ctx->kev)
        if (e) cudaEventDestroy(e);
    if (ctx->pinned) cudaFreeHost(ctx->pinned);
    if (ctx->status_h) cudaFreeHost(ctx->status_h);
    if (ctx->aux_stream) {
        cudaStreamSynchronize(ctx->aux_stream);
        cudaStreamDestroy(ctx->aux_stream);
    }
    if (ctx->fork_ev) cudaEventDestroy(ctx->fork_ev);
    if (ctx->join_ev) cudaEventDestroy(ctx->join_ev);
    for (auto& e : ctx->stage_ev)
        if (e) cudaEventDestroy(e);
    if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
    delete ctx;
}

int cr_ctx_set_stream(cr_ctx* ctx, void* stream, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr, "context is null");
        ctx->stream = stream ? (cudaStream_t)stream : ctx->own_stream;
    });
}

void* cr_ctx_stream(cr_ctx* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

int cr_ctx_synchronize(cr_ctx* ctx, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr, "context is null");
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_ctx_last_timings(cr_ctx* ctx, cr_timings* out) {
    if (!ctx || !out) return CR_INVALID;
    *out = ctx->timings;
    return CR_OK;
}

int64_t cr_ctx_launch_count(cr_ctx* ctx) { return ctx ? ctx->launches : -1; }

int64_t cr_ctx_workspace_bytes(cr_ctx* ctx) {
    if (!ctx) return -1;
    int64_t total = 0;
    for (const auto& kv : ctx->ws) total += (int64_t)kv.second.bytes;
    return total;
}

int cr_gridder_create(cr_ctx* ctx, const cr_geometry* geom, double padding, int32_t oversampling,
                      cr_gridder** out, cr_grid_info* info, char** err) {
    return guarded(err, [&] {
        need(ctx && geom && out, "null argument");
        *out = nullptr;
        need(geom->nx > 0 && geom->ny > 0, "image shape must be positive");
        need(std::isfinite(geom->cell_x_rad) && std::isfinite(geom->cell_y_rad) &&
                 geom->cell_x_rad > 0.0 && geom->cell_y_rad > 0.0,
             "cell sizes must be finite and positive");
        need(oversampling >= 1 && oversampling <= 254, "oversampling must be in [1, 254]");
        need(padding >= 1.0 && padding < 8.0, "padding must be in [1, 8)");
        bind(ctx);
        cr_gridder* g = new cr_gridder();
        g->ctx = ctx;
        g->geom = *geom;
        int64_t gnx = casa_composite_padded_len(geom->nx, padding);
        int64_t gny = casa_composite_padded_len(geom->ny, padding);
        g->info.grid_nx = gnx;
        g->info.grid_ny = gny;
        g->info.blc_x = image_blc(gnx, geom->nx);
        g->info.blc_y = image_blc(gny, geom->ny);
        g->info.du = 1.0 / ((double)gnx * geom->cell_x_rad);
        g->info.dv = 1.0 / ((double)gny * geom->cell_y_rad);
        g->info.oversampling = oversampling;
        g->taps_h = std_normalized_taps(oversampling, 3);
        g->tap_rows = 2 * (oversampling / 2) + 1;
        g->corr_x_h = correction_axis(gnx);
        g->corr_y_h = correction_axis(gny);
        try {
            g->taps_bytes = (uint32_t)((g->taps_h.size() * 4 + 15) & ~size_t(15));
            CR_CUDA_CHECK(cudaMalloc(&g->taps_d, g->taps_bytes));
            CR_CUDA_CHECK(cudaMemset(g->taps_d, 0, g->taps_bytes));
            std::vector<float> taps8((size_t)g->tap_rows * 8, 0.0f);
            for (int32_t r = 0; r < g->tap_rows; ++r)
                for (int k = 0; k < 7; ++k) taps8[(size_t)r * 8 + k] = g->taps_h[(size_t)r * 7 + k];
            CR_CUDA_CHECK(cudaMalloc(&g->taps8_d, taps8.size() * 4));
            CR_CUDA_CHECK(cudaMemcpy(g->taps8_d, taps8.data(), taps8.size() * 4,
                                     cudaMemcpyHostToDevice));
            CR_CUDA_CHECK(cudaMalloc(&g->corr_x_d, (size_t)gnx * 4));
            CR_CUDA_CHECK(cudaMalloc(&g->corr_y_d, (size_t)gny * 4));
            CR_CUDA_CHECK(cudaMemcpy(g->taps_d, g->taps_h.data(), g->taps_h.size() * 4, cudaMemcpyHostToDevice));
            CR_CUDA_CHECK(cudaMemcpy(g->corr_x_d, g->corr_x_h.data(), (size_t)gnx * 4, cudaMemcpyHostToDevice));
            CR_CUDA_CHECK(cudaMemcpy(g->corr_y_d, g->corr_y_h.data(), (size_t)gny * 4, cudaMemcpyHostToDevice));
        } catch (...) {
            cr_gridder_destroy(g);
            throw;
        }
        if (info) *info = g->info;
        *out = g;
    });
}

void cr_gridder_destroy(cr_gridder* g) {
    if (!g) return;
    cudaSetDevice(g->ctx->device);
    cudaStreamSynchronize(g->ctx->stream);
    g->ctx->cube_graphs.clear();   // captured pipelines may read this gridder's tables
    cudaFree(g->taps_d);
    cudaFree(g->taps8_d);
    cudaFree(g->corr_x_d);
    cudaFree(g->corr_y_d);
    delete g;
}

int cr_gridder_tables(cr_gridder* g, float* taps, float* corr_x, float* corr_y, char** err) {
    return guarded(err, [&] {
        need(g != nullptr, "gridder is null");
        if (taps) std::memcpy(taps, g->taps_h.data(), g->taps_h.size() * 4);
        if (corr_x) std::memcpy(corr_x, g->corr_x_h.data(), g->corr_x_h.size() * 4);
        if (corr_y) std::memcpy(corr_y, g->corr_y_h.data(), g->corr_y_h.size() * 4);
    });
}

int cr_wproj_create(cr_ctx* ctx, cr_gridder* g, double max_abs_w, int32_t planes,
                    int32_t sampling, int32_t support_min, int32_t support_max, cr_wproj** out,
                    cr_wproj_info* info, char** err) {
    return guarded(err, [&] {
        need(ctx && g && out, "null argument");
        need(g->ctx == ctx, "gridder belongs to another context");
        *out = nullptr;
        need(std::isfinite(max_abs_w) && max_abs_w >= 0.0, "max_abs_w must be finite");
        need(sampling <= 64, "sampling above 64");
        bind(ctx);
        cr_wproj* wp = new cr_wproj();
        wp->ctx = ctx;
        wp->g = g;
        try {
            build_wproj(ctx, wp, max_abs_w, planes, sampling, support_min, support_max);
        } catch (...) {
            cr_wproj_destroy(wp);
            throw;
        }
        if (info) *info = wp->info;
        *out = wp;
    });
}

void cr_wproj_destroy(cr_wproj* wp) {
    if (!wp) return;
    cudaSetDevice(wp->ctx->device);
    cudaStreamSynchronize(wp->ctx->stream);
    cudaFree(wp->support_d);
    cudaFree(wp->cube_off_d);
    cudaFree(wp->cube_q_d);
    cudaFree(wp->kernels_d);
    cudaFree(wp->norm_d);
    cudaFree(wp->cube_d);
    cudaFree(wp->sinc_x_d);
    cudaFree(wp->sinc_gx_d);
    cudaFree(wp->sinc_gy_d);
    cudaFree(wp->first_plane_d);
    delete wp;
}

int cr_wproj_tables(cr_wproj* wp, int32_t* support, float* kernels, float* norm, char** err) {
    return guarded(err, [&] {
        need(wp != nullptr, "W-projector is null");
        bind(wp->ctx);
        const cr_wproj_info& i = wp->info;
        if (support) std::memcpy(support, wp->support_h.data(), (size_t)i.planes * 4);
        if (kernels)
            CR_CUDA_CHECK(cudaMemcpy(kernels, wp->kernels_d,
                                     (size_t)i.planes * i.kernel_width * i.kernel_width * 8,
                                     cudaMemcpyDeviceToHost));
        if (norm)
            CR_CUDA_CHECK(cudaMemcpy(norm, wp->norm_d, (size_t)i.planes * wp->axis * wp->axis * 4,
                                     cudaMemcpyDeviceToHost));
    });
}

int cr_grid_dirty(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                  float* psf_grid, float* dirty_grid, int32_t out_location, cr_sums* sums,
                  char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr, "context is null");
        check_wp(g, wp);
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        StagedBatch b(ctx, batch, wp != nullptr);
        size_t gb = grid_bytes(g);
        float2* psf = out_ptr<float2>(ctx, psf_grid, out_location, gb, "psf_grid");
        float2* dirty = out_ptr<float2>(ctx, dirty_grid, out_location, gb, "dirty_grid");
        CR_CUDA_CHECK(cudaMemsetAsync(psf, 0, gb, ctx->stream));
        CR_CUDA_CHECK(cudaMemsetAsync(dirty, 0, gb, ctx->stream));
        Records r = plan(ctx, g, wp, b);
        tm.mark();
        grid_records(ctx, g, wp, r, psf, dirty, 0);
        tm.mark();
        if (out_location == CR_HOST) {
            copy_out(ctx, psf_grid, psf, gb, CR_HOST);
            copy_out(ctx, dirty_grid, dirty, gb, CR_HOST);
        }
        cr_sums s{};
        read_sums(ctx, r, &s);
        if (sums) *sums = s;
        set_timings(ctx, cr_timings{tm.between(0, 1), tm.between(1, 2), 0.f, 0.f, 0.f});
    });
}

int cr_degrid(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
              const float* model_grid, int32_t grid_location, float* pred, int32_t out_location,
              char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && model_grid != nullptr, "null argument");
        check_wp(g, wp);
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        StagedBatch b(ctx, batch, wp != nullptr);
        const float2* grid = (const float2*)device_input(ctx, model_grid, grid_bytes(g),
                                                         grid_location, "model_grid");
        Records r = plan(ctx, g, wp, b);
        tm.mark();
        degrid_records(ctx, g, wp, r, grid);
        float2* out = out_ptr<float2>(ctx, pred, out_location, (size_t)b.n * 8 + 8, "pred");
        broadcast_pred(ctx, r, out);
        tm.mark();
        if (out_location == CR_HOST) copy_out(ctx, pred, out, (size_t)b.n * 8, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        set_timings(ctx, cr_timings{tm.between(0, 1), 0.f, tm.between(1, 2), 0.f, 0.f});
    });
}

int cr_grid_residual(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                     const float* model_grid, int32_t grid_location, float* residual_grid,
                     int32_t out_location, cr_sums* sums, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr, "context is null");
        check_wp(g, wp);
        bind(ctx);
        StagedBatch b(ctx, batch, wp != nullptr);
        size_t gb = grid_bytes(g);
        Records r = plan(ctx, g, wp, b);
        if (model_grid) {
            const float2* grid = (const float2*)device_input(ctx, model_grid, gb, grid_location,
                                                             "model_grid");
            degrid_records(ctx, g, wp, r, grid);
        } else {
            CR_CUDA_CHECK(cudaMemsetAsync(r.rec_pred, 0, (size_t)(b.n > 0 ? b.n : 1) * 8, ctx->stream));
        }
        float2* res = out_ptr<float2>(ctx, residual_grid, out_location, gb, "residual_grid");
        CR_CUDA_CHECK(cudaMemsetAsync(res, 0, gb, ctx->stream));
        grid_records(ctx, g, wp, r, nullptr, res, 1);
        if (out_location == CR_HOST) copy_out(ctx, residual_grid, res, gb, CR_HOST);
        cr_sums s{};
        read_sums(ctx, r, &s);
        if (sums) *sums = s;
    });
}

// Whether the image-stage FFTs of single-plane calls run in FP32 (the
// dirty-product policy's F32 choice, lib.rs:1280-1312 and 2428-2472).
static bool image_single(const cr_ctx* ctx) { return ctx->image_fft_bits == 32; }

int cr_grid_to_image(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float* grid,
                     int32_t grid_location, float scale, float* image, int32_t out_location,
                     char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && grid != nullptr, "null argument");
        check_wp(g, wp);
        bind(ctx);
        size_t gb = grid_bytes(g);
        float2* work = (float2*)workspace(ctx, "fft_grid", gb);
        CR_CUDA_CHECK(cudaMemcpyAsync(work, grid, gb,
                                      grid_location == CR_HOST ? cudaMemcpyHostToDevice
                                                               : cudaMemcpyDeviceToDevice,
                                      ctx->stream));
        size_t ib = image_pixels(g) * 4;
        float* img = out_ptr<float>(ctx, image, out_location, ib, "image");
        grid_to_image(ctx, g, wp, work, scale, img, image_single(ctx));
        if (out_location == CR_HOST) copy_out(ctx, image, img, ib, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_image_to_grid(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const float* model,
                     int32_t model_location, float* grid, int32_t out_location, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && model != nullptr, "null argument");
        check_wp(g, wp);
        bind(ctx);
        const float* m = (const float*)device_input(ctx, model, image_pixels(g) * 4,
                                                    model_location, "model");
        size_t gb = grid_bytes(g);
        float2* out = out_ptr<float2>(ctx, grid, out_location, gb, "model_grid");
        image_to_grid(ctx, g, wp, m, out, image_single(ctx));
        if (out_location == CR_HOST) copy_out(ctx, grid, out, gb, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

// dirty_grids_to_psf_and_residual_owned (lib.rs:48987-49130): PSF and dirty
// grids with their sums -> normalised PSF and residual images and the PSF
// state (synchronises).
static void dirty_products(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, float2* psf, float2* dirty,
                           const cr_sums& s, float* psf_out, float* residual_out,
                           int32_t out_location, cr_psf_state* state) {
    if (s.normalization_sumwt <= 0.0 || s.reported_sumwt <= 0.0)
        fail(CR_NO_SAMPLES, "no usable samples");
    const float k = wp ? 2.0f : 1.0f;
    const float sumwt_f = (float)s.normalization_sumwt;
    const size_t np = image_pixels(g);
    float* psf_img = out_ptr<float>(ctx, psf_out, out_location, np * 4, "psf_image");
    float* res_img = out_ptr<float>(ctx, residual_out, out_location, np * 4, "res_image");
    unsigned int* peak_d = (unsigned int*)workspace(ctx, "di_peak", 4);
    grid_to_image(ctx, g, wp, psf, k / sumwt_f, psf_img, image_single(ctx));
    abs_peak(ctx, psf_img, (int64_t)np, peak_d);
    // the scaling reads the peak on the device; the host checks it once both
    // images are done, so nothing waits in between
    unsigned int* peak_h = (unsigned int*)((char*)ctx->pinned + 256);
    CR_CUDA_CHECK(cudaMemcpyAsync(peak_h, peak_d, 4, cudaMemcpyDeviceToHost, ctx->stream));
    scale_image(ctx, psf_img, (int64_t)np, 1.0f, peak_d);
    AuxFork fork(ctx);
    if (out_location == CR_HOST) {
        // the PSF image goes back while the residual is transformed
        fork.to_aux();
        copy_out(ctx, psf_out, psf_img, np * 4, CR_HOST);
        fork.to_main();
    }
    grid_to_image(ctx, g, wp, dirty, k / sumwt_f, res_img, image_single(ctx));
    scale_image(ctx, res_img, (int64_t)np, 1.0f, peak_d);
    if (out_location == CR_HOST) copy_out(ctx, residual_out, res_img, np * 4, CR_HOST);
    fork.join();
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    float peak;
    std::memcpy(&peak, peak_h, 4);
    if (!(std::isfinite(peak) && peak > 0.0f))
        fail(CR_NORMALIZATION, "PSF peak is non-finite or zero");
    if (state) *state = cr_psf_state{peak, sumwt_f, (float)s.reported_sumwt};
}

int cr_dirty_image(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                   float* psf_out, float* residual_out, int32_t out_location,
                   cr_psf_state* state, cr_sums* sums, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr, "context is null");
        check_wp(g, wp);
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        StagedBatch b(ctx, batch, wp != nullptr);
        size_t gb = grid_bytes(g);
        float2* psf = (float2*)workspace(ctx, "di_psf", gb);
        float2* dirty = (float2*)workspace(ctx, "di_dirty", gb);
        CR_CUDA_CHECK(cudaMemsetAsync(psf, 0, gb, ctx->stream));
        CR_CUDA_CHECK(cudaMemsetAsync(dirty, 0, gb, ctx->stream));
        Records r = plan(ctx, g, wp, b);
        tm.mark();
        grid_records(ctx, g, wp, r, psf, dirty, 0);
        tm.mark();
        cr_sums s{};
        read_sums(ctx, r, &s);
        if (sums) *sums = s;
        dirty_products(ctx, g, wp, psf, dirty, s, psf_out, residual_out, out_location, state);
        tm.mark();
        set_timings(ctx, cr_timings{tm.between(0, 1), tm.between(1, 2), 0.f, tm.between(2, 3), 0.f});
    });
}

int cr_residual_image(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                      const float* model, int32_t model_location, const cr_psf_state* state,
                      float* residual_out, int32_t out_location, cr_sums* sums, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && state != nullptr && model != nullptr, "null argument");
        need(state->normalization_sumwt > 0.0f && state->psf_peak > 0.0f, "invalid PSF state");
        check_wp(g, wp);
        bind(ctx);
        StagedBatch b(ctx, batch, wp != nullptr);
        size_t gb = grid_bytes(g);
        const size_t np = image_pixels(g);
        const float* m = (const float*)device_input(ctx, model, np * 4, model_location, "model");
        float2* mgrid = (float2*)workspace(ctx, "ri_model_grid", gb);
        image_to_grid(ctx, g, wp, m, mgrid, image_single(ctx));
        Records r = plan(ctx, g, wp, b);
        degrid_records(ctx, g, wp, r, mgrid);
        float2* res = (float2*)workspace(ctx, "ri_residual_grid", gb);
        CR_CUDA_CHECK(cudaMemsetAsync(res, 0, gb, ctx->stream));
        grid_records(ctx, g, wp, r, nullptr, res, 1);
        float* img = out_ptr<float>(ctx, residual_out, out_location, np * 4, "ri_image");
        const float k = wp ? 2.0f : 1.0f;
        grid_to_image(ctx, g, wp, res, k / state->normalization_sumwt, img, image_single(ctx));
        scale_image(ctx, img, (int64_t)np, 1.0f / state->psf_peak, nullptr);
        if (out_location == CR_HOST) copy_out(ctx, residual_out, img, np * 4, CR_HOST);
        cr_sums s{};
        read_sums(ctx, r, &s);
        if (sums) *sums = s;
    });
}

int cr_predict(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
               const float* model, int32_t model_location, float* pred, int32_t out_location,
               char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && model != nullptr, "null argument");
        check_wp(g, wp);
        bind(ctx);
        StagedBatch b(ctx, batch, wp != nullptr);
        size_t gb = grid_bytes(g);
        // the model's upload and transform run beside the plan
        AuxFork fork(ctx);
        fork.to_aux();
        const float* m = (const float*)device_input(ctx, model, image_pixels(g) * 4,
                                                    model_location, "model");
        float2* mgrid = (float2*)workspace(ctx, "pr_model_grid", gb);
        image_to_grid(ctx, g, wp, m, mgrid, image_single(ctx));
        fork.to_main();
        Records r = plan(ctx, g, wp, b);
        fork.join();
        degrid_records(ctx, g, wp, r, mgrid);
        float2* out = out_ptr<float2>(ctx, pred, out_location, (size_t)b.n * 8 + 8, "pred");
        broadcast_pred(ctx, r, out);
        if (out_location == CR_HOST) copy_out(ctx, pred, out, (size_t)b.n * 8, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_adjoint(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
               float* image, int32_t out_location, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr, "context is null");
        check_wp(g, wp);
        bind(ctx);
        StagedBatch b(ctx, batch, wp != nullptr);
        size_t gb = grid_bytes(g);
        Records r = plan(ctx, g, wp, b);
        CR_CUDA_CHECK(cudaMemsetAsync(r.rec_pred, 0, (size_t)(b.n > 0 ? b.n : 1) * 8, ctx->stream));
        float2* grid = (float2*)workspace(ctx, "adj_grid", gb);
        CR_CUDA_CHECK(cudaMemsetAsync(grid, 0, gb, ctx->stream));
        grid_records(ctx, g, wp, r, nullptr, grid, 1);
        const size_t np = image_pixels(g);
        float* img = out_ptr<float>(ctx, image, out_location, np * 4, "adj_image");
        // F^H = (Nx Ny) x the scaled inverse; the image-side factor is the
        // forward apodisation's (corr, times sinc for W-projection)
        float n2 = (float)((double)g->info.grid_nx * (double)g->info.grid_ny);
        grid_to_image_adjoint(ctx, g, wp, grid, n2, img, image_single(ctx));
        if (out_location == CR_HOST) copy_out(ctx, image, img, np * 4, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_plan_create(cr_ctx* ctx, cr_gridder* g, cr_wproj* wp, const cr_vis_batch* batch,
                   cr_plan** out, cr_sums* sums, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && out != nullptr, "null argument");
        check_wp(g, wp);
        *out = nullptr;
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        StagedBatch b(ctx, batch, wp != nullptr);
        cr_plan* p = new cr_plan();
        p->ctx = ctx;
        p->g = g;
        p->wp = wp;
        try {
            p->rec = plan(ctx, g, wp, b, &p->pool);
            tm.mark();
            read_sums(ctx, p->rec, &p->sums);
        } catch (...) {
            cr_plan_destroy(p);
            throw;
        }
        if (sums) *sums = p->sums;
        set_timings(ctx, cr_timings{tm.between(0, 1), 0.f, 0.f, 0.f, 0.f});
        *out = p;
    });
}

void cr_plan_destroy(cr_plan* p) {
    if (!p) return;
    cudaSetDevice(p->ctx->device);
    // the frees are ordered on the context's stream after the plan's work
    pool_free(p->ctx, p->pool);
    delete p;
}

int cr_plan_grid_dirty(cr_ctx* ctx, cr_plan* p, float* psf_grid, float* dirty_grid,
                       int32_t out_location, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && p != nullptr && p->ctx == ctx, "plan belongs to another context");
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        size_t gb = grid_bytes(p->g);
        float2* psf = out_ptr<float2>(ctx, psf_grid, out_location, gb, "psf_grid");
        float2* dirty = out_ptr<float2>(ctx, dirty_grid, out_location, gb, "dirty_grid");
        CR_CUDA_CHECK(cudaMemsetAsync(psf, 0, gb, ctx->stream));
        CR_CUDA_CHECK(cudaMemsetAsync(dirty, 0, gb, ctx->stream));
        grid_records(ctx, p->g, p->wp, p->rec, psf, dirty, 0);
        tm.mark();
        if (out_location == CR_HOST) {
            copy_out(ctx, psf_grid, psf, gb, CR_HOST);
            copy_out(ctx, dirty_grid, dirty, gb, CR_HOST);
        }
        set_timings(ctx, cr_timings{0.f, tm.between(0, 1), 0.f, 0.f, 0.f});
    });
}

int cr_plan_degrid(cr_ctx* ctx, cr_plan* p, const float* model_grid, int32_t grid_location,
                   float* pred, int32_t out_location, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && p != nullptr && p->ctx == ctx, "plan belongs to another context");
        need(model_grid != nullptr, "model grid is null");
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        const float2* grid = (const float2*)device_input(ctx, model_grid, grid_bytes(p->g),
                                                         grid_location, "model_grid");
        degrid_records(ctx, p->g, p->wp, p->rec, grid);
        size_t n = (size_t)p->rec.n_samples;
        float2* out = out_ptr<float2>(ctx, pred, out_location, n * 8 + 8, "pred");
        broadcast_pred(ctx, p->rec, out);
        tm.mark();
        if (out_location == CR_HOST) copy_out(ctx, pred, out, n * 8, CR_HOST);
        set_timings(ctx, cr_timings{0.f, 0.f, tm.between(0, 1), 0.f, 0.f});
    });
}

int cr_plan_grid_residual(cr_ctx* ctx, cr_plan* p, const float* model_grid,
                          int32_t grid_location, float* residual_grid, int32_t out_location,
                          char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && p != nullptr && p->ctx == ctx, "plan belongs to another context");
        bind(ctx);
        size_t gb = grid_bytes(p->g);
        size_t n = (size_t)(p->rec.n_samples > 0 ? p->rec.n_samples : 1);
        if (model_grid) {
            const float2* grid = (const float2*)device_input(ctx, model_grid, gb, grid_location,
                                                             "model_grid");
            degrid_records(ctx, p->g, p->wp, p->rec, grid);
        } else {
            CR_CUDA_CHECK(cudaMemsetAsync(p->rec.rec_pred, 0, n * 8, ctx->stream));
        }
        float2* res = out_ptr<float2>(ctx, residual_grid, out_location, gb, "residual_grid");
        CR_CUDA_CHECK(cudaMemsetAsync(res, 0, gb, ctx->stream));
        grid_records(ctx, p->g, p->wp, p->rec, nullptr, res, 1);
        if (out_location == CR_HOST) copy_out(ctx, residual_grid, res, gb, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_plan_residual_image(cr_ctx* ctx, cr_plan* p, const float* model, int32_t model_location,
                           const cr_psf_state* state, float* residual_out, int32_t out_location,
                           char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && p != nullptr && p->ctx == ctx, "plan belongs to another context");
        need(model != nullptr && state != nullptr, "null argument");
        need(state->normalization_sumwt > 0.0f && state->psf_peak > 0.0f, "invalid PSF state");
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        const size_t gb = grid_bytes(p->g);
        const size_t np = image_pixels(p->g);
        const float* m = (const float*)device_input(ctx, model, np * 4, model_location, "model");
        float2* mgrid = (float2*)workspace(ctx, "ri_model_grid", gb);
        image_to_grid(ctx, p->g, p->wp, m, mgrid, image_single(ctx));
        tm.mark();
        degrid_records(ctx, p->g, p->wp, p->rec, mgrid);
        tm.mark();
        float2* res = (float2*)workspace(ctx, "ri_residual_grid", gb);
        CR_CUDA_CHECK(cudaMemsetAsync(res, 0, gb, ctx->stream));
        grid_records(ctx, p->g, p->wp, p->rec, nullptr, res, 1);
        tm.mark();
        float* img = out_ptr<float>(ctx, residual_out, out_location, np * 4, "ri_image");
        const float k = p->wp ? 2.0f : 1.0f;
        grid_to_image(ctx, p->g, p->wp, res, k / state->normalization_sumwt, img,
                      image_single(ctx));
        scale_image(ctx, img, (int64_t)np, 1.0f / state->psf_peak, nullptr);
        tm.mark();
        if (out_location == CR_HOST) copy_out(ctx, residual_out, img, np * 4, CR_HOST);
        set_timings(ctx, cr_timings{0.f, tm.between(2, 3), tm.between(1, 2),
                                  tm.between(0, 1) + tm.between(3, 4), 0.f});
    });
}

static int apply_weighting_conv(cr_ctx* ctx, cr_gridder* g, const cr_vis_batch* batch,
                                int32_t mode, float robust, float* out_weight,
                                int32_t out_location, float* f2, int32_t convention, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && g != nullptr, "null argument");
        bind(ctx);
        DeviceBatch b = device_batch(ctx, batch, false);
        float* out = out_ptr<float>(ctx, out_weight, out_location, (size_t)b.n * 4 + 4, "weights");
        apply_weighting(ctx, g, b, mode, robust, out, f2, convention);
        if (out_location == CR_HOST) copy_out(ctx, out_weight, out, (size_t)b.n * 4, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_apply_weighting(cr_ctx* ctx, cr_gridder* g, const cr_vis_batch* batch, int32_t mode,
                       float robust, float* out_weight, int32_t out_location, float* f2,
                       char** err) {
    return apply_weighting_conv(ctx, g, batch, mode, robust, out_weight, out_location, f2, 0,
                                err);
}

int cr_apply_weighting_plane(cr_ctx* ctx, cr_gridder* g, const cr_vis_batch* batch,
                             int32_t mode, float robust, float* out_weight,
                             int32_t out_location, float* f2, char** err) {
    return apply_weighting_conv(ctx, g, batch, mode, robust, out_weight, out_location, f2, 1,
                                err);
}

int cr_apply_weighting_rows(cr_ctx* ctx, cr_gridder* g, const cr_vis_batch* batch,
                            const double* density_u, const double* density_v, int32_t mode,
                            float robust, float* out_weight, int32_t out_location, float* f2,
                            char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && g != nullptr, "null argument");
        bind(ctx);
        DeviceBatch b = device_batch(ctx, batch, false);
        const size_t n = (size_t)b.n;
        need(b.n == 0 || (density_u && density_v), "density coordinates are null");
        const double* du = (const double*)device_input(ctx, density_u, n * 8, batch->location,
                                                       "density_u");
        const double* dv = (const double*)device_input(ctx, density_v, n * 8, batch->location,
                                                       "density_v");
        float* out = out_ptr<float>(ctx, out_weight, out_location, n * 4 + 4, "weights");
        apply_weighting(ctx, g, b, mode, robust, out, f2, 0, du, dv);
        if (out_location == CR_HOST) copy_out(ctx, out_weight, out, n * 4, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_row_runs_prepare(cr_ctx* ctx, const cr_row_runs* runs, const cr_polarization* pol,
                        double* u, double* v, double* w, float* weight, float* sumwt_factor,
                        uint8_t* gridable, float* vis, double* density_u, double* density_v,
                        int32_t out_location, int64_t* n_out, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && runs != nullptr && pol != nullptr && n_out != nullptr,
             "null argument");
        bind(ctx);
        need(runs->rows >= 0 && runs->channels > 0, "row runs need rows >= 0 and channels > 0");
        const size_t n = (size_t)runs->rows * (size_t)runs->channels;
        StageTimer tm(ctx);
        tm.mark();
        RowsOut o;
        o.u = out_ptr<double>(ctx, u, out_location, n * 8 + 8, "rr_u");
        o.v = out_ptr<double>(ctx, v, out_location, n * 8 + 8, "rr_v");
        o.w = out_ptr<double>(ctx, w, out_location, n * 8 + 8, "rr_w");
        o.du = out_ptr<double>(ctx, density_u, out_location, n * 8 + 8, "rr_du");
        o.dv = out_ptr<double>(ctx, density_v, out_location, n * 8 + 8, "rr_dv");
        o.weight = out_ptr<float>(ctx, weight, out_location, n * 4 + 4, "rr_wt");
        o.sumwt_factor = out_ptr<float>(ctx, sumwt_factor, out_location, n * 4 + 4, "rr_sf");
        o.gridable = out_ptr<uint8_t>(ctx, gridable, out_location, n + 1, "rr_grd");
        o.vis = out_ptr<float2>(ctx, vis, out_location, n * 8 + 8, "rr_vis");
        const int64_t k = prepare_rows(ctx, runs, pol, o);
        tm.mark();
        if (out_location == CR_HOST) {
            const size_t m = (size_t)k;
            copy_out(ctx, u, o.u, m * 8, CR_HOST);
            copy_out(ctx, v, o.v, m * 8, CR_HOST);
            copy_out(ctx, w, o.w, m * 8, CR_HOST);
            copy_out(ctx, density_u, o.du, m * 8, CR_HOST);
            copy_out(ctx, density_v, o.dv, m * 8, CR_HOST);
            copy_out(ctx, weight, o.weight, m * 4, CR_HOST);
            copy_out(ctx, sumwt_factor, o.sumwt_factor, m * 4, CR_HOST);
            copy_out(ctx, gridable, o.gridable, m, CR_HOST);
            copy_out(ctx, vis, o.vis, m * 8, CR_HOST);
            CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        }
        *n_out = k;
        set_timings(ctx, cr_timings{tm.between(0, 1), 0.f, 0.f, 0.f, 0.f});
    });
}

int cr_polarization_for_plane(int32_t plane, const int32_t* corr_types, int32_t correlations,
                              cr_polarization* out, char** err) {
    return guarded(err, [&] {
        need(out != nullptr && (correlations == 0 || corr_types != nullptr), "null argument");
        need(plane >= 0 && plane <= 7, "plane must be 0..7");
        auto find = [&](int32_t code) {
            for (int32_t k = 0; k < correlations; ++k)
                if (corr_types[k] == code) return k;
            return -1;
        };
        // the pairs of derive_pair_selection: (first, second) codes
        const int32_t xx = find(9), yy = find(12), xy = find(10), yx = find(11);
        const int32_t rr = find(5), ll = find(8), rl = find(6), lr = find(7);
        cr_polarization p{1, -1, -1, 0, plane == 0 ? 2.0f : 1.0f};
        auto pick = [&](int32_t a, int32_t b, int32_t transform) {
            if (a < 0 || b < 0) return false;
            p.corr0 = a;
            p.corr1 = b;
            p.transform = transform;
            return true;
        };
        bool ok = false;
        switch (plane) {
            case 0: ok = pick(xx, yy, 0) || pick(rr, ll, 0); break;
            case 1: ok = pick(xx, yy, 1) || pick(rl, lr, 0); break;
            case 2: ok = pick(xy, yx, 0) || pick(rl, lr, 2); break;
            case 3: ok = pick(xy, yx, 3) || pick(rr, ll, 1); break;
            default: {
                const int32_t codes[4] = {9, 12, 5, 8};   // XX, YY, RR, LL
                const int32_t k = find(codes[plane - 4]);
                if (k >= 0) {
                    p = cr_polarization{0, k, k, 0, 1.0f};
                    ok = true;
                }
            }
        }
        if (!ok) fail(CR_INVALID, "the correlations cannot form this plane");
        *out = p;
    });
}

int cr_hogbom(cr_ctx* ctx, float* model, float* residual, const float* psf, const uint8_t* mask,
              int32_t nx, int32_t ny, int32_t location, float gain, float threshold,
              float cycle_threshold, float nsigma_threshold, int64_t cycle_niter,
              int32_t inclusive, int32_t* comp_x, int32_t* comp_y, float* comp_peak,
              float* comp_flux, int64_t* actual, int64_t* reported, int32_t* stop_reason,
              char** err) {
    return guarded(err, [&] {
        need(ctx && model && residual && psf, "null argument");
        need(nx > 0 && ny > 0, "image shape must be positive");
        need(location == CR_HOST || location == CR_DEVICE, "bad location");
        need(!comp_x == !comp_y && !comp_x == !comp_peak && !comp_x == !comp_flux,
             "component arrays must be all given or all null");
        bind(ctx);
        size_t nb = (size_t)nx * ny * 4;
        float* m = location == CR_DEVICE ? model : (float*)workspace(ctx, "hog_model", nb);
        float* r = location == CR_DEVICE ? residual : (float*)workspace(ctx, "hog_residual", nb);
        if (location == CR_HOST) {
            CR_CUDA_CHECK(cudaMemcpyAsync(m, model, nb, cudaMemcpyHostToDevice, ctx->stream));
            CR_CUDA_CHECK(cudaMemcpyAsync(r, residual, nb, cudaMemcpyHostToDevice, ctx->stream));
        }
        const float* p = (const float*)device_input(ctx, psf, nb, location, "hog_psf");
        const uint8_t* mk = (const uint8_t*)device_input(ctx, mask, (size_t)nx * ny, location,
                                                         "hog_mask");
        cr::hogbom(ctx, m, r, p, mk, nx, ny, gain, threshold, cycle_threshold, nsigma_threshold,
                   cycle_niter, inclusive, comp_x, comp_y, comp_peak, comp_flux, actual, reported,
                   stop_reason);
        if (location == CR_HOST) {
            CR_CUDA_CHECK(cudaMemcpyAsync(model, m, nb, cudaMemcpyDeviceToHost, ctx->stream));
            CR_CUDA_CHECK(cudaMemcpyAsync(residual, r, nb, cudaMemcpyDeviceToHost, ctx->stream));
        }
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_robust_rms(cr_ctx* ctx, const float* images, const uint8_t* masks, int32_t nimages,
                  int32_t nx, int32_t ny, int32_t location, const int32_t* planes,
                  int32_t nplanes, float* rms, double* madfm, int64_t* counts, char** err) {
    return guarded(err, [&] {
        need(ctx && images, "null argument");
        need(nx > 0 && ny > 0 && nimages > 0, "image shape must be positive");
        need(nplanes >= 0 && (nplanes == 0 || planes), "planes must be given");
        need(location == CR_HOST || location == CR_DEVICE, "bad location");
        for (int32_t k = 0; k < nplanes; ++k)
            need(planes[k] >= 0 && planes[k] < nimages, "plane index out of range");
        bind(ctx);
        const int64_t npix = (int64_t)nx * ny;
        need(npix < (1ll << 31), "image larger than 2^31 pixels");
        const float* im = (const float*)device_input(ctx, images, (size_t)nimages * npix * 4,
                                                     location, "rms_images");
        const uint8_t* mk = (const uint8_t*)device_input(ctx, masks, (size_t)nimages * npix,
                                                         location, "rms_masks");
        std::vector<int> pl(planes, planes + nplanes);
        cr::robust_rms(ctx, im, mk, npix, pl, rms, madfm, counts);
    });
}

int cr_hogbom_plane(cr_ctx* ctx, float* model, float* residual, const float* psf,
                    const uint8_t* mask, int32_t nx, int32_t ny, int32_t location, float gain,
                    float threshold, float cycle_threshold, float peak_relative_tolerance,
                    int64_t cycle_limit, int32_t inclusive, int32_t* comp_x, int32_t* comp_y,
                    float* comp_peak, float* comp_flux, int64_t* actual, int64_t* reported,
                    char** err) {
    return guarded(err, [&] {
        need(ctx && model && residual && psf, "null argument");
        need(nx > 0 && ny > 0, "image shape must be positive");
        need(location == CR_HOST || location == CR_DEVICE, "bad location");
        need(!comp_x == !comp_y && !comp_x == !comp_peak && !comp_x == !comp_flux,
             "component arrays must be all given or all null");
        bind(ctx);
        size_t nb = (size_t)nx * ny * 4;
        float* m = location == CR_DEVICE ? model : (float*)workspace(ctx, "hog_model", nb);
        float* r = location == CR_DEVICE ? residual : (float*)workspace(ctx, "hog_residual", nb);
        if (location == CR_HOST) {
            CR_CUDA_CHECK(cudaMemcpyAsync(m, model, nb, cudaMemcpyHostToDevice, ctx->stream));
            CR_CUDA_CHECK(cudaMemcpyAsync(r, residual, nb, cudaMemcpyHostToDevice, ctx->stream));
        }
        const float* p = (const float*)device_input(ctx, psf, nb, location, "hog_psf");
        const uint8_t* mk = (const uint8_t*)device_input(ctx, mask, (size_t)nx * ny, location,
                                                         "hog_mask");
        cr::hogbom_plane(ctx, m, r, p, mk, nx, ny, gain, threshold, cycle_threshold,
                         peak_relative_tolerance, cycle_limit, inclusive, comp_x, comp_y,
                         comp_peak, comp_flux, actual, reported);
        if (location == CR_HOST) {
            CR_CUDA_CHECK(cudaMemcpyAsync(model, m, nb, cudaMemcpyDeviceToHost, ctx->stream));
            CR_CUDA_CHECK(cudaMemcpyAsync(residual, r, nb, cudaMemcpyDeviceToHost, ctx->stream));
        }
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_cube_grid_dirty(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch,
                       int32_t weighting, float robust, float* psf_grids, float* dirty_grids,
                       int32_t out_location, cr_sums* sums, char** err) {
    if (!psf_grids || !dirty_grids) {
        set_err(err, "psf_grids and dirty_grids are required");
        return CR_INVALID;
    }
    return cube_run(ctx, g, batch, weighting, robust, psf_grids, dirty_grids, nullptr, CR_HOST,
                    nullptr, out_location, sums, err);
}

int cr_cube_degrid(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch, int32_t weighting,
                   float robust, const float* model_grids, int32_t grid_location, float* pred,
                   int32_t out_location, char** err) {
    if (!model_grids) {
        set_err(err, "model_grids is required");
        return CR_INVALID;
    }
    return cube_run(ctx, g, batch, weighting, robust, nullptr, nullptr, model_grids,
                    grid_location, pred, out_location, nullptr, err);
}

int cr_cube_grid_degrid(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch,
                        int32_t weighting, float robust, float* psf_grids, float* dirty_grids,
                        const float* model_grids, int32_t grid_location, float* pred,
                        int32_t out_location, cr_sums* sums, char** err) {
    if (!psf_grids || !dirty_grids || !model_grids) {
        set_err(err, "psf_grids, dirty_grids and model_grids are required");
        return CR_INVALID;
    }
    return cube_run(ctx, g, batch, weighting, robust, psf_grids, dirty_grids, model_grids,
                    grid_location, pred, out_location, sums, err);
}

int cr_cube_sample_taps(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch,
                        int32_t weighting, float robust, int32_t* start_x, int32_t* start_y,
                        int32_t* row_x, int32_t* row_y, float* imaging_weight,
                        int32_t out_location, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && g != nullptr, "null argument");
        need(start_x && start_y && row_x && row_y && imaging_weight, "output is null");
        bind(ctx);
        CubeInput in = cube_input(ctx, batch);
        const size_t S = (size_t)in.C * (size_t)in.R;
        CubeTaps t;
        t.start_x = out_ptr<int32_t>(ctx, start_x, out_location, S * 4 + 4, "taps_sx");
        t.start_y = out_ptr<int32_t>(ctx, start_y, out_location, S * 4 + 4, "taps_sy");
        t.row_x = out_ptr<int32_t>(ctx, row_x, out_location, S * 4 + 4, "taps_rx");
        t.row_y = out_ptr<int32_t>(ctx, row_y, out_location, S * 4 + 4, "taps_ry");
        t.weight = out_ptr<float>(ctx, imaging_weight, out_location, S * 4 + 4, "taps_w");
        cube_plan(ctx, g, in, weighting, robust, &t);
        if (out_location == CR_HOST) {
            copy_out(ctx, start_x, t.start_x, S * 4, CR_HOST);
            copy_out(ctx, start_y, t.start_y, S * 4, CR_HOST);
            copy_out(ctx, row_x, t.row_x, S * 4, CR_HOST);
            copy_out(ctx, row_y, t.row_y, S * 4, CR_HOST);
            copy_out(ctx, imaging_weight, t.weight, S * 4, CR_HOST);
        }
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_fit_beam(cr_ctx* ctx, const float* psf, int32_t nx, int32_t ny, int32_t location,
                double cell_x_rad, double cell_y_rad, float cutoff, cr_beam* beam,
                int32_t* fitted, int32_t* attempts, float* cutoff_used, char** err) {
    return guarded(err, [&] {
        need(psf && beam && fitted, "null argument");
        need(nx > 0 && ny > 0, "image shape must be positive");
        const size_t n = (size_t)nx * (size_t)ny;
        std::vector<float> host;
        const float* p = psf;
        if (location == CR_DEVICE) {
            need(ctx != nullptr, "a device PSF needs a context");
            bind(ctx);
            host.resize(n);
            CR_CUDA_CHECK(cudaMemcpyAsync(host.data(), psf, n * 4, cudaMemcpyDeviceToHost,
                                          ctx->stream));
            CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
            p = host.data();
        } else {
            need(location == CR_HOST, "location must be CR_HOST or CR_DEVICE");
        }
        int32_t at = 0;
        float cu = 0.0f;
        *beam = cr_beam{0.0, 0.0, 0.0};
        *fitted = fit_beam(p, nx, ny, cell_x_rad, cell_y_rad, cutoff, beam, &at, &cu) ? 1 : 0;
        if (attempts) *attempts = at;
        if (cutoff_used) *cutoff_used = cu;
    });
}

int cr_restore(cr_ctx* ctx, const float* model, const float* residual, int32_t nx, int32_t ny,
               int32_t location, double cell_x_rad, double cell_y_rad, const cr_beam* beam,
               float* restored, int32_t out_location, char** err) {
    return guarded(err, [&] {
        need(ctx && model && beam, "null argument");
        need(nx > 0 && ny > 0, "image shape must be positive");
        bind(ctx);
        const size_t n = (size_t)nx * (size_t)ny;
        const float* m = (const float*)device_input(ctx, model, n * 4, location, "rs_in_model");
        const float* r = (const float*)device_input(ctx, residual, n * 4, location, "rs_in_res");
        float* out = out_ptr<float>(ctx, restored, out_location, n * 4, "restored");
        restore(ctx, m, r, nx, ny, cell_x_rad, cell_y_rad, *beam, out);
        if (out_location == CR_HOST) copy_out(ctx, restored, out, n * 4, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    });
}

int cr_psf_sidelobe(cr_ctx* ctx, const float* psf, int32_t nx, int32_t ny, int32_t location,
                    double cell_x_rad, double cell_y_rad, const cr_beam* beam, float* level,
                    char** err) {
    return guarded(err, [&] {
        need(ctx && psf && beam && level, "null argument");
        need(nx > 0 && ny > 0, "image shape must be positive");
        bind(ctx);
        const size_t n = (size_t)nx * (size_t)ny;
        const float* p = (const float*)device_input(ctx, psf, n * 4, location, "sl_psf");
        *level = psf_sidelobe(ctx, p, nx, ny, cell_x_rad, cell_y_rad, *beam);
    });
}

int cr_ctx_set_cube_grid_chunk(cr_ctx* ctx, int32_t chunk) {
    if (!ctx) return CR_INVALID;
    if (chunk != 0 && !cr::cube_grid_chunk_valid((uint32_t)chunk)) return CR_INVALID;
    ctx->cube_chunk_forced = (uint32_t)chunk;
    ctx->cube_graphs.clear();
    return CR_OK;
}

int cr_ctx_set_wait_limits(cr_ctx* ctx, int64_t barrier_polls, int64_t mbar_polls) {
    if (!ctx) return CR_INVALID;
    ctx->barrier_polls = barrier_polls < 0 ? cr::kBarrierPollsDefault : barrier_polls;
    ctx->mbar_polls = mbar_polls < 0 ? cr::kMbarPollsDefault : mbar_polls;
    // captured pipelines hold the kernels' arguments, limits included
    ctx->cube_graphs.clear();
    return CR_OK;
}

int cr_ctx_set_cube_graphs(cr_ctx* ctx, int32_t enable) {
    if (!ctx) return CR_INVALID;
    ctx->cube_graphs_enabled = enable != 0;
    if (!enable) ctx->cube_graphs.clear();
    return CR_OK;
}

// FftPrecisionChoice {Auto, F32, F64} (fft_backend.rs:61-68) for the image
// stage of single-plane calls: 0 (Auto) and 64 run FP64, 32 runs FP32.
int cr_ctx_set_image_fft_precision(cr_ctx* ctx, int32_t bits) {
    if (!ctx || (bits != 0 && bits != 32 && bits != 64)) return CR_INVALID;
    ctx->image_fft_bits = bits == 32 ? 32 : 64;
    return CR_OK;
}

int cr_ctx_set_timings(cr_ctx* ctx, int32_t enable) {
    if (!ctx) return CR_INVALID;
    ctx->timings_enabled = enable != 0;
    return CR_OK;
}

int cr_ctx_set_alloc_limit(cr_ctx* ctx, int64_t bytes) {
    if (!ctx || bytes < 0) return CR_INVALID;
    ctx->alloc_limit = bytes;
    return CR_OK;
}

int cr_ctx_set_image_fft_engine(cr_ctx* ctx, int32_t engine) {
    if (!ctx || (engine != 0 && engine != 1)) return CR_INVALID;
    ctx->image_fft_engine = engine;
    return CR_OK;
}

// ---- persistent cube plans --------------------------------------------------

int cr_cube_plan_create(cr_ctx* ctx, cr_gridder* g, const cr_cube_batch* batch,
                        int32_t weighting, float robust, cr_cube_plan** out, cr_sums* sums,
                        char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && g != nullptr && out != nullptr, "null argument");
        *out = nullptr;
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        CubeInput in = cube_input(ctx, batch);
        cr_cube_plan* p = new cr_cube_plan();
        p->ctx = ctx;
        p->g = g;
        try {
            p->rec = cube_plan(ctx, g, in, weighting, robust, nullptr, &p->pool);
            tm.mark();
            p->sums.resize((size_t)in.C);
            cube_read_sums(ctx, p->rec, p->sums.data());
        } catch (...) {
            cr_cube_plan_destroy(p);
            throw;
        }
        int64_t n = 0;
        for (const cr_sums& s : p->sums) n += s.gridded;
        p->rec.n_records = n;
        if (sums) std::copy(p->sums.begin(), p->sums.end(), sums);
        set_timings(ctx, cr_timings{tm.between(0, 1), 0.f, 0.f, 0.f, 0.f});
        *out = p;
    });
}

void cr_cube_plan_destroy(cr_cube_plan* p) {
    if (!p) return;
    cudaSetDevice(p->ctx->device);
    pool_free(p->ctx, p->pool);
    cudaStreamSynchronize(p->ctx->stream);
    delete p;
}

int32_t cr_cube_plan_channels(const cr_cube_plan* p) { return p ? p->rec.C : 0; }

int cr_cube_plan_set_fft_precision(cr_cube_plan* p, int32_t bits) {
    if (!p || (bits != 32 && bits != 64)) return CR_INVALID;
    p->fft_bits = bits;
    return CR_OK;
}

namespace {

void check_cube_plan(cr_ctx* ctx, cr_cube_plan* p) {
    need(ctx != nullptr && p != nullptr && p->ctx == ctx, "plan belongs to another context");
}

// A host plane mask [C] on the device (NULL: every plane), and the planes it
// selects.
const uint8_t* cube_mask(cr_ctx* ctx, const cr_cube_plan* p, const uint8_t* planes,
                         std::vector<int>* chosen) {
    const int C = p->rec.C;
    chosen->clear();
    for (int c = 0; c < C; ++c)
        if (!planes || planes[c]) chosen->push_back(c);
    if (!planes) return nullptr;
    uint8_t* d = (uint8_t*)workspace(ctx, "cube_mask", (size_t)C);
    CR_CUDA_CHECK(cudaMemcpyAsync(d, planes, (size_t)C, cudaMemcpyHostToDevice, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));   // pageable source
    return d;
}

}  // namespace

int cr_cube_plan_grid_dirty(cr_ctx* ctx, cr_cube_plan* p, float* psf_grids, float* dirty_grids,
                            int32_t out_location, char** err) {
    return guarded(err, [&] {
        check_cube_plan(ctx, p);
        need(psf_grids != nullptr && dirty_grids != nullptr, "null argument");
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        const size_t cells = grid_bytes(p->g) / 8, C = (size_t)p->rec.C;
        float* psf = out_ptr<float>(ctx, psf_grids, out_location, C * cells * 4, "cube_psf");
        float2* dirty = out_ptr<float2>(ctx, dirty_grids, out_location, C * cells * 8,
                                        "cube_dirty");
        cube_grid(ctx, p->g, p->rec, psf, dirty);
        tm.mark();
        if (out_location == CR_HOST) {
            copy_out(ctx, psf_grids, psf, C * cells * 4, CR_HOST);
            copy_out(ctx, dirty_grids, dirty, C * cells * 8, CR_HOST);
        }
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        check_device_status(ctx);
        set_timings(ctx, cr_timings{0.f, tm.between(0, 1), 0.f, 0.f, 0.f});
    });
}

int cr_cube_plan_degrid(cr_ctx* ctx, cr_cube_plan* p, const float* model_grids,
                        int32_t grid_location, float* pred, int32_t out_location, char** err) {
    return guarded(err, [&] {
        check_cube_plan(ctx, p);
        need(model_grids != nullptr && pred != nullptr, "null argument");
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        const size_t cells = grid_bytes(p->g) / 8, C = (size_t)p->rec.C;
        const float2* mg = (const float2*)device_input(ctx, model_grids, C * cells * 8,
                                                       grid_location, "cube_model");
        float2* pr = out_ptr<float2>(ctx, pred, out_location, C * (size_t)p->rec.R * 8 + 8,
                                     "cube_pred");
        cube_degrid(ctx, p->g, p->rec, mg, pr);
        tm.mark();
        if (out_location == CR_HOST) copy_out(ctx, pred, pr, C * (size_t)p->rec.R * 8, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        check_device_status(ctx);
        set_timings(ctx, cr_timings{0.f, 0.f, tm.between(0, 1), 0.f, 0.f});
    });
}

int cr_cube_plan_grid_residual(cr_ctx* ctx, cr_cube_plan* p, const float* model_grids,
                               int32_t grid_location, const uint8_t* planes,
                               float* residual_grids, int32_t out_location, char** err) {
    return guarded(err, [&] {
        check_cube_plan(ctx, p);
        need(model_grids != nullptr && residual_grids != nullptr, "null argument");
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        const size_t cells = grid_bytes(p->g) / 8, C = (size_t)p->rec.C;
        std::vector<int> chosen;
        const uint8_t* mask = cube_mask(ctx, p, planes, &chosen);
        const float2* mg = (const float2*)device_input(ctx, model_grids, C * cells * 8,
                                                       grid_location, "cube_model");
        float2* res = out_ptr<float2>(ctx, residual_grids, out_location, C * cells * 8,
                                      "cube_residual");
        cube_grid_residual(ctx, p->g, p->rec, mg, res, mask);
        tm.mark();
        if (out_location == CR_HOST)
            for (int c : chosen)
                copy_out(ctx, (float2*)residual_grids + (size_t)c * cells, res + (size_t)c * cells,
                         cells * 8, CR_HOST);
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        check_device_status(ctx);
        set_timings(ctx, cr_timings{0.f, tm.between(0, 1), 0.f, 0.f, 0.f});
    });
}

int cr_cube_plan_dirty_images(cr_ctx* ctx, cr_cube_plan* p, float* psf_images,
                              float* residual_images, int32_t out_location,
                              cr_psf_state* states, char** err) {
    return guarded(err, [&] {
        check_cube_plan(ctx, p);
        need(psf_images != nullptr && residual_images != nullptr, "null argument");
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        cr_gridder* g = p->g;
        const size_t cells = grid_bytes(g) / 8, C = (size_t)p->rec.C, np = image_pixels(g);
        float* psf = (float*)workspace(ctx, "cpi_psf", C * cells * 4);
        float2* dirty = (float2*)workspace(ctx, "cpi_dirty", C * cells * 8);
        cube_grid(ctx, g, p->rec, psf, dirty);
        tm.mark();
        float* pi = out_ptr<float>(ctx, psf_images, out_location, C * np * 4, "cpi_psf_img");
        float* ri = out_ptr<float>(ctx, residual_images, out_location, C * np * 4, "cpi_res_img");
        unsigned int* peaks = (unsigned int*)workspace(ctx, "cpi_peaks", C * 4);
        const bool single = p->fft_bits == 32;
        CR_CUDA_CHECK(cudaMemsetAsync(peaks, 0, C * 4, ctx->stream));
        std::vector<float> sumwt(C);
        std::vector<int> live;
        std::vector<float> scales;
        for (size_t c = 0; c < C; ++c) {
            sumwt[c] = (float)p->sums[c].normalization_sumwt;
            if (!(p->sums[c].normalization_sumwt > 0.0 && p->sums[c].reported_sumwt > 0.0)) {
                CR_CUDA_CHECK(cudaMemsetAsync(pi + c * np, 0, np * 4, ctx->stream));
                CR_CUDA_CHECK(cudaMemsetAsync(ri + c * np, 0, np * 4, ctx->stream));
                continue;
            }
            live.push_back((int)c);
            scales.push_back(1.0f / sumwt[c]);
        }
        // the normalisation of dirty_grids_to_psf_and_residual_owned, as the
        // single-plane cr_dirty_image, with the transforms batched over planes
        grid_to_image_planes(ctx, g, nullptr, psf, live, scales, pi, single);
        grid_to_image_planes(ctx, g, dirty, nullptr, live, scales, ri, single);
        const std::vector<float> ones(live.size(), 1.0f);
        abs_peak_planes(ctx, pi, (int64_t)np, live, peaks);
        scale_image_planes(ctx, pi, (int64_t)np, live, ones, peaks);
        scale_image_planes(ctx, ri, (int64_t)np, live, ones, peaks);
        tm.mark();
        std::vector<unsigned int> pk(C);
        CR_CUDA_CHECK(cudaMemcpyAsync(pk.data(), peaks, C * 4, cudaMemcpyDeviceToHost,
                                      ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        for (size_t c = 0; c < C; ++c) {
            float peak;
            std::memcpy(&peak, &pk[c], 4);
            const bool ok = p->sums[c].normalization_sumwt > 0.0 &&
                            p->sums[c].reported_sumwt > 0.0 && std::isfinite(peak) &&
                            peak > 0.0f;
            if (!ok) {
                // a plane with no usable samples or a zero PSF: empty images
                CR_CUDA_CHECK(cudaMemsetAsync(pi + c * np, 0, np * 4, ctx->stream));
                CR_CUDA_CHECK(cudaMemsetAsync(ri + c * np, 0, np * 4, ctx->stream));
            }
            if (states)
                states[c] = ok ? cr_psf_state{peak, sumwt[c], (float)p->sums[c].reported_sumwt}
                               : cr_psf_state{0.0f, 0.0f, 0.0f};
        }
        if (out_location == CR_HOST) {
            copy_out(ctx, psf_images, pi, C * np * 4, CR_HOST);
            copy_out(ctx, residual_images, ri, C * np * 4, CR_HOST);
        }
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        check_device_status(ctx);
        set_timings(ctx, cr_timings{0.f, tm.between(0, 1), 0.f, tm.between(1, 2), 0.f});
    });
}

int cr_cube_plan_residual_images(cr_ctx* ctx, cr_cube_plan* p, const float* models,
                                 int32_t model_location, const uint8_t* planes,
                                 const cr_psf_state* states, float* residual_images,
                                 int32_t out_location, char** err) {
    return guarded(err, [&] {
        check_cube_plan(ctx, p);
        need(models != nullptr && states != nullptr && residual_images != nullptr,
             "null argument");
        bind(ctx);
        cr_gridder* g = p->g;
        const size_t cells = grid_bytes(g) / 8, C = (size_t)p->rec.C, np = image_pixels(g);
        std::vector<int> chosen;
        for (size_t c = 0; c < C; ++c)
            if (!planes || planes[c])
                need(states[c].normalization_sumwt > 0.0f && states[c].psf_peak > 0.0f,
                     "invalid PSF state for a selected plane");
        StageTimer tm(ctx);
        tm.mark();
        const uint8_t* mask = cube_mask(ctx, p, planes, &chosen);
        const float* m = (const float*)device_input(ctx, models, C * np * 4, model_location,
                                                    "cube_models");
        float2* mg = (float2*)workspace(ctx, "cpr_model_grids", C * cells * 8);
        const bool single = p->fft_bits == 32;
        image_to_grid_planes(ctx, g, m, chosen, mg, single);
        tm.mark();
        float2* res = (float2*)workspace(ctx, "cpr_residual_grids", C * cells * 8);
        cube_grid_residual(ctx, g, p->rec, mg, res, mask);
        tm.mark();
        float* img = out_ptr<float>(ctx, residual_images, out_location, C * np * 4, "cpr_image");
        std::vector<float> scales;
        for (int c : chosen) scales.push_back(1.0f / states[c].normalization_sumwt);
        grid_to_image_planes(ctx, g, res, nullptr, chosen, scales, img, single);
        std::vector<float> inv_peaks;
        for (int c : chosen) inv_peaks.push_back(1.0f / states[c].psf_peak);
        scale_image_planes(ctx, img, (int64_t)np, chosen, inv_peaks, nullptr);
        for (int c : chosen) {
            if (out_location == CR_HOST)
                copy_out(ctx, residual_images + (size_t)c * np, img + (size_t)c * np, np * 4,
                         CR_HOST);
        }
        tm.mark();
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        check_device_status(ctx);
        set_timings(ctx, cr_timings{0.f, tm.between(1, 2), 0.f,
                                  tm.between(0, 1) + tm.between(2, 3), 0.f});
    });
}

int cr_hogbom_planes(cr_ctx* ctx, float* model, float* residual, const float* psf,
                     const uint8_t* mask, int32_t nplanes, int32_t nx, int32_t ny,
                     const int32_t* planes, int32_t n, float gain, float threshold,
                     float cycle_threshold, float nsigma_threshold,
                     const float* nsigma_thresholds, int64_t cycle_niter, int32_t inclusive,
                     int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
                     int64_t* actual, int64_t* reported, int32_t* stop_reason, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && model != nullptr && residual != nullptr && psf != nullptr,
             "null argument");
        need(nplanes >= 0, "nplanes is negative");
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        hogbom_planes(ctx, model, residual, psf, mask, nx, ny, nplanes, planes, n, gain,
                      threshold, cycle_threshold, nsigma_threshold, nsigma_thresholds,
                      cycle_niter, inclusive, comp_x, comp_y, comp_peak, comp_flux, actual,
                      reported, stop_reason);
        tm.mark();
        set_timings(ctx, cr_timings{0.f, 0.f, 0.f, 0.f, tm.between(0, 1)});
    });
}

int cr_clark(cr_ctx* ctx, float* model, float* residual, const float* psf, const uint8_t* mask,
             int32_t nx, int32_t ny, int32_t location, int32_t ncent, float gain,
             float threshold, float cycle_threshold, float nsigma_threshold, int64_t cycle_niter,
             int32_t* comp_x, int32_t* comp_y, float* comp_peak, float* comp_flux,
             int64_t* actual, int32_t* stop_reason, float* max_exterior_abs, char** err) {
    return guarded(err, [&] {
        need(ctx && model && residual && psf, "null argument");
        need(nx > 0 && ny > 0, "image shape must be positive");
        need(location == CR_HOST || location == CR_DEVICE, "bad location");
        need(!comp_x == !comp_y && !comp_x == !comp_peak && !comp_x == !comp_flux,
             "component arrays must be all given or all null");
        bind(ctx);
        size_t nb = (size_t)nx * ny * 4;
        float* m = location == CR_DEVICE ? model : (float*)workspace(ctx, "clk_model", nb);
        float* r = location == CR_DEVICE ? residual : (float*)workspace(ctx, "clk_residual", nb);
        if (location == CR_HOST) {
            CR_CUDA_CHECK(cudaMemcpyAsync(m, model, nb, cudaMemcpyHostToDevice, ctx->stream));
            CR_CUDA_CHECK(cudaMemcpyAsync(r, residual, nb, cudaMemcpyHostToDevice, ctx->stream));
        }
        const float* p = (const float*)device_input(ctx, psf, nb, location, "clk_psf");
        const uint8_t* mk = (const uint8_t*)device_input(ctx, mask, (size_t)nx * ny, location,
                                                         "clk_mask");
        StageTimer tm(ctx);
        tm.mark();
        cr::clark_minor_cycle(ctx, m, r, p, mk, nx, ny, ncent, gain, threshold, cycle_threshold,
                              nsigma_threshold, cycle_niter, comp_x, comp_y, comp_peak,
                              comp_flux, actual, stop_reason, max_exterior_abs);
        tm.mark();
        if (location == CR_HOST) {
            CR_CUDA_CHECK(cudaMemcpyAsync(model, m, nb, cudaMemcpyDeviceToHost, ctx->stream));
            CR_CUDA_CHECK(cudaMemcpyAsync(residual, r, nb, cudaMemcpyDeviceToHost, ctx->stream));
        }
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        set_timings(ctx, cr_timings{0.f, 0.f, 0.f, 0.f, tm.between(0, 1)});
    });
}

// ---- streaming dirty accumulation -----------------------------------------------

int cr_accumulator_create(cr_ctx* ctx, cr_gridder* g, cr_accumulator** out, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && g != nullptr && out != nullptr, "null argument");
        *out = nullptr;
        bind(ctx);
        cr_accumulator* a = new cr_accumulator();
        a->ctx = ctx;
        a->g = g;
        try {
            const size_t gb = grid_bytes(g);
            a->psf = (float2*)pool_alloc(ctx, a->pool, "acc_psf", gb);
            a->dirty = (float2*)pool_alloc(ctx, a->pool, "acc_dirty", gb);
            CR_CUDA_CHECK(cudaMemsetAsync(a->psf, 0, gb, ctx->stream));
            CR_CUDA_CHECK(cudaMemsetAsync(a->dirty, 0, gb, ctx->stream));
            CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        } catch (...) {
            cr_accumulator_destroy(a);
            throw;
        }
        *out = a;
    });
}

void cr_accumulator_destroy(cr_accumulator* a) {
    if (!a) return;
    cudaSetDevice(a->ctx->device);
    pool_free(a->ctx, a->pool);
    cudaStreamSynchronize(a->ctx->stream);
    delete a;
}

int cr_accumulator_add(cr_ctx* ctx, cr_accumulator* a, const cr_vis_batch* batch,
                       cr_sums* batch_sums, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && a != nullptr && a->ctx == ctx,
             "accumulator belongs to another context");
        bind(ctx);
        StageTimer tm(ctx);
        tm.mark();
        StagedBatch b(ctx, batch, false);
        Records r = plan(ctx, a->g, nullptr, b);
        tm.mark();
        grid_records(ctx, a->g, nullptr, r, a->psf, a->dirty, 0);
        tm.mark();
        cr_sums s{};
        read_sums(ctx, r, &s);
        a->sums.normalization_sumwt += s.normalization_sumwt;
        a->sums.reported_sumwt += s.reported_sumwt;
        a->sums.gridded += s.gridded;
        a->sums.skipped += s.skipped;
        a->sums.unique_records += s.unique_records;
        a->sums.taps += s.taps;
        a->batches++;
        if (batch_sums) *batch_sums = s;
        set_timings(ctx, cr_timings{tm.between(0, 1), tm.between(1, 2), 0.f, 0.f, 0.f});
    });
}

int cr_accumulator_finish(cr_ctx* ctx, cr_accumulator* a, float* psf, float* residual,
                          int32_t out_location, cr_psf_state* state, cr_sums* total, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && a != nullptr && a->ctx == ctx,
             "accumulator belongs to another context");
        bind(ctx);
        if (total) *total = a->sums;
        StageTimer tm(ctx);
        tm.mark();
        dirty_products(ctx, a->g, nullptr, a->psf, a->dirty, a->sums, psf, residual,
                       out_location, state);
        tm.mark();
        set_timings(ctx, cr_timings{0.f, 0.f, 0.f, tm.between(0, 1), 0.f});
    });
}

}  // extern "C"
