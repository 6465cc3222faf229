// cr_feed.cu -- the row-block read-ahead feed (cr_row_feed_*).
//
// The reference streams MeasurementSet row blocks through a bounded
// producer/consumer pipeline (stream_imaging_source_read_ahead_blocks,
// casars-imager/src/lib.rs:36608-36760): a reader thread produces row blocks
// while the imager consumes the previous ones, with at most
// max_live_row_blocks blocks alive.  Here the producer is the caller's reader
// and the consumer is the device:
//
//   * every slot is a set of page-locked host arrays (the reader writes the
//     columns straight into them, no extra host copy) and their device
//     twins;
//   * submit uploads the slot on the feed's own copy stream, after the
//     device has finished with the slot's previous block (an event), so the
//     upload of block k+1 runs while block k is prepared and gridded;
//   * one worker thread takes the blocks in submission order and runs the
//     row-run preparation and the streaming accumulator on the context's
//     stream after the block's upload event; a block's slot returns to the
//     producer once the worker has consumed it.
//
// Summary fields and their meaning follow ImagingSourceReadAheadSummary
// (lib.rs:36324-36335) and the overlap tracker (lib.rs:36337-36366).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "cr_internal.cuh"

using namespace cr;

namespace {

using Clock = std::chrono::steady_clock;

double seconds(Clock::duration d) { return std::chrono::duration<double>(d).count(); }

enum SlotState { kFree = 0, kFilling = 1, kQueued = 2 };

struct Slot {
    cr_row_block host{};          // page-locked arrays
    double* d_uvw = nullptr;
    float* d_data = nullptr;
    uint8_t* d_flag = nullptr;
    float* d_weight = nullptr;
    float* d_ws = nullptr;
    uint8_t* d_gridable = nullptr;
    cudaEvent_t uploaded = nullptr;   // copy stream: the block is on the device
    cudaEvent_t consumed = nullptr;   // context stream: the device is done with it
    SlotState state = kFree;
    int64_t rows = 0;
};

}  // namespace

struct cr_row_feed {
    cr_ctx* ctx = nullptr;
    cr_gridder* g = nullptr;
    cr_accumulator* acc = nullptr;
    cr_row_feed_config cfg{};
    std::vector<double> lambda_scale;
    std::vector<Slot> slots;
    int next = 0;                       // round-robin start of the slot search
    cudaStream_t copy = nullptr;
    // prepared samples of the block in work (rows x channels entries)
    double *u = nullptr, *v = nullptr, *w = nullptr, *du = nullptr, *dv = nullptr;
    float *weight = nullptr, *sumwt_factor = nullptr;
    uint8_t* gridable = nullptr;
    float* vis = nullptr;
    // pipeline state (under m)
    std::thread worker;
    std::mutex m;
    std::condition_variable cv;
    std::deque<int> queue;
    bool stop = false;
    bool busy = false;
    int live = 0;                       // slots filling or queued
    int filling = 0;
    int error_code = CR_OK;
    std::string error;
    cr_row_feed_summary sum{};
    Clock::time_point last_transition = Clock::now();

    // Overlap bookkeeping: called under m before any change of `filling`
    // or `busy`.
    void transition() {
        const Clock::time_point now = Clock::now();
        if (filling > 0 && busy) sum.producer_consumer_overlap_s += seconds(now - last_transition);
        last_transition = now;
    }
    void check_error() {
        if (error_code != CR_OK) fail(error_code, "row feed: an earlier block failed: " + error);
    }
    void run();
    void release();
};

void cr_row_feed::run() {
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        std::lock_guard<std::mutex> lk(m);
        error_code = CR_CUDA;
        error = "cudaSetDevice failed in the feed's worker";
        return;
    }
    for (;;) {
        int k = -1;
        {
            std::unique_lock<std::mutex> lk(m);
            const Clock::time_point t0 = Clock::now();
            cv.wait(lk, [&] { return stop || !queue.empty(); });
            if (stop) return;
            sum.consumer_recv_blocked_s += seconds(Clock::now() - t0);
            k = queue.front();
            queue.pop_front();
            transition();
            busy = true;
        }
        const Clock::time_point t1 = Clock::now();
        Slot& s = slots[k];
        int rc = CR_OK;
        char* msg = nullptr;
        int64_t kept = 0;
        bool failed_before;
        {
            std::lock_guard<std::mutex> lk(m);
            failed_before = error_code != CR_OK;
        }
        if (!failed_before && s.rows > 0) {
            // the block is consumed on the context's stream after its upload
            if (cudaStreamWaitEvent(ctx->stream, s.uploaded, 0) != cudaSuccess) {
                rc = CR_CUDA;
            } else {
                cr_row_runs runs{};
                runs.rows = s.rows;
                runs.channels = cfg.channels;
                runs.correlations = cfg.correlations;
                runs.uvw_m = s.d_uvw;
                runs.lambda_scale = lambda_scale.data();
                runs.data = s.d_data;
                runs.flag = s.d_flag;
                runs.weight = s.d_weight;
                runs.weight_spectrum = s.d_ws;
                runs.gridable = s.d_gridable;
                runs.location = CR_DEVICE;
                rc = cr_row_runs_prepare(ctx, &runs, &cfg.polarization, u, v, w, weight,
                                         sumwt_factor, gridable, vis, du, dv, CR_DEVICE, &kept,
                                         &msg);
                if (rc == CR_OK && kept > 0) {
                    cr_vis_batch b{};
                    b.n = kept;
                    b.u = u;
                    b.v = v;
                    b.w = w;
                    b.weight = weight;
                    b.sumwt_factor = sumwt_factor;
                    b.gridable = gridable;
                    b.vis = vis;
                    b.location = CR_DEVICE;
                    rc = cr_accumulator_add(ctx, acc, &b, nullptr, &msg);
                }
            }
            if (rc == CR_OK && cudaEventRecord(s.consumed, ctx->stream) != cudaSuccess)
                rc = CR_CUDA;
        }
        {
            std::lock_guard<std::mutex> lk(m);
            if (rc != CR_OK && error_code == CR_OK) {
                error_code = rc;
                error = msg ? msg : "CUDA runtime failure in the feed's worker";
            }
            sum.consumer_elapsed_s += seconds(Clock::now() - t1);
            if (s.rows > 0) sum.row_blocks += 1;
            sum.streamed_samples += kept;
            transition();
            busy = false;
            s.state = kFree;
            s.rows = 0;
            --live;
        }
        std::free(msg);
        cv.notify_all();
    }
}

void cr_row_feed::release() {
    if (worker.joinable()) {
        {
            std::lock_guard<std::mutex> lk(m);
            stop = true;
        }
        cv.notify_all();
        worker.join();
    }
    if (ctx) cudaSetDevice(ctx->device);
    if (copy) cudaStreamSynchronize(copy);
    if (ctx) cudaStreamSynchronize(ctx->stream);
    for (Slot& s : slots) {
        cudaFreeHost(s.host.uvw_m);
        cudaFreeHost(s.host.data);
        cudaFreeHost(s.host.flag);
        cudaFreeHost(s.host.weight);
        cudaFreeHost(s.host.weight_spectrum);
        cudaFreeHost(s.host.gridable);
        cudaFree(s.d_uvw);
        cudaFree(s.d_data);
        cudaFree(s.d_flag);
        cudaFree(s.d_weight);
        cudaFree(s.d_ws);
        cudaFree(s.d_gridable);
        if (s.uploaded) cudaEventDestroy(s.uploaded);
        if (s.consumed) cudaEventDestroy(s.consumed);
    }
    slots.clear();
    for (void* p : {(void*)u, (void*)v, (void*)w, (void*)du, (void*)dv, (void*)weight,
                    (void*)sumwt_factor, (void*)gridable, (void*)vis})
        cudaFree(p);
    if (copy) cudaStreamDestroy(copy);
    copy = nullptr;
    if (acc) cr_accumulator_destroy(acc);
    acc = nullptr;
}

extern "C" {

int cr_row_feed_create(cr_ctx* ctx, cr_gridder* g, const cr_row_feed_config* config,
                       cr_row_feed** out, char** err) {
    return guarded(err, [&] {
        need(ctx != nullptr && g != nullptr && config != nullptr && out != nullptr,
             "null argument");
        need(g->ctx == ctx, "gridder belongs to another context");
        const cr_row_feed_config& c = *config;
        need(c.max_live_row_blocks >= 1 && c.max_live_row_blocks <= 64,
             "max_live_row_blocks must lie in [1, 64]");
        need(c.row_block_rows >= 1, "row_block_rows must be >= 1");
        need(c.channels >= 1 && c.correlations >= 1, "channels and correlations must be >= 1");
        need(c.lambda_scale != nullptr, "lambda_scale is required");
        const int64_t samples = c.row_block_rows * (int64_t)c.channels;
        need(samples < (1ll << 31), "row_block_rows x channels must stay below 2^31");
        *out = nullptr;
        CR_CUDA_CHECK(cudaSetDevice(ctx->device));
        cr_row_feed* f = new cr_row_feed();
        f->ctx = ctx;
        f->g = g;
        f->cfg = c;
        f->lambda_scale.assign(c.lambda_scale, c.lambda_scale + c.channels);
        f->cfg.lambda_scale = f->lambda_scale.data();
        try {
            char* msg = nullptr;
            const int rc = cr_accumulator_create(ctx, g, &f->acc, &msg);
            if (rc != CR_OK) {
                const std::string m = msg ? msg : "accumulator";
                std::free(msg);
                fail(rc, m);
            }
            CR_CUDA_CHECK(cudaStreamCreateWithFlags(&f->copy, cudaStreamNonBlocking));
            const size_t R = (size_t)c.row_block_rows, S = (size_t)samples;
            const size_t X = S * (size_t)c.correlations;
            f->slots.resize((size_t)c.max_live_row_blocks);
            for (int k = 0; k < c.max_live_row_blocks; ++k) {
                Slot& s = f->slots[(size_t)k];
                s.host.slot = k;
                s.host.max_rows = c.row_block_rows;
                auto host = [](void** p, size_t bytes) {
                    CR_CUDA_CHECK(cudaHostAlloc(p, bytes, cudaHostAllocDefault));
                };
                host((void**)&s.host.uvw_m, R * 24);
                host((void**)&s.host.data, X * 8);
                host((void**)&s.host.weight, R * (size_t)c.correlations * 4);
                if (c.has_flag) host((void**)&s.host.flag, X);
                if (c.has_weight_spectrum) host((void**)&s.host.weight_spectrum, X * 4);
                if (c.has_gridable) host((void**)&s.host.gridable, R);
                CR_CUDA_CHECK(cudaMalloc((void**)&s.d_uvw, R * 24));
                CR_CUDA_CHECK(cudaMalloc((void**)&s.d_data, X * 8));
                CR_CUDA_CHECK(cudaMalloc((void**)&s.d_weight, R * (size_t)c.correlations * 4));
                if (c.has_flag) CR_CUDA_CHECK(cudaMalloc((void**)&s.d_flag, X));
                if (c.has_weight_spectrum) CR_CUDA_CHECK(cudaMalloc((void**)&s.d_ws, X * 4));
                if (c.has_gridable) CR_CUDA_CHECK(cudaMalloc((void**)&s.d_gridable, R));
                CR_CUDA_CHECK(cudaEventCreateWithFlags(&s.uploaded, cudaEventDisableTiming));
                CR_CUDA_CHECK(cudaEventCreateWithFlags(&s.consumed, cudaEventDisableTiming));
            }
            // the prepared samples of one block (cr_row_runs_prepare sizes)
            CR_CUDA_CHECK(cudaMalloc((void**)&f->u, S * 8 + 8));
            CR_CUDA_CHECK(cudaMalloc((void**)&f->v, S * 8 + 8));
            CR_CUDA_CHECK(cudaMalloc((void**)&f->w, S * 8 + 8));
            CR_CUDA_CHECK(cudaMalloc((void**)&f->du, S * 8 + 8));
            CR_CUDA_CHECK(cudaMalloc((void**)&f->dv, S * 8 + 8));
            CR_CUDA_CHECK(cudaMalloc((void**)&f->weight, S * 4 + 4));
            CR_CUDA_CHECK(cudaMalloc((void**)&f->sumwt_factor, S * 4 + 4));
            CR_CUDA_CHECK(cudaMalloc((void**)&f->gridable, S + 1));
            CR_CUDA_CHECK(cudaMalloc((void**)&f->vis, S * 8 + 8));
            f->worker = std::thread([f] { f->run(); });
        } catch (...) {
            f->release();
            delete f;
            throw;
        }
        *out = f;
    });
}

void cr_row_feed_destroy(cr_row_feed* feed) {
    if (!feed) return;
    feed->release();
    delete feed;
}

int cr_row_feed_acquire(cr_row_feed* f, cr_row_block* block, char** err) {
    return guarded(err, [&] {
        need(f != nullptr && block != nullptr, "null argument");
        std::unique_lock<std::mutex> lk(f->m);
        f->check_error();
        const Clock::time_point t0 = Clock::now();
        const int n = (int)f->slots.size();
        int k = -1;
        f->cv.wait(lk, [&] {
            if (f->error_code != CR_OK) return true;
            for (int j = 0; j < n; ++j)
                if (f->slots[(size_t)((f->next + j) % n)].state == kFree) {
                    k = (f->next + j) % n;
                    return true;
                }
            return false;
        });
        f->sum.producer_send_blocked_s += seconds(Clock::now() - t0);
        f->check_error();
        f->next = (k + 1) % n;
        f->transition();
        f->slots[(size_t)k].state = kFilling;
        ++f->filling;
        ++f->live;
        f->sum.live_row_block_high_water = std::max(f->sum.live_row_block_high_water, f->live);
        *block = f->slots[(size_t)k].host;
    });
}

int cr_row_feed_submit(cr_row_feed* f, int32_t slot, int64_t rows, char** err) {
    return guarded(err, [&] {
        need(f != nullptr, "null argument");
        {
            std::lock_guard<std::mutex> lk(f->m);
            f->check_error();
            need(slot >= 0 && slot < (int32_t)f->slots.size() &&
                     f->slots[(size_t)slot].state == kFilling,
                 "submit needs a slot taken by cr_row_feed_acquire");
            need(rows >= 0 && rows <= f->cfg.row_block_rows,
                 "rows must lie in [0, row_block_rows]");
        }
        Slot& s = f->slots[(size_t)slot];
        const cr_row_feed_config& c = f->cfg;
        const size_t R = (size_t)rows, X = R * (size_t)c.channels * (size_t)c.correlations;
        size_t bytes = 0;
        if (rows > 0) {
            CR_CUDA_CHECK(cudaSetDevice(f->ctx->device));
            // the slot's device arrays are free once its previous block is consumed
            CR_CUDA_CHECK(cudaStreamWaitEvent(f->copy, s.consumed, 0));
            auto up = [&](void* dst, const void* src, size_t n) {
                if (!src || n == 0) return;
                CR_CUDA_CHECK(cudaMemcpyAsync(dst, src, n, cudaMemcpyHostToDevice, f->copy));
                bytes += n;
            };
            up(s.d_uvw, s.host.uvw_m, R * 24);
            up(s.d_data, s.host.data, X * 8);
            up(s.d_weight, s.host.weight, R * (size_t)c.correlations * 4);
            up(s.d_flag, s.host.flag, X);
            up(s.d_ws, s.host.weight_spectrum, X * 4);
            up(s.d_gridable, s.host.gridable, R);
            CR_CUDA_CHECK(cudaEventRecord(s.uploaded, f->copy));
        }
        {
            std::lock_guard<std::mutex> lk(f->m);
            s.rows = rows;
            f->transition();
            s.state = kQueued;
            --f->filling;
            f->sum.source_bytes += (int64_t)bytes;
            f->queue.push_back(slot);
        }
        f->cv.notify_all();
    });
}

int cr_row_feed_finish(cr_row_feed* f, float* psf, float* residual, int32_t out_location,
                       cr_psf_state* state, cr_sums* total, cr_row_feed_summary* summary,
                       char** err) {
    return guarded(err, [&] {
        need(f != nullptr, "null argument");
        {
            std::unique_lock<std::mutex> lk(f->m);
            f->cv.wait(lk, [&] { return f->queue.empty() && !f->busy; });
            if (summary) *summary = f->sum;
            f->check_error();
        }
        char* msg = nullptr;
        const int rc =
            cr_accumulator_finish(f->ctx, f->acc, psf, residual, out_location, state, total, &msg);
        if (rc != CR_OK) {
            const std::string m = msg ? msg : "accumulator finish";
            std::free(msg);
            fail(rc, m);
        }
    });
}

}  // extern "C"
