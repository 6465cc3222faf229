// cr_clark.cu -- the Clark minor cycle.
//
// Restates run_clark_minor_cycle_cpu (lib.rs:62129-62355) with the PSF patch
// of build_clark_psf_patch (lib.rs:64422-64456), the active set of
// collect_clark_active_pixels (lib.rs:64467-64487), the peak of
// peak_clark_active_pixel (lib.rs:64489-64501: the first strictly largest
// |value| in row-major order), the patch subtraction of
// subtract_clark_component_from_active (lib.rs:64503-64539) and the residual
// update by fft_convolve_real (lib.rs:64415-64420).
//
// Per subcycle the control (flux limit, factor, iteration caps, at most
// CASA_CLARK_MAX_MAJOR_CYCLES = 10 subcycles) runs on the host; the active
// pixels are gathered on the device (mark, scan, scatter, with a pixel ->
// slot map), and one block runs the subcycle's component loop -- block
// argmax over the active values, the stop rules, the model update and the
// patch subtraction over active pixels -- without leaving the device.  The
// subcycle's components are then convolved with the PSF through cuFFT (FP64,
// circular, centred as the reference's centred transforms) and subtracted
// from the residual in float32.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "cr_internal.cuh"

namespace cr {

namespace {

constexpr int kClarkThreads = 1024;

__device__ __forceinline__ bool c_threshold_reached(float peak, float thr) {
    if (thr <= 0.0f) return peak <= thr;
    float tol = fmaxf(__fmul_rn(0.01f, thr), 2.0e-8f);
    return peak <= thr || fabsf(__fsub_rn(peak, thr)) <= tol;
}

// minor_cycle_stop_reason (lib.rs:74653-74676)
__device__ int c_stop_reason(float peak_abs, float thr, float cyc, float nsig) {
    bool floor_active = thr > 0.0f && __fmul_rn(0.01f, thr) < 2.0e-8f && cyc <= thr;
    if (peak_abs < thr || (floor_active && c_threshold_reached(peak_abs, thr)))
        return CR_STOP_GLOBAL_THRESHOLD;
    if (cyc >= nsig) return peak_abs < cyc ? CR_STOP_CYCLE_THRESHOLD : 0;
    if (nsig > thr) return peak_abs < nsig ? CR_STOP_NSIGMA_THRESHOLD : 0;
    return 0;
}

// |value| bits of a non-negative float order like the value
__global__ void exterior_max_kernel(const float* psf, int nx, int ny, int x0, int x1, int y0,
                                    int y1, unsigned int* out) {
    float m = 0.0f;
    const int64_t n = (int64_t)nx * ny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(t / ny), y = (int)(t - (int64_t)x * ny);
        if (x < x0 || x >= x1 || y < y0 || y >= y1) {
            const float a = fabsf(psf[t]);
            if (a > m) m = a;   // NaN never raises the maximum, as f32::max
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

__global__ void abs_max_masked_kernel(const float* img, const uint8_t* mask, int64_t n,
                                      unsigned int* out) {
    float m = 0.0f;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        if (mask && !mask[t]) continue;
        const float a = fabsf(img[t]);
        if (a > m) m = a;
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// keep = |r| >= limit (and unmasked); the comparison is the reference's
// `!(|value| < limit)`, so a NaN residual is kept
__global__ void active_mark_kernel(const float* r, const uint8_t* mask, int64_t n, float limit,
                                   uint32_t* keep) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x)
        keep[t] = (!(fabsf(r[t]) < limit) && (!mask || mask[t])) ? 1u : 0u;
}

__global__ void active_fill_kernel(const float* r, int64_t n, const uint32_t* keep,
                                   const uint32_t* slot, int* map, int* pix, float* val) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        if (keep[t]) {
            const uint32_t k = slot[t];
            map[t] = (int)k;
            pix[k] = (int)t;
            val[k] = r[t];
        } else {
            map[t] = -1;
        }
    }
}

struct SubArgs {
    int n_active;
    const int* pix;       // [n_active] x ny + y
    float* val;           // [n_active] working values
    const int* map;       // [nx ny] pixel -> slot or -1
    int nx, ny;
    const float* patch;   // [pnx][pny]
    int pnx, pny, rx, ry;
    float* model;
    float* delta;
    float gain, threshold, cycle_threshold, nsigma;
    float flux_limit, selection_limit;
    int limit;            // components this subcycle may add
    int updates0;         // components of the minor cycle so far
    int cap;              // component list capacity
    int* comp_x;
    int* comp_y;
    float* comp_peak;
    float* comp_flux;
    int* out;             // [0] components added, [1] stop reason
    float* out_peak;      // approximate peak after the subcycle
};

// block argmax: the first index of the largest |val| (strictly greater wins)
__device__ void active_peak(const SubArgs& a, int* best_i, float* best_v) {
    __shared__ float s_a[kClarkThreads / 32];
    __shared__ int s_i[kClarkThreads / 32];
    float ba = -1.0f;
    int bi = 0x7fffffff;
    for (int k = threadIdx.x; k < a.n_active; k += blockDim.x) {
        const float v = fabsf(a.val[k]);
        if (v > ba) {   // k increases within a thread: the first maximum is kept
            ba = v;
            bi = k;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const float a2 = __shfl_xor_sync(0xffffffffu, ba, o);
        const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
        if (a2 > ba || (a2 == ba && i2 < bi)) {
            ba = a2;
            bi = i2;
        }
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        s_a[warp] = ba;
        s_i[warp] = bi;
    }
    __syncthreads();
    if (warp == 0) {
        ba = lane < (int)(blockDim.x >> 5) ? s_a[lane] : -1.0f;
        bi = lane < (int)(blockDim.x >> 5) ? s_i[lane] : 0x7fffffff;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const float a2 = __shfl_xor_sync(0xffffffffu, ba, o);
            const int i2 = __shfl_xor_sync(0xffffffffu, bi, o);
            if (a2 > ba || (a2 == ba && i2 < bi)) {
                ba = a2;
                bi = i2;
            }
        }
        if (lane == 0) {
            s_i[0] = ba < 0.0f ? -1 : bi;
        }
    }
    __syncthreads();
    *best_i = s_i[0];
    *best_v = *best_i >= 0 ? a.val[*best_i] : 0.0f;
    __syncthreads();
}

__global__ void __launch_bounds__(kClarkThreads) clark_subcycle_kernel(SubArgs a) {
    __shared__ int s_stop;
    int bi;
    float bv;
    active_peak(a, &bi, &bv);
    const float init_peak = bi >= 0 ? fabsf(bv) : 0.0f;
    const float fac = (a.flux_limit > 0.0f && init_peak > 0.0f)
                          ? __fdiv_rn(init_peak, a.flux_limit) : 1.0f;
    float fmn = 0.0f;
    float iter_limit = a.selection_limit;
    int added = 0;
    int stop = 0;
    while (added < a.limit) {
        if (added > 0) active_peak(a, &bi, &bv);
        if (bi < 0) break;
        const float pabs = fabsf(bv);
        if (threadIdx.x == 0) s_stop = c_stop_reason(pabs, a.threshold, iter_limit, a.nsigma);
        __syncthreads();
        if (s_stop) {
            stop = s_stop;
            break;
        }
        const float comp = __fmul_rn(a.gain, bv);
        const int p = a.pix[bi];
        const int px = p / a.ny, py = p - px * a.ny;
        const int k = a.updates0 + added;
        if (threadIdx.x == 0) {
            a.model[p] = __fadd_rn(a.model[p], comp);
            a.delta[p] = __fadd_rn(a.delta[p], comp);
            if (a.comp_x && k < a.cap) {
                a.comp_x[k] = px;
                a.comp_y[k] = py;
                a.comp_peak[k] = bv;
                a.comp_flux[k] = comp;
            }
        }
        // subtract component x patch from the active pixels under the patch
        const int np = a.pnx * a.pny;
        for (int q = threadIdx.x; q < np; q += blockDim.x) {
            const int qx = q / a.pny, qy = q - qx * a.pny;
            const int x = px + qx - a.rx, y = py + qy - a.ry;
            if (x < 0 || x >= a.nx || y < 0 || y >= a.ny) continue;
            const int s = a.map[x * a.ny + y];
            if (s >= 0) a.val[s] = __fsub_rn(a.val[s], __fmul_rn(comp, a.patch[q]));
        }
        __syncthreads();
        ++added;
        fmn = __fadd_rn(fmn, __fdiv_rn(fac, (float)(a.updates0 + added)));
        iter_limit = fmaxf(__fmul_rn(a.flux_limit, fmn), a.cycle_threshold);
    }
    active_peak(a, &bi, &bv);
    if (threadIdx.x == 0) {
        a.out[0] = added;
        a.out[1] = stop;
        *a.out_peak = bi >= 0 ? fabsf(bv) : 0.0f;
    }
}

// residual -= float32(circular convolution of delta with the PSF centred at
// (nx/2, ny/2)): the centred transforms of fft_convolve_real (ifftshift, DFT,
// fftshift) reduce to conv[x] = sum_p delta[p] psf[(x - p + floor(n/2)) mod n]
__global__ void clark_pack_kernel(const float* src, int nx, int ny, int shift, double2* out) {
    const int64_t n = (int64_t)nx * ny;
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const int x = (int)(t / ny), y = (int)(t - (int64_t)x * ny);
        // out[k] = src[(k + n/2) mod n] when shift, else src[k]
        const int sx = shift ? (x + nx / 2) % nx : x, sy = shift ? (y + ny / 2) % ny : y;
        out[t] = make_double2((double)src[(int64_t)sx * ny + sy], 0.0);
    }
}

__global__ void clark_mul_kernel(double2* a, const double2* b, int64_t n, double scale) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x) {
        const double2 x = a[t], y = b[t];
        a[t] = make_double2((x.x * y.x - x.y * y.y) * scale, (x.x * y.y + x.y * y.x) * scale);
    }
}

__global__ void clark_subtract_kernel(float* residual, const double2* conv, int64_t n) {
    for (int64_t t = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; t < n;
         t += (int64_t)gridDim.x * blockDim.x)
        residual[t] = __fsub_rn(residual[t], (float)conv[t].x);
}

float read_float_bits(cr_ctx* ctx, const unsigned int* d) {
    unsigned int h = 0;
    CR_CUDA_CHECK(cudaMemcpyAsync(&h, d, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    float f;
    std::memcpy(&f, &h, 4);
    return f;
}

}  // namespace

void clark_minor_cycle(cr_ctx* ctx, float* model, float* residual, const float* psf,
                       const uint8_t* mask, int32_t nx, int32_t ny, int32_t ncent, float gain,
                       float threshold, float cycle_threshold, float nsigma_threshold,
                       int64_t cycle_niter, int32_t* comp_x, int32_t* comp_y, float* comp_peak,
                       float* comp_flux, int64_t* actual, int32_t* stop_out,
                       float* max_exterior_out) {
    if (nx <= 0 || ny <= 0) fail(CR_INVALID, "image shape must be positive");
    if ((int64_t)nx * ny >= (1ll << 31)) fail(CR_INVALID, "image larger than 2^31 pixels");
    if (cycle_niter < 0 || cycle_niter >= (1ll << 31)) fail(CR_INVALID, "invalid cycle_niter");
    if (ncent < 1) fail(CR_INVALID, "ncent must be positive");
    const int64_t n = (int64_t)nx * ny;
    // build_clark_psf_patch: a (3 ncent + 1)^2 window about the centre
    const int psize = 3 * ncent + 1;
    const int rx = psize / 2, ry = psize / 2;
    const int x0 = std::max(0, nx / 2 - rx), y0 = std::max(0, ny / 2 - ry);
    const int x1 = std::min(x0 + psize, nx), y1 = std::min(y0 + psize, ny);
    const int pnx = x1 - x0, pny = y1 - y0;
    float* patch = (float*)workspace(ctx, "clark_patch", (size_t)pnx * pny * 4);
    CR_CUDA_CHECK(cudaMemcpy2DAsync(patch, (size_t)pny * 4, psf + (int64_t)x0 * ny + y0,
                                    (size_t)ny * 4, (size_t)pny * 4, (size_t)pnx,
                                    cudaMemcpyDeviceToDevice, ctx->stream));
    unsigned int* scal = (unsigned int*)workspace(ctx, "clark_scal", 64);
    CR_CUDA_CHECK(cudaMemsetAsync(scal, 0, 64, ctx->stream));
    exterior_max_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(psf, nx, ny, x0, x1, y0,
                                                                       y1, scal);
    note_launch(ctx, "exterior_max_kernel");
    abs_max_masked_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(residual, mask, n,
                                                                         scal + 1);
    note_launch(ctx, "abs_max_masked_kernel");
    const float mea = read_float_bits(ctx, scal);
    float approx = read_float_bits(ctx, scal + 1);
    if (max_exterior_out) *max_exterior_out = mea;

    // FFT of the shifted PSF, once per call; the subcycle's delta model
    double2* fpsf = (double2*)workspace(ctx, "clark_fpsf", (size_t)n * 16);
    double2* work = (double2*)workspace(ctx, "clark_work", (size_t)n * 16);
    float* delta = (float*)workspace(ctx, "clark_delta", (size_t)n * 4);
    cufftHandle fft = fft_plan(ctx, nx, ny);
    clark_pack_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(psf, nx, ny, 1, fpsf);
    note_launch(ctx, "clark_pack_kernel");
    check_cufft(cufftExecZ2Z(fft, (cufftDoubleComplex*)fpsf, (cufftDoubleComplex*)fpsf,
                             CUFFT_FORWARD), "cufftExecZ2Z");
    uint32_t* keep = (uint32_t*)workspace(ctx, "clark_keep", (size_t)n * 4);
    uint32_t* slot = (uint32_t*)workspace(ctx, "clark_slot", (size_t)n * 4);
    int* map = (int*)workspace(ctx, "clark_map", (size_t)n * 4);
    int* pix = (int*)workspace(ctx, "clark_pix", (size_t)n * 4);
    float* val = (float*)workspace(ctx, "clark_val", (size_t)n * 4);
    unsigned long long* total = (unsigned long long*)workspace(ctx, "clark_total", 8);
    int* dout = (int*)workspace(ctx, "clark_out", 16);
    float* dpeak = (float*)(dout + 2);
    const int cap = (int)std::max<int64_t>(cycle_niter, 1);
    int* cx = (int*)workspace(ctx, "clark_comps", (size_t)cap * 16);
    int* cy = cx + cap;
    float* cp = (float*)(cy + cap);
    float* cf = cp + cap;

    int64_t updates = 0;
    bool updated = false;
    int stop = 0;
    float prev = approx;
    float factor = 1.5f / 4.5f;
    bool warn = false;
    int64_t max_iter = cycle_niter;
    if (mea > 0.5f)
        max_iter = std::min<int64_t>(max_iter, 5);
    else if (mea > 0.35f)
        max_iter = std::min<int64_t>(max_iter, 50);
    int subcycle = 0;
    constexpr int kMaxSubcycles = 10;   // CASA_CLARK_MAX_MAJOR_CYCLES
    auto host_stop = [](float peak, float thr, float cyc, float nsig) {
        auto reached = [](float p, float t) {
            if (t <= 0.0f) return p <= t;
            volatile float tol = std::max(0.01f * t, 2.0e-8f);
            volatile float diff = p - t;
            return p <= t || std::fabs(diff) <= tol;
        };
        volatile float small = 0.01f * thr;
        bool floor_active = thr > 0.0f && small < 2.0e-8f && cyc <= thr;
        if (peak < thr || (floor_active && reached(peak, thr))) return CR_STOP_GLOBAL_THRESHOLD;
        if (cyc >= nsig) return peak < cyc ? CR_STOP_CYCLE_THRESHOLD : 0;
        if (nsig > thr) return peak < nsig ? CR_STOP_NSIGMA_THRESHOLD : 0;
        return 0;
    };
    while (updates < cycle_niter && subcycle < kMaxSubcycles) {
        const int r = host_stop(approx, threshold, cycle_threshold, nsigma_threshold);
        if (r) {
            stop = r;
            break;
        }
        volatile float fl0 = approx * mea;
        float flux_limit = fl0 * factor;
        if (factor > 1.0f) {
            volatile float cap95 = 0.95f * approx;
            flux_limit = std::min(flux_limit, (float)cap95);
        }
        const float selection = std::max(flux_limit, cycle_threshold);
        active_mark_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(residual, mask, n,
                                                                          selection, keep);
        note_launch(ctx, "active_mark_kernel");
        exclusive_scan_u32(ctx, keep, slot, n, total);
        active_fill_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(residual, n, keep, slot,
                                                                          map, pix, val);
        note_launch(ctx, "active_fill_kernel");
        unsigned long long n_active = 0;
        CR_CUDA_CHECK(cudaMemcpyAsync(&n_active, total, 8, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        if (n_active == 0) {
            if (warn) {
                stop = CR_STOP_NO_CLEANABLE_PIXELS;
                break;
            }
            factor *= 1.2f;
            warn = true;
            ++subcycle;
            continue;
        }
        const int64_t limit = std::min<int64_t>(cycle_niter - updates, max_iter);
        CR_CUDA_CHECK(cudaMemsetAsync(delta, 0, (size_t)n * 4, ctx->stream));
        SubArgs sa{(int)n_active, pix, val, map, nx, ny, patch, pnx, pny, rx, ry, model, delta,
                   gain, threshold, cycle_threshold, nsigma_threshold, flux_limit, selection,
                   (int)limit, (int)updates, cap, comp_x ? cx : nullptr, cy, cp, cf, dout,
                   dpeak};
        clark_subcycle_kernel<<<1, kClarkThreads, 0, ctx->stream>>>(sa);
        note_launch(ctx, "clark_subcycle_kernel");
        struct {
            int added, stop;
            float peak;
        } h;
        CR_CUDA_CHECK(cudaMemcpyAsync(&h, dout, 12, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
        approx = h.peak;
        if (h.stop) stop = h.stop;
        updates += h.added;
        if (h.added > 0) {
            updated = true;
            clark_pack_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(delta, nx, ny, 0, work);
            note_launch(ctx, "clark_pack_kernel");
            check_cufft(cufftExecZ2Z(fft, (cufftDoubleComplex*)work, (cufftDoubleComplex*)work,
                                     CUFFT_FORWARD), "cufftExecZ2Z");
            clark_mul_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(work, fpsf, n,
                                                                            1.0 / (double)n);
            note_launch(ctx, "clark_mul_kernel");
            check_cufft(cufftExecZ2Z(fft, (cufftDoubleComplex*)work, (cufftDoubleComplex*)work,
                                     CUFFT_INVERSE), "cufftExecZ2Z");
            clark_subtract_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(residual, work,
                                                                                 n);
            note_launch(ctx, "clark_subtract_kernel");
        }
        if (approx > prev) {
            factor *= 3.0f;
            max_iter = std::min<int64_t>(max_iter, 10);
            warn = true;
        }
        prev = approx;
        if (h.added == 0) break;
        if (stop && updates < cycle_niter) stop = 0;
        ++subcycle;
    }
    if (!updated && !stop) stop = CR_STOP_NO_CLEANABLE_PIXELS;
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    if (comp_x && updates > 0) {
        const size_t m = (size_t)updates * 4;
        // one synchronisation for the four lists, on the context's stream
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_x, cx, m, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_y, cy, m, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_peak, cp, m, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaMemcpyAsync(comp_flux, cf, m, cudaMemcpyDeviceToHost, ctx->stream));
        CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    }
    if (actual) *actual = updates;
    if (stop_out) *stop_out = stop;
}

}  // namespace cr
