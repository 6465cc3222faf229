// cr_beam.cu -- restoring-beam fit, restoration and the PSF sidelobe level.
//
// The fit restates fit_beam_from_psf (beam.rs:27-103) and its helpers: the
// main-lobe search of CASA's FindNpoints (find_points_in_lobe,
// beam.rs:411-480), the square padded window, its bicubic resampling
// (resample_psf / casa_interp_cubic / casa_interp_linear, beam.rs:505-890,
// the bicubic coefficients of Press et al., Numerical Recipes, "bcucof"),
// and the Levenberg-Marquardt fit of CASA's NonLinearFitLM with a final
// undamped Gauss-Newton step (beam.rs:527-610) over width, axial ratio and
// position angle (casa_gaussian_value_and_jacobian, beam.rs:676-713), the
// 3x3 normal equations solved by LDL^T in casacore's order
// (least_squares.rs:10-51), and the float32 arcsec/degree quantisation of the
// result (casa_params_to_beam, beam.rs:721-768).  It is a serial fit of a few
// thousand points and runs on the host in FP64.
//
// Restoration (restore_model, beam.rs:105-120) convolves the model with the
// analytic Gaussian of make_casa_gaussian_psf_image (beam.rs:330-372) by a
// full-plane (circular) FFT convolution on the device, then adds the
// residual; the sidelobe level is estimate_psf_sidelobe_level_with_beam
// (beam.rs:319-328): max(|min psf|, |max(psf - gaussian)|).
#include <cmath>
#include <cstring>
#include <vector>

#include "cr_internal.cuh"

namespace cr {

namespace {

constexpr double kFwhmToInternal = 0.6005612043932249;   // 1 / (2 sqrt(ln 2))
constexpr int kPatchRadius = 20;
constexpr int kRegionPadding = 5;
constexpr int kTargetPoints = 3001;
constexpr int kMaxAttempts = 50;
constexpr double kMinSigma = 1.0e-12;

struct Sample {
    double x, y, v;
};

struct Params {
    double width, ratio, pa;
};

// The image as the fit sees it: x-major, y contiguous.
struct Plane {
    const float* p;
    int64_t nx, ny;
    float at(int64_t x, int64_t y) const { return p[x * ny + y]; }
};

// First occurrence of the largest value, scanning x-major.
bool first_max(const Plane& img, int64_t* px, int64_t* py, float* v) {
    if (img.nx * img.ny == 0) return false;
    int64_t bx = 0, by = 0;
    float best = img.at(0, 0);
    for (int64_t x = 0; x < img.nx; ++x)
        for (int64_t y = 0; y < img.ny; ++y)
            if (img.at(x, y) > best) {
                best = img.at(x, y);
                bx = x;
                by = y;
            }
    *px = bx;
    *py = by;
    *v = best;
    return true;
}

struct Lobe {
    std::vector<Sample> s;
    int64_t blc_x, blc_y, trc_x, trc_y;
};

// The main lobe around the peak: rows outward from the peak in both
// directions, each row walked outward both ways until the values fall below
// amin after having been above it.
bool lobe_points(const Plane& img, int64_t px, int64_t py, int64_t nrow, float amin, double dx,
                 double dy, Lobe* out) {
    Lobe L;
    L.blc_x = img.nx - 1;
    L.blc_y = img.ny - 1;
    L.trc_x = 0;
    L.trc_y = 0;
    int64_t iflip = 1, jflip = 1;
    const size_t maxn = (size_t)((2 * nrow + 1) * (2 * nrow + 1));
    bool full = false;
    for (int jlo = 0; jlo < 2 && !full; ++jlo) {
        jflip = -jflip;
        for (int64_t j = jlo; j <= nrow && !full; ++j) {
            const int64_t jrow = py + j * jflip;
            for (int ilo = 0; ilo < 2 && !full; ++ilo) {
                iflip = -iflip;
                if (jrow > img.ny - 1 || jrow < 0) break;
                bool inlobe = img.at(px, jrow) > amin;
                for (int64_t i = ilo; i <= nrow; ++i) {
                    if (L.s.size() >= maxn) {
                        full = true;
                        break;
                    }
                    const int64_t irow = px + i * iflip;
                    if (irow > img.nx - 1 || irow < 0) break;
                    const float value = img.at(irow, jrow);
                    if (inlobe && value < amin) break;
                    if (value > amin) {
                        inlobe = true;
                        L.blc_x = std::min(L.blc_x, irow);
                        L.blc_y = std::min(L.blc_y, jrow);
                        L.trc_x = std::max(L.trc_x, irow);
                        L.trc_y = std::max(L.trc_y, jrow);
                        L.s.push_back(Sample{(double)(irow - px) * dx, (double)(jrow - py) * dy,
                                             (double)value});
                    }
                }
            }
        }
    }
    if (L.s.empty()) return false;
    // a square bounding box, as FindNpoints forces it
    if (L.blc_x > L.blc_y)
        L.blc_x = L.blc_y;
    else
        L.blc_y = L.blc_x;
    if (L.trc_x > L.trc_y)
        L.trc_y = L.trc_x;
    else
        L.trc_x = L.trc_y;
    *out = std::move(L);
    return true;
}

double interp_linear(const Plane& d, double x, double y) {
    int64_t i = (int64_t)x, j = (int64_t)y;
    if (i == d.nx - 1) --i;
    if (j == d.ny - 1) --j;
    const double tt = x - (double)i, uu = y - (double)j;
    return (1.0 - tt) * (1.0 - uu) * (double)d.at(i, j) + tt * (1.0 - uu) * (double)d.at(i + 1, j) +
           tt * uu * (double)d.at(i + 1, j + 1) + (1.0 - tt) * uu * (double)d.at(i, j + 1);
}

// Bicubic interpolation coefficients from corner values and derivatives
// (the published bcucof weight table).
void bicubic_coefficients(const double y[4], const double y1[4], const double y2[4],
                          const double y12[4], double c[4][4]) {
    static const int wt[16][16] = {
        {1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0},
        {-3, 0, 0, 3, 0, 0, 0, 0, -2, 0, 0, -1, 0, 0, 0, 0},
        {2, 0, 0, -2, 0, 0, 0, 0, 1, 0, 0, 1, 0, 0, 0, 0},
        {0, 0, 0, 0, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 1, 0, 0, 0},
        {0, 0, 0, 0, -3, 0, 0, 3, 0, 0, 0, 0, -2, 0, 0, -1},
        {0, 0, 0, 0, 2, 0, 0, -2, 0, 0, 0, 0, 1, 0, 0, 1},
        {-3, 3, 0, 0, -2, -1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 0, -3, 3, 0, 0, -2, -1, 0, 0},
        {9, -9, 9, -9, 6, 3, -3, -6, 6, -6, -3, 3, 4, 2, 1, 2},
        {-6, 6, -6, 6, -4, -2, 2, 4, -3, 3, 3, -3, -2, -1, -1, -2},
        {2, -2, 0, 0, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0},
        {0, 0, 0, 0, 0, 0, 0, 0, 2, -2, 0, 0, 1, 1, 0, 0},
        {-6, 6, -6, 6, -3, -3, 3, 3, -4, 4, 2, -2, -2, -2, -1, -1},
        {4, -4, 4, -4, 2, 2, -2, -2, 2, -2, -2, 2, 1, 1, 1, 1}};
    double x[16];
    for (int k = 0; k < 4; ++k) {
        x[k] = y[k];
        x[k + 4] = y1[k];
        x[k + 8] = y2[k];
        x[k + 12] = y12[k];
    }
    for (int r = 0; r < 16; ++r) {
        double acc = 0.0;
        for (int k = 0; k < 16; ++k) acc += (double)wt[r][k] * x[k];
        c[r / 4][r % 4] = acc;
    }
}

// Bicubic interpolation with central-difference derivatives formed in
// float32 (as the float image type does), linear near the edges.
double interp_cubic(const Plane& d, double x, double y) {
    const int64_t i = (int64_t)x, j = (int64_t)y;
    if (i <= 0 || i >= d.nx - 2 || j <= 0 || j >= d.ny - 2) return interp_linear(d, x, y);
    const double tt = x - (double)i, uu = y - (double)j;
    auto f = [&](int64_t a, int64_t b) { return d.at(a, b); };
    double v[4] = {f(i, j), f(i + 1, j), f(i + 1, j + 1), f(i, j + 1)};
    double gx[4] = {(double)(f(i + 1, j) - f(i - 1, j)), (double)(f(i + 2, j) - f(i, j)),
                    (double)(f(i + 2, j + 1) - f(i, j + 1)),
                    (double)(f(i + 1, j + 1) - f(i - 1, j + 1))};
    double gy[4] = {(double)(f(i, j + 1) - f(i, j - 1)),
                    (double)(f(i + 1, j + 1) - f(i + 1, j - 1)),
                    (double)(f(i + 1, j + 2) - f(i + 1, j)), (double)(f(i, j + 2) - f(i, j))};
    double gxy[4] = {
        (double)(f(i + 1, j + 1) + f(i - 1, j - 1) - f(i - 1, j + 1) - f(i + 1, j - 1)),
        (double)(f(i + 2, j + 1) + f(i, j - 1) - f(i, j + 1) - f(i + 2, j - 1)),
        (double)(f(i + 2, j + 2) + f(i, j) - f(i, j + 2) - f(i + 2, j)),
        (double)(f(i + 1, j + 2) + f(i - 1, j) - f(i - 1, j + 2) - f(i + 1, j))};
    for (int k = 0; k < 4; ++k) {
        gx[k] /= 2.0;
        gy[k] /= 2.0;
        gxy[k] /= 4.0;
    }
    double c[4][4];
    bicubic_coefficients(v, gx, gy, gxy, c);
    float result = 0.0f;
    for (int r = 3; r >= 0; --r)
        result = (float)(tt * (double)result + ((c[r][3] * uu + c[r][2]) * uu + c[r][1]) * uu +
                         c[r][0]);
    return (double)result;
}

bool fit_samples(const Plane& psf, int64_t px, int64_t py, float peak, double dx, double dy,
                 float cutoff, std::vector<Sample>* out) {
    Lobe first;
    if (!lobe_points(psf, px, py, kPatchRadius, cutoff, dx, dy, &first)) return false;
    int64_t bx = std::max<int64_t>(first.blc_x - kRegionPadding, 0);
    int64_t by = std::max<int64_t>(first.blc_y - kRegionPadding, 0);
    int64_t tx = std::min<int64_t>(first.trc_x + kRegionPadding, psf.nx - 1);
    int64_t ty = std::min<int64_t>(first.trc_y + kRegionPadding, psf.ny - 1);
    const int64_t side = std::max(tx - bx + 1, ty - by + 1);
    if (tx - bx + 1 < side) {
        bx = std::max<int64_t>(bx - (side - (tx - bx + 1)) / 2, 0);
        tx = std::min<int64_t>(bx + side - 1, psf.nx - 1);
        bx = tx + 1 - side;
    }
    if (ty - by + 1 < side) {
        by = std::max<int64_t>(by - (side - (ty - by + 1)) / 2, 0);
        ty = std::min<int64_t>(by + side - 1, psf.ny - 1);
        by = ty + 1 - side;
    }
    const int64_t nx = tx - bx + 1, ny = ty - by + 1;
    std::vector<float> win((size_t)(nx * ny));
    for (int64_t x = 0; x < nx; ++x)
        for (int64_t y = 0; y < ny; ++y) win[x * ny + y] = psf.at(bx + x, by + y) / peak;
    int64_t os = kTargetPoints / (nx * ny);
    os = (int64_t)std::sqrt((double)os);
    if (os == 0) os = 1;
    const Plane w{win.data(), nx, ny};
    const int64_t rx = nx * os - os + 1, ry = ny * os - os + 1;
    std::vector<float> res((size_t)(rx * ry));
    for (int64_t i = 0; i < rx; ++i)
        for (int64_t j = 0; j < ry; ++j) {
            const double x = (double)((float)i / (float)os);
            const double y = (double)((float)j / (float)os);
            res[i * ry + j] = (float)interp_cubic(w, x, y);
        }
    float mx = -INFINITY;
    for (float v : res) mx = std::fmax(mx, v);
    if (!(std::isfinite(mx) && mx > 0.0f)) return false;
    for (float& v : res) v = v / mx;
    const Plane r{res.data(), rx, ry};
    int64_t qx, qy;
    float qv;
    if (!first_max(r, &qx, &qy, &qv)) return false;
    const int64_t min_len = std::min(nx, ny);
    const int64_t nrow = std::max<int64_t>(os * min_len - 1, 0) / 2;
    Lobe second;
    if (!lobe_points(r, qx, qy, nrow, cutoff, dx / (double)os, dy / (double)os, &second))
        return false;
    *out = std::move(second.s);
    return true;
}

bool model_and_jacobian(const Params& p, double x, double y, double* m, double jac[3]) {
    const double w = p.width, q = p.ratio;
    if (!(std::isfinite(w) && std::fabs(w) > kMinSigma && std::isfinite(q) &&
          std::fabs(q) > 1.0e-6 && std::isfinite(p.pa)))
        return false;
    const double c = std::cos(p.pa), s = std::sin(p.pa);
    const double xn = x * c + y * s, yn = -x * s + y * c;
    const double xw = w * q;
    const double xw2 = xw * xw * kFwhmToInternal * kFwhmToInternal;
    const double yw2 = w * w * kFwhmToInternal * kFwhmToInternal;
    const double x2w = 2.0 * xn / xw2, y2w = 2.0 * yn / yw2;
    const double x2w2 = x2w * xn, y2w2 = y2w * yn;
    const double v = std::exp(-(xn * xn / xw2 + yn * yn / yw2));
    jac[0] = v * ((x2w2 + y2w2) / w);
    jac[1] = v * x2w2 * w / xw;
    jac[2] = -v * (x2w * (-x * s + y * c) + y2w * (-x * c - y * s));
    *m = v;
    return std::isfinite(v) && std::isfinite(jac[0]) && std::isfinite(jac[1]) &&
           std::isfinite(jac[2]);
}

bool cost_of(const std::vector<Sample>& S, const Params& p, double* cost) {
    if (!(std::isfinite(p.width) && std::fabs(p.width) > kMinSigma && std::isfinite(p.ratio) &&
          std::isfinite(p.pa)))
        return false;
    double acc = 0.0;
    for (const Sample& s : S) {
        double m, j[3];
        if (!model_and_jacobian(p, s.x, s.y, &m, j)) m = 0.0;
        const double r = m - s.v;
        acc += r * r;
    }
    *cost = acc;
    return std::isfinite(acc);
}

// J^T J (symmetric, upper triangle accumulated) and J^T r.
bool normal_equations(const std::vector<Sample>& S, const Params& p, double N[3][3],
                      double g[3]) {
    for (int a = 0; a < 3; ++a) {
        g[a] = 0.0;
        for (int b = 0; b < 3; ++b) N[a][b] = 0.0;
    }
    for (const Sample& s : S) {
        double m, j[3];
        if (!model_and_jacobian(p, s.x, s.y, &m, j)) return false;
        const double r = m - s.v;
        for (int a = 0; a < 3; ++a) {
            g[a] += j[a] * r;
            for (int b = a; b < 3; ++b) N[a][b] += j[a] * j[b];
        }
    }
    for (int a = 0; a < 3; ++a)
        for (int b = 0; b < a; ++b) N[a][b] = N[b][a];
    return true;
}

// LDL^T of a symmetric 3 x 3 system with the pivot test of casacore's solver.
bool solve_ldlt(double N[3][3], const double k[3], double out[3]) {
    for (int r = 0; r < 3; ++r) {
        const double orig = N[r][r];
        double d = orig;
        for (int p = 0; p < r; ++p) d -= N[p][r] * N[p][r] / N[p][p];
        if (!std::isfinite(d) || d * d / orig <= 1.0e-12) return false;
        N[r][r] = d;
        for (int c = r + 1; c < 3; ++c)
            for (int p = 0; p < r; ++p) N[r][c] -= N[p][r] * N[p][c] / N[p][p];
    }
    double x[3];
    for (int r = 0; r < 3; ++r) {
        x[r] = k[r];
        for (int p = 0; p < r; ++p) x[r] -= N[p][r] * x[p] / N[p][p];
    }
    for (int r = 2; r >= 0; --r) {
        for (int c = r + 1; c < 3; ++c) x[r] -= N[r][c] * x[c];
        x[r] /= N[r][r];
    }
    for (int r = 0; r < 3; ++r) out[r] = x[r];
    return true;
}

double wrap_pa(double a) {
    const double pi = M_PI, h = M_PI / 2.0, th = 3.0 * M_PI / 2.0;
    while (std::fabs(a / h) > 1.0) {
        if (a > th)
            a -= 2.0 * pi;
        else if (a > h)
            a -= pi;
        else if (a < -th)
            a += 2.0 * pi;
        else
            a += pi;
    }
    return a;
}

bool params_to_beam(const Params& p, cr_beam* b) {
    if (!(std::isfinite(p.width) && std::isfinite(p.ratio) && std::isfinite(p.pa))) return false;
    double maj, mn, pa;
    if (std::fabs(p.ratio) > 1.0) {
        maj = std::fabs(p.width * p.ratio);
        mn = std::fabs(p.width);
        pa = p.pa - M_PI / 2.0;
    } else {
        maj = std::fabs(p.width);
        mn = std::fabs(p.width * p.ratio);
        pa = p.pa;
    }
    pa = wrap_pa(pa);
    if (mn > maj) {
        std::swap(maj, mn);
        pa = wrap_pa(pa + M_PI / 2.0);
    }
    // fitted in FP64, reported as float32 arcseconds and degrees
    const double r2d = 180.0 / M_PI, r2as = 3600.0 * r2d;
    b->major_fwhm_rad = (double)(float)(maj * r2as) / r2as;
    b->minor_fwhm_rad = (double)(float)(mn * r2as) / r2as;
    b->position_angle_rad = (double)(float)(pa * r2d) / r2d;
    return true;
}

bool fit_lm(const std::vector<Sample>& S, double cell_x, cr_beam* beam) {
    Params acc{2.5 * std::fabs(cell_x), 0.5, 1.0};
    double N[3][3], k[3];
    if (!normal_equations(S, acc, N, k)) return false;
    for (double& v : k) v = -v;
    double cost;
    if (!cost_of(S, acc, &cost)) return false;
    double lambda = 1.0e-3, step = 2.0;
    Params cand = acc;
    double delta[3] = {0.0, 0.0, 0.0};
    bool first = true;
    for (int it = 0; it < 1000; ++it) {
        if (!first) {
            double ccost;
            if (!cost_of(S, cand, &ccost)) return false;
            double expected = 0.0;
            for (int a = 0; a < 3; ++a) expected += delta[a] * (lambda * delta[a] * N[a][a] + k[a]);
            expected *= 0.5;
            const double actual = (cost - ccost) * 0.5;
            if (expected > 0.0 && actual > 0.0) {
                acc = cand;
                cost = ccost;
                if (!normal_equations(S, acc, N, k)) return false;
                for (double& v : k) v = -v;
                lambda *= 0.3;
                step = 2.0;
                if (std::fabs(k[0]) <= 1.0e-8 && std::fabs(k[1]) <= 1.0e-8 &&
                    std::fabs(k[2]) <= 1.0e-8)
                    break;
            } else {
                lambda *= step;
                step *= 2.0;
                if (step > 1.0e10) break;
            }
        }
        double D[3][3];
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) D[a][b] = N[a][b];
        for (int a = 0; a < 3; ++a) D[a][a] *= 1.0 + lambda;
        if (!solve_ldlt(D, k, delta)) return false;
        cand = Params{acc.width + delta[0], acc.ratio + delta[1], acc.pa + delta[2]};
        first = false;
        const double dn = std::sqrt(delta[0] * delta[0] + delta[1] * delta[1] + delta[2] * delta[2]);
        const double pn = std::sqrt(acc.width * acc.width + acc.ratio * acc.ratio + acc.pa * acc.pa);
        if (dn <= 1.0e-8 * (pn + 1.0e-8)) break;
    }
    // one undamped Gauss-Newton step from the last candidate
    double F[3][3], fk[3], fd[3];
    if (!normal_equations(S, cand, F, fk)) return false;
    for (double& v : fk) v = -v;
    if (!solve_ldlt(F, fk, fd)) return false;
    const Params fin{cand.width + fd[0], cand.ratio + fd[1], cand.pa + fd[2]};
    double fc;
    if (!cost_of(S, fin, &fc)) return false;
    return params_to_beam(fin, beam);
}

// ---- device: the analytic Gaussian, restoration, sidelobe level -------------------
struct GaussArgs {
    int32_t nx, ny;
    double cos_pa, sin_pa, dx, dy, sbmaj, sbmin, ref_x, ref_y;
};

__device__ __forceinline__ float gauss_at(const GaussArgs& g, int64_t x, int64_t y) {
    const double fx = (double)x - g.ref_x, fy = (double)y - g.ref_y;
    const double major = g.cos_pa * fx * g.dx + g.sin_pa * fy * g.dy;
    const double minor = -g.sin_pa * fx * g.dx + g.cos_pa * fy * g.dy;
    const double r = g.sbmaj * major * major + g.sbmin * minor * minor;
    return r < 20.0 ? (float)exp(-r) : 0.0f;
}

// The Gaussian moved so that its reference pixel sits at (0, 0) (circular),
// as complex FP64: convolving with it keeps components in place.
__global__ void gauss_shifted_kernel(GaussArgs g, double2* out) {
    const int64_t n = (int64_t)g.nx * g.ny;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = k / g.ny, y = k % g.ny;
        const int64_t sx = (x + (int64_t)g.ref_x) % g.nx, sy = (y + (int64_t)g.ref_y) % g.ny;
        out[k] = make_double2((double)gauss_at(g, sx, sy), 0.0);
    }
}

__global__ void widen_real_kernel(const float* in, int64_t n, double2* out) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        out[k] = make_double2((double)in[k], 0.0);
}

__global__ void multiply_kernel(double2* a, const double2* b, int64_t n) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const double2 x = a[k], y = b[k];
        a[k] = make_double2(x.x * y.x - x.y * y.y, x.x * y.y + x.y * y.x);
    }
}

__global__ void restore_out_kernel(const double2* conv, const float* residual, int64_t n,
                                   double inv_n, float* out) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const float m = (float)(conv[k].x * inv_n);
        out[k] = residual ? m + residual[k] : m;
    }
}

__global__ void restore_out_kernel_copy(const float* model, const float* residual, int64_t n,
                                        float* out) {
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x)
        out[k] = residual ? model[k] + residual[k] : model[k];
}

// all_min = min(0, psf), all_max = max(0, psf - gaussian), as float bits
__global__ void sidelobe_kernel(const float* psf, GaussArgs g, unsigned int* mins,
                                unsigned int* maxs) {
    const int64_t n = (int64_t)g.nx * g.ny;
    float lo = 0.0f, hi = 0.0f;
    for (int64_t k = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; k < n;
         k += (int64_t)gridDim.x * blockDim.x) {
        const float v = psf[k];
        lo = fminf(lo, v);
        hi = fmaxf(hi, v - gauss_at(g, k / g.ny, k % g.ny));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
    }
    // |lo| for lo <= 0 and hi >= 0 compare as unsigned float bits
    if ((threadIdx.x & 31) == 0) {
        atomicMax(mins, __float_as_uint(0.0f - lo));   // +0 for an all-positive range
        atomicMax(maxs, __float_as_uint(hi + 0.0f));
    }
}

GaussArgs gauss_args(int32_t nx, int32_t ny, double cell_x, double cell_y, const cr_beam& b) {
    GaussArgs g{};
    g.nx = nx;
    g.ny = ny;
    const double pa = b.position_angle_rad + M_PI / 2.0;
    g.cos_pa = std::cos(pa);
    g.sin_pa = std::sin(pa);
    g.ref_x = (double)(nx / 2);
    g.ref_y = (double)(ny / 2);
    g.dx = std::fabs(cell_x);
    g.dy = std::fabs(cell_y);
    g.sbmaj = 4.0 * M_LN2 * std::pow(1.0 / b.major_fwhm_rad, 2);
    g.sbmin = 4.0 * M_LN2 * std::pow(1.0 / b.minor_fwhm_rad, 2);
    return g;
}

bool beam_ok(const cr_beam& b) {
    return std::isfinite(b.major_fwhm_rad) && b.major_fwhm_rad > 0.0 &&
           std::isfinite(b.minor_fwhm_rad) && b.minor_fwhm_rad > 0.0;
}

}  // namespace

bool fit_beam(const float* psf, int64_t nx, int64_t ny, double cell_x, double cell_y,
              float cutoff, cr_beam* beam, int32_t* attempts, float* cutoff_used) {
    const Plane img{psf, nx, ny};
    int64_t px, py;
    float peak;
    *attempts = 0;
    *cutoff_used = 0.0f;
    if (!first_max(img, &px, &py, &peak) || !(std::isfinite(peak) && peak > 0.0f)) return false;
    float active = std::min(std::max(cutoff, 0.01f), 0.99f);
    const double dx = std::fabs(cell_x), dy = std::fabs(cell_y);
    for (int attempt = 1; attempt <= kMaxAttempts; ++attempt) {
        *attempts = attempt;
        std::vector<Sample> S;
        if (fit_samples(img, px, py, peak, dx, dy, active, &S) && S.size() >= 12 &&
            fit_lm(S, cell_x, beam)) {
            *cutoff_used = active;
            return true;
        }
        active /= 1.5f;
    }
    return false;
}

void restore(cr_ctx* ctx, const float* model, const float* residual, int32_t nx, int32_t ny,
             double cell_x, double cell_y, const cr_beam& beam, float* out) {
    const int64_t n = (int64_t)nx * ny;
    if (!beam_ok(beam)) fail(CR_INVALID, "beam axes must be finite and positive");
    if (nx % 2 || ny % 2) fail(CR_INVALID, "restoration needs even image sides");
    // an empty model (every |value| <= 1e-12) is returned as it is
    unsigned int* pk = (unsigned int*)workspace(ctx, "rs_peak", 4);
    abs_peak(ctx, model, n, pk);
    unsigned int pkh = 0;
    CR_CUDA_CHECK(cudaMemcpyAsync(&pkh, pk, 4, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    float peak;
    std::memcpy(&peak, &pkh, 4);
    if (!(peak > 1.0e-12f)) {
        restore_out_kernel_copy<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(model, residual, n,
                                                                              out);
        note_launch(ctx, "restore_out_kernel_copy");
        return;
    }
    double2* a = (double2*)workspace(ctx, "rs_model", (size_t)n * 16);
    double2* g = (double2*)workspace(ctx, "rs_gauss", (size_t)n * 16);
    const GaussArgs ga = gauss_args(nx, ny, cell_x, cell_y, beam);
    widen_real_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(model, n, a);
    note_launch(ctx, "widen_real_kernel");
    gauss_shifted_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(ga, g);
    note_launch(ctx, "gauss_shifted_kernel");
    cufftHandle plan = fft_plan(ctx, nx, ny);
    check_cufft(cufftExecZ2Z(plan, (cufftDoubleComplex*)a, (cufftDoubleComplex*)a, CUFFT_FORWARD),
                "cufftExecZ2Z");
    check_cufft(cufftExecZ2Z(plan, (cufftDoubleComplex*)g, (cufftDoubleComplex*)g, CUFFT_FORWARD),
                "cufftExecZ2Z");
    multiply_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(a, g, n);
    note_launch(ctx, "multiply_kernel");
    check_cufft(cufftExecZ2Z(plan, (cufftDoubleComplex*)a, (cufftDoubleComplex*)a, CUFFT_INVERSE),
                "cufftExecZ2Z");
    restore_out_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(a, residual, n,
                                                                     1.0 / (double)n, out);
    note_launch(ctx, "restore_out_kernel");
}

float psf_sidelobe(cr_ctx* ctx, const float* psf, int32_t nx, int32_t ny, double cell_x,
                   double cell_y, const cr_beam& beam) {
    if (!beam_ok(beam)) return 0.0f;
    const int64_t n = (int64_t)nx * ny;
    unsigned int* mm = (unsigned int*)workspace(ctx, "sl_minmax", 8);
    CR_CUDA_CHECK(cudaMemsetAsync(mm, 0, 8, ctx->stream));
    sidelobe_kernel<<<grid_blocks(n, 256), 256, 0, ctx->stream>>>(
        psf, gauss_args(nx, ny, cell_x, cell_y, beam), mm, mm + 1);
    note_launch(ctx, "sidelobe_kernel");
    unsigned int h[2];
    CR_CUDA_CHECK(cudaMemcpyAsync(h, mm, 8, cudaMemcpyDeviceToHost, ctx->stream));
    CR_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    float lo, hi;
    std::memcpy(&lo, &h[0], 4);
    std::memcpy(&hi, &h[1], 4);
    return std::fmax(lo, hi);
}

}  // namespace cr
