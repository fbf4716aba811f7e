// fg_host.cpp -- host-side parameter resolution of the C-ABI (no GPU involved).
//
// Restates the crate's host arithmetic around the integrators: ParamsBuilder::build and its
// validators (src/params.rs:141-179, 223-261, 282-390), derive_common and resolve_output_size
// (src/model.rs:181-226, 267-298), RadiusProfile::quantile (src/model.rs:150-164), make_offsets
// (src/rng.rs:9-24), normalize_plane / lambda_plane (src/model.rs:228-265) and choose_algorithm
// (src/choose.rs:4-26).  Compiled with -ffp-contract=off so every f32/f64 expression rounds as the
// Rust source's does.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <mutex>
#include <thread>
#include <vector>

#include "../../include/film_grain_gb300.h"
#include "fg_host.h"
#include "fg_internal.h"
#include "fg_rng.cuh"

namespace fg {

static thread_local std::string g_last_error;

fg_status set_error(fg_status code, const std::string &msg) {
    g_last_error = msg;
    return code;
}
void clear_error() { g_last_error.clear(); }
const char *last_error() { return g_last_error.c_str(); }

static const float kEps = 1e-6f;  // src/model.rs:10

static fg_status params_error(const char *field, const char *msg) {
    return set_error(FG_ERR_PARAMS, std::string("parameter error: ") + field + ": " + msg);
}
static bool ensure_positive(float v, const char *field, fg_status *st) {
    if (!std::isfinite(v)) { *st = params_error(field, "value must be finite"); return false; }
    if (v <= 0.0f) { *st = params_error(field, "value must be greater than 0"); return false; }
    return true;
}
static bool ensure_non_negative(float v, const char *field, fg_status *st) {
    if (!std::isfinite(v)) { *st = params_error(field, "value must be finite"); return false; }
    if (v < 0.0f) { *st = params_error(field, "value must be >= 0"); return false; }
    return true;
}

float default_cell_delta(float radius_mean) {
    if (radius_mean <= 0.0f) return 1.0f;
    float inv = std::ceil(1.0f / radius_mean);
    if (inv < 1.0f) inv = 1.0f;
    return 1.0f / inv;
}

fg_status params_build(const fg_params_builder &b, fg_params *out) {
    fg_status st = FG_OK;
    if (!ensure_positive(b.radius_mean, "radius", &st)) return st;
    if (!ensure_non_negative(b.radius_stddev, "radius-stddev", &st)) return st;
    if (!ensure_positive(b.zoom, "zoom", &st)) return st;
    if (!ensure_positive(b.sigma_px, "sigma", &st)) return st;
    if (b.radius_dist != FG_RADIUS_CONST && b.radius_dist != FG_RADIUS_LOGNORM)
        return params_error("radius-dist", "expected const or lognorm");
    if (b.algo < FG_ALGO_AUTO || b.algo > FG_ALGO_PIXEL) return params_error("algo", "expected auto, grain or pixel");
    if (b.color_mode != FG_COLOR_LUMA && b.color_mode != FG_COLOR_RGB)
        return params_error("color-mode", "expected luma or rgb");
    if (b.max_radius_kind == FG_MAXR_ABSOLUTE) {
        if (!std::isfinite(b.max_radius_value)) return params_error("max-radius", "absolute radius must be finite");
        if (b.max_radius_value <= 0.0f) return params_error("max-radius", "absolute radius must be > 0");
    } else if (b.max_radius_kind == FG_MAXR_QUANTILE) {
        if (!std::isfinite(b.max_radius_value)) return params_error("max-radius", "quantile must be finite");
        if (!(0.0f < b.max_radius_value && b.max_radius_value < 1.0f))
            return params_error("max-radius", "quantile must lie in the open interval (0,1)");
    } else {
        return params_error("max-radius", "expected a positive number or 'quantile'");
    }
    if (b.has_roi && (b.roi_x1 <= b.roi_x0 || b.roi_y1 <= b.roi_y0))
        return params_error("roi", "roi end must be greater than start (exclusive bounds)");
    // size: width 0 means "no size"; a height alone is not expressible here (size_w == 0 wins).
    float cell;
    if (std::isnan(b.cell_delta) || b.cell_delta <= 0.0f) {
        if (b.cell_delta < 0.0f) return params_error("cell", "cell size must be > 0");
        cell = default_cell_delta(b.radius_mean);
    } else {
        if (!std::isfinite(b.cell_delta)) return params_error("cell", "cell size must be finite");
        cell = b.cell_delta;
    }

    fg_params p;
    std::memset(&p, 0, sizeof p);
    p.radius_dist = b.radius_dist;
    p.radius_mean = b.radius_mean;
    // derive_radius_parameters (src/params.rs:223-253)
    if (b.radius_dist == FG_RADIUS_CONST) {
        p.radius_stddev = 0.0f;
        p.has_log_params = 0;
    } else {
        if (b.radius_stddev == 0.0f) {
            p.radius_stddev = 0.0f;
            p.radius_log_mu = std::log(b.radius_mean);
            p.radius_log_sigma = 0.0f;
        } else {
            float vr = (b.radius_stddev * b.radius_stddev) / (b.radius_mean * b.radius_mean);
            float sigma_sq = std::log(1.0f + vr);
            float sigma = std::sqrt(sigma_sq);
            float mu = std::log(b.radius_mean) - 0.5f * sigma_sq;
            p.radius_stddev = b.radius_stddev;
            p.radius_log_mu = mu;
            p.radius_log_sigma = sigma;
        }
        p.has_log_params = 1;
    }
    p.zoom = b.zoom;
    p.sigma_px = b.sigma_px;
    p.n_samples = b.n_samples > 0 ? b.n_samples : 1;
    p.algo = b.algo;
    p.max_radius_kind = b.max_radius_kind;
    p.max_radius_value = b.max_radius_value;
    p.cell_delta = cell;
    p.color_mode = b.color_mode;
    p.has_roi = b.has_roi;
    p.roi_x0 = b.roi_x0; p.roi_y0 = b.roi_y0; p.roi_x1 = b.roi_x1; p.roi_y1 = b.roi_y1;
    p.size_w = b.size_w;
    p.size_h = b.size_w ? b.size_h : 0;
    p.seed = b.seed;
    *out = p;
    clear_error();
    return FG_OK;
}

// Phi^-1(p) to double accuracy: a rational first guess, then Newton steps on the erfc form of the
// CDF, Phi(x) = erfc(-x / sqrt 2) / 2.  Feeds only the f32 max radius.
static double inv_std_normal_cdf(double p) {
    double t = std::sqrt(-2.0 * std::log(p < 0.5 ? p : 1.0 - p));
    // Abramowitz & Stegun 26.2.23 starting point (|error| < 4.5e-4)
    double x = t - (2.515517 + 0.802853 * t + 0.010328 * t * t) / (1.0 + 1.432788 * t + 0.189269 * t * t + 0.001308 * t * t * t);
    if (p < 0.5) x = -x;
    for (int it = 0; it < 6; it++) {
        double cdf = 0.5 * std::erfc(-x / 1.4142135623730951);
        double pdf = std::exp(-0.5 * x * x) / 2.5066282746310002;
        double step = (cdf - p) / pdf;
        x -= step;
        if (std::fabs(step) < 1e-17 * (1.0 + std::fabs(x))) break;
    }
    return x;
}

float radius_quantile(const fg_params &p, float prob) {
    if (p.radius_dist == FG_RADIUS_CONST) return p.radius_mean;
    double mu = p.has_log_params ? (double)p.radius_log_mu : (double)p.radius_mean;
    double sigma = p.has_log_params ? (double)p.radius_log_sigma : 0.0;
    if (sigma == 0.0) return (float)std::exp(mu);
    double z = inv_std_normal_cdf((double)prob);
    return (float)std::exp(mu + sigma * z);
}

void make_offsets(uint64_t seed, uint32_t n, float sigma, float *out) {
    if (n == 0) return;
    float s = sigma > 1.1920928955078125e-07f ? sigma : 1.1920928955078125e-07f;  // max(f32::EPSILON)
    double sd = (double)s;
    ChaChaStream rng{chacha12_seed_from_u64(splitmix64(seed ^ kOffsetStream))};
    for (uint32_t k = 0; k < n; k++) {
        out[2 * k] = (float)normal_sample(0.0, sd, rng);
        out[2 * k + 1] = (float)normal_sample(0.0, sd, rng);
    }
}

fg_status derive(const fg_params &p, int64_t in_w, int64_t in_h, fg_derived *d, float *offsets, float *offsets_input) {
    if (in_w <= 0 || in_h <= 0) return set_error(FG_ERR_INVALID, "input image is empty after ROI");
    int64_t out_w, out_h;
    if (p.size_w > 0) {
        out_w = p.size_w;
        if (p.size_h > 0) out_h = p.size_h;
        else {
            float aspect = (float)in_h / (float)in_w;
            float c = std::round((float)p.size_w * aspect);
            if (c < 1.0f) c = 1.0f;
            out_h = (int64_t)c;
        }
        if (out_h == 0) return set_error(FG_ERR_INVALID, "output height must be > 0");
    } else {
        float w = std::ceil((float)in_w * p.zoom); if (w < 1.0f) w = 1.0f;
        float h = std::ceil((float)in_h * p.zoom); if (h < 1.0f) h = 1.0f;
        out_w = (int64_t)w;
        out_h = (int64_t)h;
    }
    if (out_w <= 0 || out_h <= 0) return set_error(FG_ERR_INVALID, "output dimensions must be positive");
    if (p.radius_dist == FG_RADIUS_LOGNORM) {
        if (!p.has_log_params) return set_error(FG_ERR_INVALID, "missing log-normal mean; parameters were not derived");
        if (!(p.radius_log_sigma >= 0.0f) || !std::isfinite(p.radius_log_sigma) || !std::isfinite(p.radius_log_mu))
            return set_error(FG_ERR_INVALID, "invalid log-normal parameters");
    }
    const float PI = 3.14159265358979323846f;
    float mean_sq = p.radius_mean * p.radius_mean;
    float var = p.radius_stddev * p.radius_stddev;
    float ms = mean_sq + var;
    if (ms < kEps) ms = kEps;
    d->input_width = in_w;
    d->input_height = in_h;
    d->output_width = out_w;
    d->output_height = out_h;
    d->inv_e_pi_r2 = 1.0f / (PI * ms);
    float rm = (p.max_radius_kind == FG_MAXR_ABSOLUTE) ? p.max_radius_value : radius_quantile(p, p.max_radius_value);
    d->rm = rm > kEps ? rm : kEps;
    float delta = p.cell_delta > 0.0f ? p.cell_delta : default_cell_delta(p.radius_mean);
    d->delta = delta > kEps ? delta : kEps;
    d->n_offsets = p.n_samples;
    if (offsets || offsets_input) {
        std::vector<float> tmp(2 * (size_t)p.n_samples);
        make_offsets(p.seed, p.n_samples, p.sigma_px, tmp.data());
        if (offsets) std::memcpy(offsets, tmp.data(), tmp.size() * sizeof(float));
        if (offsets_input)
            for (size_t i = 0; i < tmp.size(); i++) offsets_input[i] = tmp[i] / p.zoom;
    }
    clear_error();
    return FG_OK;
}

int32_t choose_algorithm(const fg_params &p, const fg_derived &d) {
    if (p.algo != FG_ALGO_AUTO) return p.algo;
    float mean = std::max(p.radius_mean, 1e-6f);
    float sr = mean > 0.0f ? p.radius_stddev / mean : 0.0f;
    float rr = d.rm / mean;
    if (sr < 0.1f && mean < 0.5f && p.n_samples <= 64) return FG_ALGO_PIXEL;
    if (rr > 8.0f || sr > 0.6f || p.n_samples > 96) return FG_ALGO_GRAIN;
    if (p.n_samples <= 24 && rr < 5.0f) return FG_ALGO_PIXEL;
    return FG_ALGO_GRAIN;
}

// Chunks a parallel pass over n elements uses: one per host core, at least 16384 elements each (a
// 256x256 plane already splits four ways; its lambda pass took 1.2 ms on one core, 0.6 ms on four).
static int64_t chunk_count(int64_t n) {
    unsigned hw = std::thread::hardware_concurrency();
    return std::min<int64_t>(hw ? hw : 1, std::max<int64_t>(1, n / 16384));
}

// Parallel-for over [0, n) in chunk_count(n) contiguous chunks on the host's cores; f(t, b, e) runs
// chunk t = [b, e).
template <class F>
static void parallel_chunks(int64_t n, F f) {
    const int64_t nt = chunk_count(n);
    if (nt <= 1) { f(0, 0, n); return; }
    std::vector<std::thread> th;
    int64_t per = (n + nt - 1) / nt;
    for (int64_t t = 0; t < nt; t++) {
        int64_t b = t * per, e = std::min(n, b + per);
        if (b < e) th.emplace_back(f, t, b, e);
    }
    for (auto &t : th) t.join();
}

static inline float clampf(float x, float lo, float hi) {
    if (x < lo) x = lo;
    if (x > hi) x = hi;
    return x;
}

// The plane's maximum as the reference folds it, fold(0.0, f32::max): f32::max (fmax) ignores NaN and
// is commutative and associative, so per-chunk folds from 0.0 combined with fmax give the same value.
static float plane_max(const float *src, int64_t n) {
    std::vector<float> part((size_t)chunk_count(n), 0.0f);
    parallel_chunks(n, [&](int64_t t, int64_t b, int64_t e) {
        float m = 0.0f;
        for (int64_t i = b; i < e; i++) m = std::fmax(m, src[i]);
        part[(size_t)t] = m;
    });
    float mx = 0.0f;
    for (float m : part) mx = std::fmax(mx, m);
    return mx;
}

static inline float normalized_value(float v, bool already, float den) {
    return clampf(already ? v : v / den, 0.0f, 1.0f - kEps);
}

static inline float lambda_value(float norm, float inv_e_pi_r2) {
    float c = clampf(norm, 0.0f, 1.0f - kEps);
    float safe = std::fmax(1.0f - c, kEps);
    float act = -inv_e_pi_r2 * std::log(safe);
    return std::fmin(act, 1.0e6f);
}

float normalize_plane(const float *src, int64_t n, float *dst) {
    const float mx = plane_max(src, n);
    const bool already = mx <= 1.0f + kEps;
    float den = mx + kEps;
    if (den < kEps) den = kEps;
    parallel_chunks(n, [&](int64_t, int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) dst[i] = normalized_value(src[i], already, den);
    });
    return mx;
}

void lambda_plane(const float *norm, int64_t n, float inv_e_pi_r2, float *dst) {
    parallel_chunks(n, [&](int64_t, int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) dst[i] = lambda_value(norm[i], inv_e_pi_r2);
    });
}

float lambda_from_plane(const float *src, int64_t n, float inv_e_pi_r2, float *dst) {
    const float mx = plane_max(src, n);
    const bool already = mx <= 1.0f + kEps;
    float den = mx + kEps;
    if (den < kEps) den = kEps;
    parallel_chunks(n, [&](int64_t, int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) dst[i] = lambda_value(normalized_value(src[i], already, den), inv_e_pi_r2);
    });
    return mx;
}

// ------------------------------------------------------------------ the platform logf, tabulated
// lambda_plane takes the logarithm of safe = max(1 - c, 1e-6) with c clamped to [0, 1 - 1e-6]
// (src/model.rs:259-262).  1 - c is always a multiple of 2^-24 in f32, so safe is k * 2^-24 with
// 17 <= k <= 2^24, or 1e-6 itself when c is NaN: 16,777,201 possible inputs.  The device evaluates
// RN_f32(log((double)x)), the correctly rounded logarithm unless log(x) lies within a few double ulps
// of an f32 rounding boundary; the platform logf differs from the correctly rounded value on about
// 0.1 % of inputs.  Every reachable input where the two differ, or where a last-ulp difference between
// this host's and the device's double log could move the f32 rounding (|log x| * 2^-50 margin,
// several double ulps), is recorded with the platform logf's result, so the device reproduces this
// process's logf bit for bit on every input lambda_plane can produce.
static uint32_t f32_bits_host(float f) {
    uint32_t b;
    std::memcpy(&b, &f, 4);
    return b;
}

// Whether x needs a table entry; *g receives the platform logf.
static bool logf_exception(float x, float *g) {
    *g = std::log(x);  // the platform logf, as lambda_value calls it
    const double d = std::log((double)x);
    const float f = (float)d;
    if (d != 0.0) {
        const double m = std::ldexp(std::fabs(d), -50);
        if ((float)(d - m) != f || (float)(d + m) != f) return true;
    }
    return f32_bits_host(*g) != f32_bits_host(f);
}

const LogfTable &logf_table() {
    static LogfTable t;
    static std::once_flag once;
    std::call_once(once, [] {
        t.lo_bits = f32_bits_host(kEps);
        t.hi_bits = f32_bits_host(1.0f);
        t.shift = 13;
        float g;
        if (logf_exception(kEps, &g)) {  // 1e-6 < 17 * 2^-24: the first key
            t.keys.push_back(t.lo_bits);
            t.vals.push_back(f32_bits_host(g));
        }
        const int64_t k0 = 17, n = (1 << 24) - k0 + 1;
        std::vector<std::vector<uint32_t>> part((size_t)chunk_count(n));
        parallel_chunks(n, [&](int64_t c, int64_t b, int64_t e) {
            std::vector<uint32_t> &out = part[(size_t)c];
            for (int64_t i = b; i < e; i++) {
                const float x = std::ldexp((float)(k0 + i), -24);  // exact
                float gx;
                if (logf_exception(x, &gx)) {
                    out.push_back(f32_bits_host(x));
                    out.push_back(f32_bits_host(gx));
                }
            }
        });
        for (const auto &v : part)
            for (size_t k = 0; k < v.size(); k += 2) {
                t.keys.push_back(v[k]);
                t.vals.push_back(v[k + 1]);
            }
        const uint32_t nb = ((t.hi_bits - t.lo_bits) >> t.shift) + 1;
        t.bucket_start.assign((size_t)nb + 1, 0);
        size_t j = 0;
        for (uint32_t k = 0; k <= nb; k++) {
            const uint64_t first = (uint64_t)t.lo_bits + ((uint64_t)k << t.shift);  // first input of bucket k
            while (j < t.keys.size() && t.keys[j] < first) j++;
            t.bucket_start[k] = (uint32_t)j;
        }
    });
    return t;
}

// load_luma_workspace / load_rgb_workspace (src/color.rs:158-213) from interleaved f32 RGB, with the
// optional ROI crop of apply_roi (src/color.rs:215-231).
static inline float clamp01(float v) { return clampf(v, 0.0f, 1.0f); }

void split_planes(const float *rgb, int64_t w, int64_t x0, int64_t y0, int64_t cw, int64_t ch, int luma,
                  float *p0, float *p1, float *p2) {
    const float YR = 0.2126f, YG = 0.7152f, YB = 0.0722f, CBD = 1.8556f, CRD = 1.5748f;
    parallel_chunks(cw * ch, [&](int64_t, int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            int64_t x = x0 + i % cw, y = y0 + i / cw;
            const float *px = rgb + 3 * (y * w + x);
            float r = clamp01(px[0]), g = clamp01(px[1]), bl = clamp01(px[2]);
            if (luma) {
                float l = YR * r + YG * g + YB * bl;
                p1[i] = (bl - l) / CBD;
                p2[i] = (r - l) / CRD;
                p0[i] = clamp01(l);
            } else {
                p0[i] = r; p1[i] = g; p2[i] = bl;
            }
        }
    });
}

}  // namespace fg

// The plane entry points on device memory (src and dst both device pointers): the same passes on the
// GPU, bit-identical (fg_lambda.cu).  Returns the plane maximum when normalizing; NaN with the error
// message set when the call fails.
namespace fg {
static float device_pass(const float *src, int64_t n, int normalize, int lambda, float inv_e_pi_r2, float *dst) {
    if (!is_device_ptr(src) || !is_device_ptr(dst)) {
        set_error(FG_ERR_INVALID, "src and dst must both be host memory or both device memory");
        return std::nanf("");
    }
    float mx = 0.0f;
    if (device_plane_pass(src, n, normalize, lambda, inv_e_pi_r2, dst, &mx) != FG_OK) return std::nanf("");
    clear_error();
    return mx;
}
}  // namespace fg

// ------------------------------------------------------------------ C-ABI (host-only entry points)
extern "C" {

FG_API fg_status fg_params_build(const fg_params_builder *builder, fg_params *out) {
    if (!builder || !out) return fg::set_error(FG_ERR_INVALID, "null pointer");
    return fg::params_build(*builder, out);
}

FG_API fg_status fg_derive(const fg_params *params, int64_t input_width, int64_t input_height, fg_derived *out,
                           float *offsets, float *offsets_input) {
    if (!params || !out) return fg::set_error(FG_ERR_INVALID, "null pointer");
    return fg::derive(*params, input_width, input_height, out, offsets, offsets_input);
}

FG_API int32_t fg_choose_algorithm(const fg_params *params, const fg_derived *derived) {
    if (!params || !derived) return FG_ALGO_GRAIN;
    return fg::choose_algorithm(*params, *derived);
}

FG_API float fg_default_cell_delta(float radius_mean) { return fg::default_cell_delta(radius_mean); }

FG_API float fg_normalize_plane(const float *src, int64_t n, float *dst) {
    if (!src || !dst || n <= 0) return 0.0f;
    if (fg::is_device_ptr(src) || fg::is_device_ptr(dst)) return fg::device_pass(src, n, 1, 0, 0.0f, dst);
    return fg::normalize_plane(src, n, dst);
}

FG_API float fg_lambda_from_plane(const float *src, int64_t n, float inv_e_pi_r2, float *dst) {
    if (!src || !dst || n <= 0) return 0.0f;
    if (fg::is_device_ptr(src) || fg::is_device_ptr(dst)) return fg::device_pass(src, n, 1, 1, inv_e_pi_r2, dst);
    return fg::lambda_from_plane(src, n, inv_e_pi_r2, dst);
}

FG_API void fg_lambda_plane(const float *normalized, int64_t n, float inv_e_pi_r2, float *dst) {
    if (!normalized || !dst || n <= 0) return;
    if (fg::is_device_ptr(normalized) || fg::is_device_ptr(dst)) {
        fg::device_pass(normalized, n, 0, 1, inv_e_pi_r2, dst);
        return;
    }
    fg::lambda_plane(normalized, n, inv_e_pi_r2, dst);
}

FG_API fg_status fg_dry_run(int64_t width, int64_t height, const fg_params *params, fg_render_stats *stats) {
    if (!params || !stats) return fg::set_error(FG_ERR_INVALID, "null pointer");
    int64_t w = width, h = height;
    if (params->has_roi) {
        if ((int64_t)params->roi_x1 > width || (int64_t)params->roi_y1 > height)
            return fg::set_error(FG_ERR_INVALID, "ROI exceeds image bounds");
        w = params->roi_x1 - params->roi_x0;
        h = params->roi_y1 - params->roi_y0;
    }
    fg_derived d;
    fg_status st = fg::derive(*params, w, h, &d, nullptr, nullptr);
    if (st != FG_OK) return st;
    fg::fill_stats(*params, d, fg::choose_algorithm(*params, d), stats);
    return FG_OK;
}

FG_API const char *fg_last_error_message(void) { return fg::last_error(); }

FG_API const char *fg_version(void) { return "film_grain_gb300 0.1.0 (sm_103a)"; }

}  // extern "C"

namespace fg {
// make_stats (src/lib.rs:205-222)
void fill_stats(const fg_params &p, const fg_derived &d, int32_t algo, fg_render_stats *s) {
    float mean = std::max(p.radius_mean, 1e-6f);
    s->algorithm = algo;
    s->input_width = d.input_width;
    s->input_height = d.input_height;
    s->output_width = d.output_width;
    s->output_height = d.output_height;
    s->n_samples = p.n_samples;
    s->sigma_ratio = mean > 0.0f ? p.radius_stddev / mean : 0.0f;
    s->rm_ratio = d.rm / mean;
}
}  // namespace fg
