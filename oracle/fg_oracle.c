/*
 * fg_oracle.c -- TEST INFRASTRUCTURE ONLY (the parity checker), never the product.
 *
 * A plain-C CPU restatement of joseph-wardle/film_grain's two Monte Carlo integrators and the
 * host arithmetic around them, written to follow the Rust source's loop order and float
 * expression order exactly (compiled with -ffp-contract=off, no fast-math, so every f32/f64
 * operation rounds as Rust's does).  Only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline may load it.
 *
 * Parity status: UNPINNED against the real Rust crates.  The reference ships no tests, fixtures or
 * golden vectors, and neither cargo nor the crate sources (rand 0.8.5, rand_core 0.6.4,
 * rand_chacha 0.3.1, rand_distr 0.4.3, statrs 0.16.1) exist in this environment, so the
 * third-party algorithms below are restated from their published definitions:
 *   - SplitMix64 finaliser (Steele/Lea/Flood), used by src/rng.rs:46-52 and by rand's
 *     Xoshiro256PlusPlus::seed_from_u64 (reached only through the all-zero-seed remap of from_seed);
 *   - xoshiro256++ (Blackman & Vigna), rand 0.8.5's SmallRng on 64-bit targets; next_u32 takes the
 *     high 32 bits of next_u64;
 *   - rand_core 0.6.4 SeedableRng::seed_from_u64 default (PCG32 output function filling the seed).
 *     rand 0.8.5's SmallRng implements only from_seed and from_rng of SeedableRng, so
 *     SmallRng::seed_from_u64 (src/rng.rs:28,33) is this default: eight PCG32 words written
 *     little-endian into the 32-byte seed, then Xoshiro256PlusPlus::from_seed (four little-endian
 *     u64 words; an all-zero seed is replaced by Xoshiro256PlusPlus::seed_from_u64(0)).  StdRng
 *     (src/rng.rs:15) takes the same eight words as its ChaCha key;
 *   - ChaCha with 12 rounds, 64-bit block counter, stream 0 (rand_chacha 0.3.1 ChaCha12Rng = StdRng);
 *     the ChaCha block function alone IS pinned: tests check it at 20 rounds against OpenSSL's
 *     ChaCha20 keystream (vectors committed under tests/golden/);
 *   - rand 0.8.5 UniformFloat<f32> (23-bit mantissa draw, [1,2) - 1, scale*v + low, scale
 *     shrink loop), Standard f64 (53-bit multiply method), Open01 f64 (52-bit transmute method);
 *   - rand_distr 0.4.3 Poisson (Numerical Recipes: Knuth product for lambda < 12, Cauchy-comparison
 *     rejection otherwise, log_gamma = NR gammln Lanczos g=5 n=6), Cauchy (tan(pi*x)), Normal
 *     (mean + sd*z) with the ZIGNOR 256-layer ziggurat (Marsaglia & Tsang 2000, Doornik 2005;
 *     tables built at run time by the published recursion with r = 3.6541528853610088,
 *     v = 0.00492867323399 and rounded through 18 decimals as the crate's generated table is),
 *     LogNormal (exp of Normal);
 *   - statrs Normal::inverse_cdf: computed here to full double accuracy (only feeds the f32 rm).
 * Platform libm (glibc) supplies logf/exp/log/tan, exactly as Rust's std does on Linux.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------------ integer helpers */
static inline uint64_t o_rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
static inline uint32_t o_rotr32(uint32_t x, uint32_t k) { k &= 31u; return k ? (x >> k) | (x << (32u - k)) : x; }

/* Rust `f as i32` / `f as u32` / `f as isize`: saturating, NaN -> 0. */
static inline int32_t o_f32_to_i32(float f) {
    if (f != f) return 0;
    if (f >= 2147483648.0f) return INT32_MAX;
    if (f <= -2147483648.0f) return INT32_MIN;
    return (int32_t)f;
}
static inline int64_t o_f32_to_i64(float f) {
    if (f != f) return 0;
    if (f >= 9223372036854775808.0f) return INT64_MAX;
    if (f <= -9223372036854775808.0f) return INT64_MIN;
    return (int64_t)f;
}
static inline uint32_t o_f64_to_u32(double d) {
    if (d != d || d <= 0.0) return 0;
    if (d >= 4294967295.0) return UINT32_MAX;
    return (uint32_t)d;
}
/* Rust f32::clamp (NaN passes through). */
static inline float o_clampf(float x, float lo, float hi) { if (x < lo) x = lo; if (x > hi) x = hi; return x; }

/* ------------------------------------------------------------------ src/rng.rs */
#define O_OFFSET_STREAM 0x9E3779B97F4A7C15ull /* src/rng.rs:5 */
#define O_CELL_STREAM 0xA24B1C30BEBCCF59ull   /* src/rng.rs:6 */
#define O_PIXEL_STREAM 0x6935FA5C55F65F1Bull  /* src/rng.rs:7 */

/* src/rng.rs:46-52 */
static uint64_t o_splitmix64(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    uint64_t z = x;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
/* src/rng.rs:36-38 */
static uint64_t o_mix(uint64_t seed, uint64_t stream) { return o_splitmix64(seed ^ stream); }
/* src/rng.rs:40-44 */
static uint64_t o_mix3(uint64_t seed, uint64_t stream, int64_t a, int64_t b) {
    uint64_t state = seed ^ stream;
    state = o_splitmix64(o_rotl64(state + (uint64_t)a, 17));
    return o_splitmix64(o_rotl64(state + (uint64_t)b, 41));
}

/* rand_core 0.6.4 SeedableRng::seed_from_u64 default: the state advances by the PCG32 LCG first,
 * then the XSH-RR output function gives one u32 seed word (written little-endian). */
static void o_pcg32_fill(uint64_t state, uint32_t words[8]) {
    for (int i = 0; i < 8; i++) {
        state = state * 6364136223846793005ull + 11634580027462260723ull;
        uint32_t xorshifted = (uint32_t)(((state >> 18) ^ state) >> 27);
        uint32_t rot = (uint32_t)(state >> 59);
        words[i] = o_rotr32(xorshifted, rot);
    }
}

/* xoshiro256++ (SmallRng, src/rng.rs:26-34 call sites). */
typedef struct { uint64_t s[4]; } o_small_rng;

/* Xoshiro256PlusPlus::seed_from_u64 of rand 0.8.5 (SplitMix64 fill); from_seed sends the all-zero
 * seed here with state 0. */
static o_small_rng o_xoshiro_splitmix_seed(uint64_t state) {
    o_small_rng r;
    for (int i = 0; i < 4; i++) {
        state += 0x9E3779B97F4A7C15ull;
        uint64_t z = state;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        r.s[i] = z ^ (z >> 31);
    }
    return r;
}
/* SmallRng::seed_from_u64 = rand_core's default: PCG32 words -> 32 seed bytes -> from_seed, which
 * reads the bytes as four little-endian u64 (word 2k low, word 2k+1 high). */
static o_small_rng o_small_seed(uint64_t state) {
    uint32_t w[8];
    o_pcg32_fill(state, w);
    o_small_rng r;
    for (int i = 0; i < 4; i++) r.s[i] = (uint64_t)w[2 * i] | ((uint64_t)w[2 * i + 1] << 32);
    if ((r.s[0] | r.s[1] | r.s[2] | r.s[3]) == 0) return o_xoshiro_splitmix_seed(0); /* all-zero seed remap */
    return r;
}
static uint64_t o_small_next_u64(o_small_rng *r) {
    uint64_t *s = r->s;
    uint64_t res = o_rotl64(s[0] + s[3], 23) + s[0];
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = o_rotl64(s[3], 45);
    return res;
}
/* src/rng.rs:26-29 */
static o_small_rng o_cell_rng(uint64_t seed, int32_t i, int32_t j) {
    return o_small_seed(o_mix3(seed, O_CELL_STREAM, (int64_t)i, (int64_t)j));
}
/* src/rng.rs:31-34 */
static o_small_rng o_pixel_rng(uint64_t seed, int32_t i, int32_t j) {
    return o_small_seed(o_mix3(seed, O_PIXEL_STREAM, (int64_t)i, (int64_t)j));
}

/* ChaCha block function (DJB layout: 64-bit counter in words 12-13, 64-bit stream in 14-15). */
#define O_QR(a, b, c, d)                       \
    a += b; d ^= a; d = (d << 16) | (d >> 16); \
    c += d; b ^= c; b = (b << 12) | (b >> 20); \
    a += b; d ^= a; d = (d << 8) | (d >> 24);  \
    c += d; b ^= c; b = (b << 7) | (b >> 25);

static void o_chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream, int rounds, uint32_t out[16]) {
    uint32_t in[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u,
                       key[0], key[1], key[2], key[3], key[4], key[5], key[6], key[7],
                       (uint32_t)counter, (uint32_t)(counter >> 32), (uint32_t)stream, (uint32_t)(stream >> 32)};
    uint32_t x[16];
    memcpy(x, in, sizeof x);
    for (int r = 0; r < rounds; r += 2) {
        O_QR(x[0], x[4], x[8], x[12]) O_QR(x[1], x[5], x[9], x[13])
        O_QR(x[2], x[6], x[10], x[14]) O_QR(x[3], x[7], x[11], x[15])
        O_QR(x[0], x[5], x[10], x[15]) O_QR(x[1], x[6], x[11], x[12])
        O_QR(x[2], x[7], x[8], x[13]) O_QR(x[3], x[4], x[9], x[14])
    }
    for (int i = 0; i < 16; i++) out[i] = x[i] + in[i];
}

/* StdRng = ChaCha12 keystream, consumed as consecutive little-endian u64 pairs. */
typedef struct { uint32_t key[8]; uint64_t block; uint32_t buf[16]; int idx; } o_std_rng;

/* rand_core 0.6.4 default seed_from_u64: PCG32 output words fill the 32-byte seed (the ChaCha key). */
static o_std_rng o_std_seed(uint64_t state) {
    o_std_rng r;
    o_pcg32_fill(state, r.key);
    r.block = 0;
    r.idx = 16;
    return r;
}
static uint64_t o_std_next_u64(o_std_rng *r) {
    if (r->idx >= 16) { o_chacha_block(r->key, r->block++, 0, 12, r->buf); r->idx = 0; }
    uint64_t lo = r->buf[r->idx], hi = r->buf[r->idx + 1];
    r->idx += 2;
    return (hi << 32) | lo;
}

/* ------------------------------------------------------------------ rand / rand_distr samplers */
typedef uint64_t (*o_next_fn)(void *);
static uint64_t o_small_next_v(void *p) { return o_small_next_u64((o_small_rng *)p); }
static uint64_t o_std_next_v(void *p) { return o_std_next_u64((o_std_rng *)p); }

static inline double o_bits_f64(uint64_t b) { double d; memcpy(&d, &b, 8); return d; }
static inline float o_bits_f32(uint32_t b) { float f; memcpy(&f, &b, 4); return f; }
static inline uint32_t o_f32_bits(float f) { uint32_t b; memcpy(&b, &f, 4); return b; }

/* Standard f64: 53 high bits times 2^-53. */
static double o_gen_f64(o_next_fn nx, void *r) {
    uint64_t v = nx(r) >> 11;
    return (1.0 / 9007199254740992.0) * (double)v;
}
/* Open01 f64: 52 high bits into [1,2), minus (1 - eps/2). */
static double o_open01_f64(o_next_fn nx, void *r) {
    uint64_t v = nx(r) >> 12;
    return o_bits_f64(v | 0x3FF0000000000000ull) - (1.0 - 2.220446049250313080847263336181640625e-16 / 2.0);
}

/* UniformFloat<f32>::new */
typedef struct { float low, scale; } o_uniform_f32;
static o_uniform_f32 o_uniform_new(float low, float high) {
    const float max_rand = o_bits_f32(0x3F800000u | (0xFFFFFFFFu >> 9)) - 1.0f;
    float scale = high - low;
    for (;;) {
        float t = scale * max_rand;
        t = t + low;
        if (!(t >= high)) break;
        scale = o_bits_f32(o_f32_bits(scale) - 1u);
    }
    o_uniform_f32 u = {low, scale};
    return u;
}
static float o_uniform_sample(const o_uniform_f32 *u, o_small_rng *r) {
    uint32_t x = (uint32_t)(o_small_next_u64(r) >> 32);
    float v12 = o_bits_f32((x >> 9) | 0x3F800000u);
    float v01 = v12 - 1.0f;
    float t = v01 * u->scale;
    return t + u->low;
}

/* Numerical Recipes gammln (rand_distr::utils::log_gamma). */
static double o_log_gamma(double x) {
    static const double coef[6] = {76.18009172947146, -86.50532032941677, 24.01409824083091,
                                   -1.231739572450155, 0.1208650973866179e-2, -0.5395239384953e-5};
    double tmp = x + 5.5;
    double lg = (x + 0.5) * log(tmp) - tmp;
    double a = 1.000000000190015;
    double denom = x;
    for (int i = 0; i < 6; i++) {
        denom = denom + 1.0;
        a = a + coef[i] / denom;
    }
    return lg + log(2.5066282746310005 * a / x);
}

typedef struct { double lambda, exp_lambda, log_lambda, sqrt_2lambda, magic_val; } o_poisson;
static o_poisson o_poisson_new(double lambda) {
    o_poisson p;
    p.lambda = lambda;
    p.log_lambda = log(lambda);
    p.exp_lambda = exp(-lambda);
    p.sqrt_2lambda = sqrt(2.0 * lambda);
    p.magic_val = lambda * p.log_lambda - o_log_gamma(1.0 + lambda);
    return p;
}
static double o_poisson_sample(const o_poisson *P, o_next_fn nx, void *r) {
    if (P->lambda < 12.0) {
        double result = 1.0;
        double p = o_gen_f64(nx, r);
        while (p > P->exp_lambda) {
            p = p * o_gen_f64(nx, r);
            result = result + 1.0;
        }
        return result - 1.0;
    }
    const double PI = 3.14159265358979323846264338327950288;
    double result, comp_dev;
    for (;;) {
        for (;;) {
            double x = o_gen_f64(nx, r);
            comp_dev = tan(PI * x);
            comp_dev = 0.0 + 1.0 * comp_dev; /* Cauchy(median 0, scale 1) */
            result = P->sqrt_2lambda * comp_dev + P->lambda;
            if (result >= 0.0) break;
        }
        result = floor(result);
        double e = exp(result * P->log_lambda - o_log_gamma(1.0 + result) - P->magic_val);
        double check = 0.9 * (1.0 + comp_dev * comp_dev) * e;
        if (o_gen_f64(nx, r) <= check) break;
    }
    return result;
}

/* Ziggurat tables (257 entries each) rebuilt from the published ZIGNOR recursion. */
static double o_zig_x[257], o_zig_f[257];
static const double O_ZIG_NORM_R = 3.654152885361008796;
static int o_zig_ready = 0;

static double o_round18(double v) {
    char buf[64];
    snprintf(buf, sizeof buf, "%.18f", v);
    return strtod(buf, NULL);
}
static void o_zig_init(void) {
    if (o_zig_ready) return;
    const double r = 3.6541528853610088, v = 0.00492867323399;
    double xs[257], fs[257];
    for (int i = 0; i < 257; i++) xs[i] = 0.0;
    xs[0] = v / exp(-r * r / 2.0);
    xs[1] = r;
    for (int i = 2; i < 256; i++) {
        double last = xs[i - 1];
        double y = v / last + exp(-last * last / 2.0);
        xs[i] = sqrt(-2.0 * log(y));
    }
    for (int i = 0; i < 257; i++) fs[i] = exp(-xs[i] * xs[i] / 2.0);
    for (int i = 0; i < 257; i++) { o_zig_x[i] = o_round18(xs[i]); o_zig_f[i] = o_round18(fs[i]); }
    o_zig_ready = 1;
}

static double o_std_normal(o_next_fn nx, void *r) {
    for (;;) {
        uint64_t bits = nx(r);
        unsigned i = (unsigned)(bits & 0xff);
        double u = o_bits_f64((bits >> 12) | ((uint64_t)(1023 + 1) << 52)) - 3.0;
        double x = u * o_zig_x[i];
        double test_x = fabs(x);
        if (test_x < o_zig_x[i + 1]) return x;
        if (i == 0) {
            double xx = 1.0, yy = 0.0;
            while (-2.0 * yy < xx * xx) {
                double x_ = o_open01_f64(nx, r);
                double y_ = o_open01_f64(nx, r);
                xx = log(x_) / O_ZIG_NORM_R;
                yy = log(y_);
            }
            return (u < 0.0) ? xx - O_ZIG_NORM_R : O_ZIG_NORM_R - xx;
        }
        double pdf = exp(-x * x / 2.0);
        if (o_zig_f[i + 1] + (o_zig_f[i] - o_zig_f[i + 1]) * o_gen_f64(nx, r) < pdf) return x;
    }
}
static double o_normal(double mean, double sd, o_next_fn nx, void *r) {
    return mean + sd * o_std_normal(nx, r);
}

/* ------------------------------------------------------------------ params / model */
/* Mirrors of the resolved Params and Derived fields the integrators read. */
typedef struct {
    int32_t radius_dist; /* 0 = Const, 1 = Lognorm */
    float radius_mean, radius_stddev, radius_log_mu, radius_log_sigma;
    float zoom, sigma_px;
    uint32_t n_samples;
    uint64_t seed;
} o_params;

typedef struct {
    int64_t in_w, in_h, out_w, out_h;
    float inv_e_pi_r2, rm, delta;
} o_derived;

/* RadiusProfile::sample (src/model.rs:137-148) */
static inline float o_radius_sample(const o_params *p, o_small_rng *r) {
    if (p->radius_dist == 0) return p->radius_mean;
    double v = o_normal((double)p->radius_log_mu, (double)p->radius_log_sigma, o_small_next_v, r);
    return (float)exp(v);
}

/* src/rng.rs:9-24 */
ORC_EXPORT void orc_make_offsets(uint64_t seed, uint32_t n, float sigma, float *out_xy) {
    o_zig_init();
    if (n == 0) return;
    float s = sigma > 1.1920928955078125e-07f ? sigma : 1.1920928955078125e-07f;
    double sd = (double)s;
    o_std_rng r = o_std_seed(o_mix(seed, O_OFFSET_STREAM));
    for (uint32_t k = 0; k < n; k++) {
        out_xy[2 * k] = (float)o_normal(0.0, sd, o_std_next_v, &r);
        out_xy[2 * k + 1] = (float)o_normal(0.0, sd, o_std_next_v, &r);
    }
}

/* Inverse standard normal CDF to full double accuracy: Acklam's rational start, then Halley
 * steps on erfc.  Feeds only the f32 max radius, as statrs' inverse_cdf does in the reference. */
static double o_norm_inv(double p) {
    static const double a[6] = {-3.969683028665376e+01, 2.209460984245205e+02, -2.759285104469687e+02,
                                1.383577518672690e+02, -3.066479806614716e+01, 2.506628277459239e+00};
    static const double b[5] = {-5.447609879822406e+01, 1.615858368580409e+02, -1.556989798598866e+02,
                                6.680131188771972e+01, -1.328068155288572e+01};
    static const double c[6] = {-7.784894002430293e-03, -3.223964580411365e-01, -2.400758277161838e+00,
                                -2.549732539343734e+00, 4.374664141464968e+00, 2.938163982698783e+00};
    static const double d[4] = {7.784695709041462e-03, 3.224671290700398e-01, 2.445134137142996e+00,
                                3.754408661907416e+00};
    double q, x;
    if (p < 0.02425) {
        q = sqrt(-2 * log(p));
        x = (((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
            ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1);
    } else if (p > 1 - 0.02425) {
        q = sqrt(-2 * log(1 - p));
        x = -(((((c[0] * q + c[1]) * q + c[2]) * q + c[3]) * q + c[4]) * q + c[5]) /
            ((((d[0] * q + d[1]) * q + d[2]) * q + d[3]) * q + 1);
    } else {
        q = p - 0.5;
        double rr = q * q;
        x = (((((a[0] * rr + a[1]) * rr + a[2]) * rr + a[3]) * rr + a[4]) * rr + a[5]) * q /
            (((((b[0] * rr + b[1]) * rr + b[2]) * rr + b[3]) * rr + b[4]) * rr + 1);
    }
    for (int it = 0; it < 3; it++) {
        double e = 0.5 * erfc(-x / 1.4142135623730951) - p;
        double u = e * 2.5066282746310002 * exp(x * x / 2);
        x = x - u / (1 + x * u / 2);
    }
    return x;
}

/* RadiusProfile::quantile (src/model.rs:150-164) */
ORC_EXPORT float orc_radius_quantile(const o_params *p, float prob) {
    if (p->radius_dist == 0) return p->radius_mean;
    double mu = (double)p->radius_log_mu, sigma = (double)p->radius_log_sigma;
    if (sigma == 0.0) return (float)exp(mu);
    double z = o_norm_inv((double)prob);
    return (float)exp(mu + sigma * z);
}

/* params.rs:223-253 -> (stddev, log_mu, log_sigma) */
ORC_EXPORT void orc_lognormal_params(float mean, float sd, float out[3]) {
    if (sd == 0.0f) { out[0] = 0.0f; out[1] = logf(mean); out[2] = 0.0f; return; }
    float vr = (sd * sd) / (mean * mean);
    float sigma_sq = logf(1.0f + vr);
    float sigma = sqrtf(sigma_sq);
    float mu = logf(mean) - 0.5f * sigma_sq;
    out[0] = sd; out[1] = mu; out[2] = sigma;
}

/* params.rs:255-261 */
ORC_EXPORT float orc_default_cell_delta(float mean) {
    if (mean <= 0.0f) return 1.0f;
    float inv = ceilf(1.0f / mean);
    if (inv < 1.0f) inv = 1.0f;
    return 1.0f / inv;
}

/* derive_common's scalar part (src/model.rs:181-226): inv_e_pi_r2, rm, delta and the output size.
 * max_radius_kind 0 = Absolute(v), 1 = Quantile(v); cell_delta <= 0 means "default". */
ORC_EXPORT int orc_derive(const o_params *p, int64_t in_w, int64_t in_h, int32_t max_radius_kind,
                          float max_radius_value, float cell_delta, int64_t size_w, int64_t size_h,
                          o_derived *d) {
    if (in_w <= 0 || in_h <= 0) return -1;
    d->in_w = in_w; d->in_h = in_h;
    if (size_w > 0) {
        d->out_w = size_w;
        if (size_h > 0) d->out_h = size_h;
        else {
            float aspect = (float)in_h / (float)in_w;
            float c = roundf((float)size_w * aspect);
            if (c < 1.0f) c = 1.0f;
            d->out_h = (int64_t)c;
        }
    } else {
        float w = ceilf((float)in_w * p->zoom); if (w < 1.0f) w = 1.0f;
        float h = ceilf((float)in_h * p->zoom); if (h < 1.0f) h = 1.0f;
        d->out_w = (int64_t)w; d->out_h = (int64_t)h;
    }
    const float EPS = 1e-6f;
    const float PI = 3.14159265358979323846f;
    float mean_sq = p->radius_mean * p->radius_mean;
    float var = p->radius_stddev * p->radius_stddev;
    float ms = mean_sq + var; if (ms < EPS) ms = EPS;
    d->inv_e_pi_r2 = 1.0f / (PI * ms);
    float rm = (max_radius_kind == 0) ? max_radius_value : orc_radius_quantile(p, max_radius_value);
    d->rm = rm > EPS ? rm : EPS;
    float delta = cell_delta > 0.0f ? cell_delta : orc_default_cell_delta(p->radius_mean);
    d->delta = delta > EPS ? delta : EPS;
    return 0;
}

/* normalize_plane + lambda_plane (src/model.rs:228-265) */
ORC_EXPORT float orc_normalize_plane(const float *src, int64_t n, float *dst) {
    const float EPS = 1e-6f;
    float mx = 0.0f;
    for (int64_t i = 0; i < n; i++) mx = fmaxf(mx, src[i]);
    int already = mx <= 1.0f + EPS;
    for (int64_t i = 0; i < n; i++) {
        float v;
        if (already) v = src[i];
        else {
            float den = mx + EPS; if (den < EPS) den = EPS;
            v = src[i] / den;
        }
        dst[i] = o_clampf(v, 0.0f, 1.0f - EPS);
    }
    return mx;
}
ORC_EXPORT void orc_lambda_plane(const float *norm, int64_t n, float inv_e_pi_r2, float *dst) {
    const float EPS = 1e-6f;
    for (int64_t i = 0; i < n; i++) {
        float c = o_clampf(norm[i], 0.0f, 1.0f - EPS);
        float safe = fmaxf(1.0f - c, EPS);
        float act = -inv_e_pi_r2 * logf(safe);
        dst[i] = fminf(act, 1.0e6f);
    }
}

/* choose.rs:4-26 ; algo 0 = Auto, 1 = Grain, 2 = Pixel */
ORC_EXPORT int orc_choose_algorithm(const o_params *p, int32_t algo, float rm) {
    if (algo != 0) return algo;
    float mean = fmaxf(p->radius_mean, 1e-6f);
    float sr = mean > 0.0f ? p->radius_stddev / mean : 0.0f;
    float rr = rm / mean;
    if (sr < 0.1f && mean < 0.5f && p->n_samples <= 64) return 2;
    if (rr > 8.0f || sr > 0.6f || p->n_samples > 96) return 1;
    if (p->n_samples <= 24 && rr < 5.0f) return 2;
    return 1;
}

/* ------------------------------------------------------------------ pixel-wise (src/pixelwise.rs) */
static inline float o_get_clamped(const float *lam, int64_t w, int64_t h, int64_t x, int64_t y) {
    if (w <= 0 || h <= 0) return 0.0f;
    if (x < 0) x = 0;
    if (x > w - 1) x = w - 1;
    if (y < 0) y = 0;
    if (y > h - 1) y = h - 1;
    return lam[y * w + x];
}

/* evaluate_indicator (src/pixelwise.rs:47-106) */
static float o_evaluate_indicator(float xg, float yg, const float *lam, const o_params *p, const o_derived *d) {
    float rm = d->rm, delta = d->delta;
    if (rm <= 0.0f) return 0.0f;
    int32_t i0 = o_f32_to_i32(floorf((xg - rm) / delta));
    int32_t i1 = o_f32_to_i32(floorf((xg + rm) / delta));
    int32_t j0 = o_f32_to_i32(floorf((yg - rm) / delta));
    int32_t j1 = o_f32_to_i32(floorf((yg + rm) / delta));
    if (i0 > i1 || j0 > j1) return 0.0f;
    o_uniform_f32 uni = o_uniform_new(0.0f, delta);
    for (int32_t i = i0; i <= i1; i++) {
        for (int32_t j = j0; j <= j1; j++) {
            o_small_rng rng = o_cell_rng(p->seed, i, j);
            float sx = (float)i * delta;
            float sy = (float)j * delta;
            int64_t ix = o_f32_to_i64(floorf(sx));
            int64_t iy = o_f32_to_i64(floorf(sy));
            float lc = o_get_clamped(lam, d->in_w, d->in_h, ix, iy);
            if (lc <= 0.0f) continue;
            float expected = lc * delta * delta;
            if (expected <= 0.0f) continue;
            o_poisson P = o_poisson_new((double)expected);
            uint32_t q = o_f64_to_u32(o_poisson_sample(&P, o_small_next_v, &rng));
            if (q == 0) continue;
            for (uint32_t g = 0; g < q; g++) {
                float cx = sx + o_uniform_sample(&uni, &rng);
                float cy = sy + o_uniform_sample(&uni, &rng);
                float radius = o_radius_sample(p, &rng);
                if (radius > d->rm) radius = d->rm;
                if (radius <= 0.0f) continue;
                float dx = xg - cx, dy = yg - cy;
                float a = dx * dx, b = dy * dy, rr = radius * radius;
                if (a + b <= rr) return 1.0f;
            }
        }
    }
    return 0.0f;
}

/* render_pixelwise over the output rectangle [ox0,ox1) x [oy0,oy1) (the whole plane when it is
 * [0,out_w) x [0,out_h)); out has (ox1-ox0)*(oy1-oy0) floats, counts (optional) the raw hit counts. */
ORC_EXPORT int orc_render_pixelwise(const float *lam, const o_params *p, const o_derived *d, const float *offsets_input,
                                    int64_t ox0, int64_t oy0, int64_t ox1, int64_t oy1, float *out, uint32_t *counts,
                                    int32_t threads) {
    o_zig_init();
    uint32_t n = p->n_samples > 0 ? p->n_samples : 1;
    float inv_samples = 1.0f / (float)n;
    float inv_zoom = 1.0f / p->zoom;
    int64_t rw = ox1 - ox0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t y = oy0; y < oy1; y++) {
        for (int64_t x = ox0; x < ox1; x++) {
            float sum = 0.0f;
            for (uint32_t k = 0; k < p->n_samples; k++) {
                float xg = (((float)x + 0.5f) * inv_zoom) - offsets_input[2 * k];
                float yg = (((float)y + 0.5f) * inv_zoom) - offsets_input[2 * k + 1];
                sum += o_evaluate_indicator(xg, yg, lam, p, d);
            }
            out[(y - oy0) * rw + (x - ox0)] = sum * inv_samples;
            if (counts) counts[(y - oy0) * rw + (x - ox0)] = (uint32_t)sum;
        }
    }
    return 0;
}

/* ------------------------------------------------------------------ grain-wise (src/grainwise.rs) */
/* bounds (src/grainwise.rs:126-142); returns 0 when None. */
static inline int o_bounds(float center, float radius, int32_t limit, int32_t *mn, int32_t *mx) {
    int32_t lo = o_f32_to_i32(ceilf((center - radius) - 0.5f));
    int32_t hi = o_f32_to_i32(floorf((center + radius) - 0.5f));
    if (hi < lo) return 0;
    if (limit <= 0) return 0;
    int32_t last = limit - 1;
    if (lo > last || hi < 0) return 0;
    if (lo < 0) lo = 0;
    if (lo > last) lo = last;
    if (hi < 0) hi = 0;
    if (hi > last) hi = last;
    if (lo > hi) return 0;
    *mn = lo; *mx = hi;
    return 1;
}

/* render_grainwise restricted to the output rectangle [ox0,ox1) x [oy0,oy1): grains from every input
 * pixel whose splats can reach the rectangle are rasterised with the reference's exact arithmetic; bits
 * outside the rectangle are dropped (they belong to other pixels). The whole plane is the rectangle
 * [0,out_w) x [0,out_h). */
ORC_EXPORT int orc_render_grainwise(const float *lam, const o_params *p, const o_derived *d, const float *offsets,
                                    int64_t ox0, int64_t oy0, int64_t ox1, int64_t oy1, float *out, uint32_t *counts,
                                    int32_t threads) {
    o_zig_init();
    uint32_t n = p->n_samples;
    int64_t out_w = d->out_w, out_h = d->out_h;
    int64_t rw = ox1 - ox0, rh = oy1 - oy0;
    int64_t lanes = ((int64_t)n + 63) / 64;
    uint64_t *bits = (uint64_t *)calloc((size_t)(rw * rh * lanes > 0 ? rw * rh * lanes : 1), sizeof(uint64_t));
    if (!bits) return -2;
    float zoom = p->zoom;
    float inv_samples = 1.0f / (float)(n > 0 ? n : 1);
    /* input rows/cols that can reach the rectangle */
    float mnx = 0, mxx = 0, mny = 0, mxy = 0;
    for (uint32_t k = 0; k < n; k++) {
        mnx = fminf(mnx, offsets[2 * k]); mxx = fmaxf(mxx, offsets[2 * k]);
        mny = fminf(mny, offsets[2 * k + 1]); mxy = fmaxf(mxy, offsets[2 * k + 1]);
    }
    float reach = d->rm * zoom + 2.0f;
    int64_t ix0 = (int64_t)floorf(((float)ox0 - mxx - reach) / zoom) - 1;
    int64_t ix1 = (int64_t)ceilf(((float)ox1 - mnx + reach) / zoom) + 1;
    int64_t iy0 = (int64_t)floorf(((float)oy0 - mxy - reach) / zoom) - 1;
    int64_t iy1 = (int64_t)ceilf(((float)oy1 - mny + reach) / zoom) + 1;
    if (ix0 < 0) ix0 = 0;
    if (iy0 < 0) iy0 = 0;
    if (ix1 > d->in_w) ix1 = d->in_w;
    if (iy1 > d->in_h) iy1 = d->in_h;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
    o_uniform_f32 uni = o_uniform_new(0.0f, 1.0f);
#pragma omp parallel for schedule(dynamic, 1)
    for (int64_t y = iy0; y < iy1; y++) {
        for (int64_t x = ix0; x < ix1; x++) {
            float lv = lam[y * d->in_w + x];
            if (lv <= 0.0f) continue;
            o_small_rng rng = o_pixel_rng(p->seed, (int32_t)x, (int32_t)y);
            o_poisson P = o_poisson_new((double)lv);
            uint32_t q = o_f64_to_u32(o_poisson_sample(&P, o_small_next_v, &rng));
            for (uint32_t g = 0; g < q; g++) {
                float cx = (float)x + o_uniform_sample(&uni, &rng);
                float cy = (float)y + o_uniform_sample(&uni, &rng);
                float radius = o_radius_sample(p, &rng);
                if (radius > d->rm) radius = d->rm;
                if (radius <= 0.0f) continue;
                float ro = radius * zoom;
                if (ro <= 0.0f) continue;
                float rsq = ro * ro;
                for (uint32_t k = 0; k < n; k++) {
                    float tx = (cx * zoom) + offsets[2 * k];
                    float ty = (cy * zoom) + offsets[2 * k + 1];
                    int32_t xa, xb, ya, yb;
                    if (!o_bounds(tx, ro, (int32_t)out_w, &xa, &xb)) continue;
                    if (!o_bounds(ty, ro, (int32_t)out_h, &ya, &yb)) continue;
                    int64_t lane = k / 64;
                    uint64_t bm = 1ull << (k % 64);
                    for (int32_t oy = ya; oy <= yb; oy++) {
                        float cyp = (float)oy + 0.5f;
                        float dy = cyp - ty;
                        float dysq = dy * dy;
                        if (dysq > rsq) continue;
                        if (oy < oy0 || oy >= oy1) continue;
                        for (int32_t ox = xa; ox <= xb; ox++) {
                            float cxp = (float)ox + 0.5f;
                            float dx = cxp - tx;
                            float dd = dx * dx;
                            if (dd + dysq <= rsq) {
                                if (ox < ox0 || ox >= ox1) continue;
                                int64_t idx = (oy - oy0) * rw + (ox - ox0);
                                __atomic_fetch_or(&bits[idx * lanes + lane], bm, __ATOMIC_RELAXED);
                            }
                        }
                    }
                }
            }
        }
    }
    for (int64_t i = 0; i < rw * rh; i++) {
        uint32_t c = 0;
        for (int64_t l = 0; l < lanes; l++) c += (uint32_t)__builtin_popcountll(bits[i * lanes + l]);
        out[i] = (float)c * inv_samples;
        if (counts) counts[i] = c;
    }
    free(bits);
    return 0;
}

/* ------------------------------------------------------------------ colour (src/color.rs) */
#define O_YR 0.2126f
#define O_YG 0.7152f
#define O_YB 0.0722f
#define O_CBD 1.8556f
#define O_CRD 1.5748f
static inline float o_clamp01(float v) { return o_clampf(v, 0.0f, 1.0f); }
static inline uint8_t o_to_u8(float v) { return (uint8_t)o_f32_to_i32(floorf(o_clamp01(v) * 255.0f + 0.5f)); }

/* load_luma_workspace (src/color.rs:181-213) from interleaved f32 RGB */
ORC_EXPORT void orc_luma_split(const float *rgb, int64_t n, float *y, float *cb, float *cr) {
    for (int64_t i = 0; i < n; i++) {
        float r = o_clamp01(rgb[3 * i]), g = o_clamp01(rgb[3 * i + 1]), b = o_clamp01(rgb[3 * i + 2]);
        float l = O_YR * r + O_YG * g + O_YB * b;
        cb[i] = (b - l) / O_CBD;
        cr[i] = (r - l) / O_CRD;
        y[i] = o_clamp01(l);
    }
}
/* load_rgb_workspace (src/color.rs:158-179) */
ORC_EXPORT void orc_rgb_split(const float *rgb, int64_t n, float *p0, float *p1, float *p2) {
    for (int64_t i = 0; i < n; i++) {
        p0[i] = o_clamp01(rgb[3 * i]); p1[i] = o_clamp01(rgb[3 * i + 1]); p2[i] = o_clamp01(rgb[3 * i + 2]);
    }
}
/* Plane::resize_nearest (src/model.rs:72-99) */
ORC_EXPORT void orc_resize_nearest(const float *src, int64_t w, int64_t h, int64_t nw, int64_t nh, float *dst) {
    if (nw == w && nh == h) { memcpy(dst, src, sizeof(float) * (size_t)(w * h)); return; }
    if (nw == 0 || nh == 0 || w == 0 || h == 0) { memset(dst, 0, sizeof(float) * (size_t)(nw * nh)); return; }
    float sxs = (float)w / (float)nw, sys = (float)h / (float)nh;
    for (int64_t y = 0; y < nh; y++) {
        float syf = o_clampf(((float)y + 0.5f) * sys - 0.5f, 0.0f, (float)(h - 1));
        int64_t sy = (int64_t)roundf(syf);
        for (int64_t x = 0; x < nw; x++) {
            float sxf = o_clampf(((float)x + 0.5f) * sxs - 0.5f, 0.0f, (float)(w - 1));
            int64_t sx = (int64_t)roundf(sxf);
            dst[y * nw + x] = src[sy * w + sx];
        }
    }
}
/* into_rgb_image, Luma arm (src/color.rs:66-100); cb/cr already at the output size */
ORC_EXPORT void orc_luma_to_rgb8(const float *y, const float *cb, const float *cr, int64_t n, uint8_t *out) {
    for (int64_t i = 0; i < n; i++) {
        float yv = y[i];
        float r = o_clamp01(yv + O_CRD * cr[i]);
        float b = o_clamp01(yv + O_CBD * cb[i]);
        float gu = (yv - O_YR * r - O_YB * b) / O_YG;
        float g = o_clamp01(gu);
        out[3 * i] = o_to_u8(r); out[3 * i + 1] = o_to_u8(g); out[3 * i + 2] = o_to_u8(b);
    }
}
/* into_rgb_image, Rgb arm (src/color.rs:101-113) */
ORC_EXPORT void orc_planes_to_rgb8(const float *p0, const float *p1, const float *p2, int64_t n, uint8_t *out) {
    for (int64_t i = 0; i < n; i++) { out[3 * i] = o_to_u8(p0[i]); out[3 * i + 1] = o_to_u8(p1[i]); out[3 * i + 2] = o_to_u8(p2[i]); }
}

/* ------------------------------------------------------------------ probes for the RNG tests */
ORC_EXPORT uint64_t orc_splitmix64(uint64_t x) { return o_splitmix64(x); }
ORC_EXPORT uint64_t orc_mix3(uint64_t seed, uint64_t stream, int64_t a, int64_t b) { return o_mix3(seed, stream, a, b); }
ORC_EXPORT void orc_small_stream(uint64_t seed_u64, int64_t n, uint64_t *out) {
    o_small_rng r = o_small_seed(seed_u64);
    for (int64_t i = 0; i < n; i++) out[i] = o_small_next_u64(&r);
}
ORC_EXPORT void orc_cell_stream(uint64_t seed, int32_t i, int32_t j, int32_t pixel_stream, int64_t n, uint64_t *out) {
    o_small_rng r = pixel_stream ? o_pixel_rng(seed, i, j) : o_cell_rng(seed, i, j);
    for (int64_t k = 0; k < n; k++) out[k] = o_small_next_u64(&r);
}
ORC_EXPORT void orc_chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream, int32_t rounds, uint32_t out[16]) {
    o_chacha_block(key, counter, stream, rounds, out);
}
ORC_EXPORT void orc_std_stream(uint64_t seed_u64, int64_t n, uint64_t *out) {
    o_std_rng r = o_std_seed(seed_u64);
    for (int64_t i = 0; i < n; i++) out[i] = o_std_next_u64(&r);
}
ORC_EXPORT void orc_std_key(uint64_t seed_u64, uint32_t key[8]) {
    o_std_rng r = o_std_seed(seed_u64);
    memcpy(key, r.key, sizeof r.key);
}
ORC_EXPORT void orc_zig_tables(double *x, double *f) {
    o_zig_init();
    memcpy(x, o_zig_x, sizeof o_zig_x);
    memcpy(f, o_zig_f, sizeof o_zig_f);
}
/* n Poisson(lambda) draws from the SmallRng seeded by seed_u64 */
ORC_EXPORT void orc_poisson_draws(double lambda, uint64_t seed_u64, int64_t n, double *out) {
    o_small_rng r = o_small_seed(seed_u64);
    o_poisson P = o_poisson_new(lambda);
    for (int64_t i = 0; i < n; i++) out[i] = o_poisson_sample(&P, o_small_next_v, &r);
}
ORC_EXPORT void orc_normal_draws(double mean, double sd, uint64_t seed_u64, int64_t n, double *out) {
    o_zig_init();
    o_small_rng r = o_small_seed(seed_u64);
    for (int64_t i = 0; i < n; i++) out[i] = o_normal(mean, sd, o_small_next_v, &r);
}
ORC_EXPORT void orc_uniform_f32_draws(float low, float high, uint64_t seed_u64, int64_t n, float *out) {
    o_small_rng r = o_small_seed(seed_u64);
    o_uniform_f32 u = o_uniform_new(low, high);
    for (int64_t i = 0; i < n; i++) out[i] = o_uniform_sample(&u, &r);
}
ORC_EXPORT double orc_log_gamma(double x) { return o_log_gamma(x); }
/* The platform libm's f64 exp / log / tan (what the crate's samplers call) over an array: which = 0 exp,
 * 1 log, 2 tan. */
ORC_EXPORT void orc_libm_f64(int32_t which, const double *x, int64_t n, double *out) {
    for (int64_t i = 0; i < n; i++) out[i] = which == 0 ? exp(x[i]) : (which == 1 ? log(x[i]) : tan(x[i]));
}
ORC_EXPORT int32_t orc_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------ bench support (grain-wise work accounting) */
/* Sum of the Poisson grain counts of input rows [iy0, iy1) (the draw of src/grainwise.rs:41-43). */
ORC_EXPORT uint64_t orc_grain_total(const float *lam, const o_params *p, const o_derived *d, int64_t iy0, int64_t iy1,
                                    int32_t threads) {
    uint64_t total = 0;
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
    for (int64_t y = iy0; y < iy1; y++) {
        for (int64_t x = 0; x < d->in_w; x++) {
            float lv = lam[y * d->in_w + x];
            if (lv <= 0.0f) continue;
            o_small_rng rng = o_pixel_rng(p->seed, (int32_t)x, (int32_t)y);
            o_poisson P = o_poisson_new((double)lv);
            total += o_f64_to_u32(o_poisson_sample(&P, o_small_next_v, &rng));
        }
    }
    return total;
}

/* The reference's grain-wise work for input rows [iy0, iy1) over the whole output plane, exactly as
 * src/grainwise.rs:29-107 does it (rayon's decomposition: rows of the input).  bits: out_w*out_h*lanes
 * u64, zeroed by the caller.  With count != 0 it also tallies, over all (grain, offset) pairs,
 * stats[0] grains, [1] pairs whose x bounds are Some, [2] pairs whose x and y bounds are Some,
 * [3] centre tests passed (bits set). */
ORC_EXPORT int orc_grainwise_rows(const float *lam, const o_params *p, const o_derived *d, const float *offsets,
                                  int64_t iy0, int64_t iy1, uint64_t *bits, int32_t count, uint64_t stats[4],
                                  int32_t threads) {
    o_zig_init();
    uint32_t n = p->n_samples;
    int64_t out_w = d->out_w, out_h = d->out_h;
    int64_t lanes = ((int64_t)n + 63) / 64;
    float zoom = p->zoom;
    uint64_t g_tot = 0, px_tot = 0, py_tot = 0, h_tot = 0;
    o_uniform_f32 uni = o_uniform_new(0.0f, 1.0f);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#endif
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : g_tot, px_tot, py_tot, h_tot)
    for (int64_t y = iy0; y < iy1; y++) {
        for (int64_t x = 0; x < d->in_w; x++) {
            float lv = lam[y * d->in_w + x];
            if (lv <= 0.0f) continue;
            o_small_rng rng = o_pixel_rng(p->seed, (int32_t)x, (int32_t)y);
            o_poisson P = o_poisson_new((double)lv);
            uint32_t q = o_f64_to_u32(o_poisson_sample(&P, o_small_next_v, &rng));
            for (uint32_t g = 0; g < q; g++) {
                float cx = (float)x + o_uniform_sample(&uni, &rng);
                float cy = (float)y + o_uniform_sample(&uni, &rng);
                float radius = o_radius_sample(p, &rng);
                if (radius > d->rm) radius = d->rm;
                if (radius <= 0.0f) continue;
                float ro = radius * zoom;
                if (ro <= 0.0f) continue;
                float rsq = ro * ro;
                g_tot++;
                for (uint32_t k = 0; k < n; k++) {
                    float tx = (cx * zoom) + offsets[2 * k];
                    float ty = (cy * zoom) + offsets[2 * k + 1];
                    int32_t xa, xb, ya, yb;
                    if (!o_bounds(tx, ro, (int32_t)out_w, &xa, &xb)) continue;
                    px_tot++;
                    if (!o_bounds(ty, ro, (int32_t)out_h, &ya, &yb)) continue;
                    py_tot++;
                    int64_t lane = k / 64;
                    uint64_t bm = 1ull << (k % 64);
                    for (int32_t oy = ya; oy <= yb; oy++) {
                        float dy = ((float)oy + 0.5f) - ty;
                        float dysq = dy * dy;
                        if (dysq > rsq) continue;
                        for (int32_t ox = xa; ox <= xb; ox++) {
                            float dx = ((float)ox + 0.5f) - tx;
                            if (dx * dx + dysq <= rsq) {
                                h_tot++;
                                __atomic_fetch_or(&bits[((int64_t)oy * out_w + ox) * lanes + lane], bm, __ATOMIC_RELAXED);
                            }
                        }
                    }
                }
            }
        }
    }
    if (stats) { stats[0] = g_tot; stats[1] = count ? px_tot : 0; stats[2] = count ? py_tot : 0; stats[3] = count ? h_tot : 0; }
    return 0;
}
