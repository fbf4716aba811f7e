// fg_rng.cuh -- the film_grain RNG streams and samplers, bit-identical on host and device.
//
// Restates src/rng.rs:1-52 and the third-party samplers it calls:
//   rand 0.8.5     SmallRng = xoshiro256++; next_u32 = high half of next_u64; UniformFloat<f32>
//                  (23-bit mantissa draw); Standard f64 (53-bit multiply method); Open01 f64 (52-bit
//                  transmute method).
//   rand_core 0.6.4  SeedableRng::seed_from_u64 default (PCG32 output words fill the seed).  Both
//                  SmallRng::seed_from_u64 (src/rng.rs:28,33; rand 0.8.5's SmallRng implements only
//                  from_seed and from_rng, so the default applies) and StdRng::seed_from_u64 in
//                  make_offsets (src/rng.rs:15) take it.
//   rand_chacha    ChaCha12Rng = StdRng: ChaCha block function, 12 rounds, 64-bit counter, stream 0.
//   rand_distr 0.4.3  Poisson (Knuth product below lambda 12, Cauchy-comparison rejection above,
//                  Numerical Recipes' log-gamma), Normal via the 256-layer ziggurat, LogNormal.
// Every floating-point operation on the coverage path is an explicit round-to-nearest intrinsic on
// the device (no FMA contraction), matching Rust's unfused expression order.
#pragma once
#include <stdint.h>
#include <math.h>
#include "zig_tables.h"

#if defined(__CUDACC__)
#define FG_HD __host__ __device__ __forceinline__
#define FG_HDC __host__ __device__ constexpr
#else
#define FG_HD inline
#define FG_HDC constexpr
#endif

#ifdef __CUDA_ARCH__
#define FG_FMUL(a, b) __fmul_rn((a), (b))
#define FG_FADD(a, b) __fadd_rn((a), (b))
#define FG_FSUB(a, b) __fsub_rn((a), (b))
#define FG_FDIV(a, b) __fdiv_rn((a), (b))
#define FG_DMUL(a, b) __dmul_rn((a), (b))
#define FG_DADD(a, b) __dadd_rn((a), (b))
#define FG_DSUB(a, b) __dsub_rn((a), (b))
#define FG_DDIV(a, b) __ddiv_rn((a), (b))
#else
#define FG_FMUL(a, b) ((float)(a) * (float)(b))
#define FG_FADD(a, b) ((float)(a) + (float)(b))
#define FG_FSUB(a, b) ((float)(a) - (float)(b))
#define FG_FDIV(a, b) ((float)(a) / (float)(b))
#define FG_DMUL(a, b) ((double)(a) * (double)(b))
#define FG_DADD(a, b) ((double)(a) + (double)(b))
#define FG_DSUB(a, b) ((double)(a) - (double)(b))
#define FG_DDIV(a, b) ((double)(a) / (double)(b))
#endif

namespace fg {

constexpr uint64_t kPhi = 0x9E3779B97F4A7C15ull;
constexpr uint64_t kOffsetStream = 0x9E3779B97F4A7C15ull;  // src/rng.rs:5
constexpr uint64_t kCellStream = 0xA24B1C30BEBCCF59ull;    // src/rng.rs:6
constexpr uint64_t kPixelStream = 0x6935FA5C55F65F1Bull;   // src/rng.rs:7

FG_HD uint64_t rotl64(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

// The SplitMix64 output function.
FG_HD uint64_t fmix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// src/rng.rs:46-52
FG_HD uint64_t splitmix64(uint64_t x) { return fmix64(x + kPhi); }
// src/rng.rs:40-44 (i64 -> u64 reinterpretation, wrapping adds, rotations 17 and 41)
FG_HD uint64_t mix3(uint64_t seed, uint64_t stream, int64_t a, int64_t b) {
    uint64_t st = seed ^ stream;
    st = splitmix64(rotl64(st + (uint64_t)a, 17));
    return splitmix64(rotl64(st + (uint64_t)b, 41));
}

// xoshiro256++ (rand 0.8.5 SmallRng on 64-bit targets).
struct Xoshiro {
    uint64_t s0, s1, s2, s3;
    FG_HD uint64_t next() {
        uint64_t r = rotl64(s0 + s3, 23) + s0;
        uint64_t t = s1 << 17;
        s2 ^= s0;
        s3 ^= s1;
        s1 ^= s2;
        s0 ^= s3;
        s2 ^= t;
        s3 = rotl64(s3, 45);
        return r;
    }
};
// ---- SmallRng::seed_from_u64 (rand_core 0.6.4's default, which rand 0.8.5's SmallRng keeps)
// The PCG32 LCG advances the state before each output; the XSH-RR output function turns state k
// (k = 1..8) into seed word k; the eight words fill the 32-byte seed little-endian, and
// Xoshiro256PlusPlus::from_seed reads it as four little-endian u64: s0 = w1 | w2 << 32, s1 = w3 | w4 << 32,
// s2 = w5 | w6 << 32, s3 = w7 | w8 << 32.  An all-zero seed is replaced by
// Xoshiro256PlusPlus::seed_from_u64(0) (SplitMix64 words fmix64(k * phi), k = 1..4).
// State k is a jump-ahead of the input: M^k * h + I * (M^(k-1) + ... + M + 1) (mod 2^64), so the
// words do not depend on each other and the emptiness tests compute only words 1, 2, 7 and 8.
constexpr uint64_t kPcgMul = 6364136223846793005ull;
constexpr uint64_t kPcgInc = 11634580027462260723ull;
FG_HDC uint64_t pcg_jump_mul(int k) {
    uint64_t a = 1;
    for (int i = 0; i < k; i++) a *= kPcgMul;
    return a;
}
FG_HDC uint64_t pcg_jump_add(int k) {
    uint64_t c = 0;
    for (int i = 0; i < k; i++) c = c * kPcgMul + kPcgInc;
    return c;
}
FG_HDC uint64_t splitmix_word(int k) {  // fmix64(k * phi): word k-1 of seed_from_u64(0)
    uint64_t z = (uint64_t)k * kPhi;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
FG_HD uint32_t rotr32(uint32_t x, uint32_t r) {
#ifdef __CUDA_ARCH__
    return __funnelshift_r(x, x, r);
#else
    r &= 31u;
    return r ? (x >> r) | (x << (32u - r)) : x;
#endif
}
FG_HD uint32_t funnel_r32(uint32_t lo, uint32_t hi, int s) {  // low word of (hi:lo) >> s, 0 < s < 32
#ifdef __CUDA_ARCH__
    return __funnelshift_r(lo, hi, s);
#else
    return (lo >> s) | (hi << (32 - s));
#endif
}
// Seed word k (1..8) of seed_from_u64(h).  The state st = a*h + c (mod 2^64) in 32-bit halves: the
// low product with c added in one wide multiply-add, the cross products into the high half; the
// output needs bits 27..58 of st ^ (st >> 18), i.e. (st >> 27) ^ (st >> 45) cut to 32 bits, rotated
// right by st >> 59.
template <int K>
FG_HD uint32_t pcg_word(uint64_t h) {
    constexpr uint64_t a = pcg_jump_mul(K), c = pcg_jump_add(K);
    const uint32_t hl = (uint32_t)h, hh = (uint32_t)(h >> 32);
    const uint64_t w = (uint64_t)hl * (uint32_t)a + c;
    const uint32_t L = (uint32_t)w;
    const uint32_t H = (uint32_t)(w >> 32) + hl * (uint32_t)(a >> 32) + hh * (uint32_t)a;
    return rotr32(funnel_r32(L, H, 27) ^ (H >> 13), H >> 27);
}
FG_HD uint64_t pcg_pair(uint32_t lo, uint32_t hi) { return (uint64_t)lo | ((uint64_t)hi << 32); }
FG_HD Xoshiro small_seed_zero() {
    Xoshiro x;
    x.s0 = splitmix_word(1);
    x.s1 = splitmix_word(2);
    x.s2 = splitmix_word(3);
    x.s3 = splitmix_word(4);
    return x;
}
FG_HD Xoshiro small_seed(uint64_t h) {
    Xoshiro x;
    x.s0 = pcg_pair(pcg_word<1>(h), pcg_word<2>(h));
    x.s1 = pcg_pair(pcg_word<3>(h), pcg_word<4>(h));
    x.s2 = pcg_pair(pcg_word<5>(h), pcg_word<6>(h));
    x.s3 = pcg_pair(pcg_word<7>(h), pcg_word<8>(h));
    if ((x.s0 | x.s1 | x.s2 | x.s3) == 0) return small_seed_zero();
    return x;
}
// The first next_u64 output of small_seed(h), from seed words 1, 2, 7 and 8 alone (the other two
// state words enter only through the all-zero remap, checked when s0 and s3 are both zero).
FG_HD uint64_t small_first_u64(uint64_t h) {
    const uint64_t s0 = pcg_pair(pcg_word<1>(h), pcg_word<2>(h));
    const uint64_t s3 = pcg_pair(pcg_word<7>(h), pcg_word<8>(h));
    if ((s0 | s3) == 0) {
        const Xoshiro x = small_seed(h);
        return rotl64(x.s0 + x.s3, 23) + x.s0;
    }
    return rotl64(s0 + s3, 23) + s0;
}
// The emptiness screen of a cell with hash h: true when its first draw v = small_first_u64(h) >> 11
// exceeds its Knuth threshold, computed as r1 - 1 >= screen_bound(thresh) (unsigned) on the first
// output r1 built from seed words 1, 2, 7 and 8 without the all-zero remap -- (thresh + 1) * 2^11 - 1,
// 0 for a negative threshold (always true), all ones from 2^53 - 1 up (never).  An all-zero seed wraps
// to true: every caller follows a passing screen with the exact count (cell_count_h), so the wrap costs
// work, never a result.
FG_HD uint64_t screen_bound(long long thresh) {
    if (thresh < 0) return 0ull;
    if (thresh >= (1ll << 53) - 1) return ~0ull;
    return (((uint64_t)thresh + 1ull) << 11) - 1ull;
}
FG_HD bool first_draw_screen(uint64_t h, uint64_t bound) {
    const uint64_t s0 = pcg_pair(pcg_word<1>(h), pcg_word<2>(h));
    const uint64_t s3 = pcg_pair(pcg_word<7>(h), pcg_word<8>(h));
    return rotl64(s0 + s3, 23) + s0 - 1ull >= bound;
}
// src/rng.rs:26-29 / 31-34
FG_HD Xoshiro cell_rng(uint64_t seed, int32_t i, int32_t j) { return small_seed(mix3(seed, kCellStream, i, j)); }
FG_HD Xoshiro pixel_rng(uint64_t seed, int32_t i, int32_t j) { return small_seed(mix3(seed, kPixelStream, i, j)); }

FG_HD float bits_f32(uint32_t b) {
#ifdef __CUDA_ARCH__
    return __uint_as_float(b);
#else
    union { uint32_t u; float f; } c; c.u = b; return c.f;
#endif
}
FG_HD uint32_t f32_bits(float f) {
#ifdef __CUDA_ARCH__
    return __float_as_uint(f);
#else
    union { uint32_t u; float f; } c; c.f = f; return c.u;
#endif
}
FG_HD double bits_f64(uint64_t b) {
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long)b);
#else
    union { uint64_t u; double d; } c; c.u = b; return c.d;
#endif
}
FG_HD uint64_t f64_bits(double d) {
#ifdef __CUDA_ARCH__
    return (uint64_t)__double_as_longlong(d);
#else
    union { uint64_t u; double d; } c; c.d = d; return c.u;
#endif
}

// v * 2^-53 for v < 2^53, built from integer operations only (exact; no FP64 conversion unit).
FG_HD double u53_unit(uint64_t v) {
    if (v == 0) return 0.0;
#ifdef __CUDA_ARCH__
    int lz = __clzll((long long)v);
#else
    int lz = __builtin_clzll(v);
#endif
    int e = 63 - lz;  // 0..52
    uint64_t mant = (v << (52 - e)) & 0x000FFFFFFFFFFFFFull;
    uint64_t ex = (uint64_t)(1023 - 53 + e);
    return bits_f64((ex << 52) | mant);
}
// v * 2^-51 for |v| <= 2^51, built from integer operations only (exact).
FG_HD double i51_scaled(int64_t v) {
    if (v == 0) return 0.0;
    const uint64_t sign = v < 0 ? 0x8000000000000000ull : 0ull;
    const uint64_t a = v < 0 ? (uint64_t)(-v) : (uint64_t)v;
#ifdef __CUDA_ARCH__
    const int e = 63 - __clzll((long long)a);
#else
    const int e = 63 - __builtin_clzll(a);
#endif
    const uint64_t mant = (a << (52 - e)) & 0x000FFFFFFFFFFFFFull;  // e <= 51
    return bits_f64(sign | ((uint64_t)(1023 - 51 + e) << 52) | mant);
}
// Standard f64 from one raw draw.
FG_HD double std_f64_from(uint64_t raw) { return u53_unit(raw >> 11); }
// Open01 f64 from one raw draw: [1,2) minus (1 - eps/2).
FG_HD double open01_from(uint64_t raw) {
    return FG_DSUB(bits_f64((raw >> 12) | 0x3FF0000000000000ull), 0.99999999999999988897769753748434595763683319091796875);
}

// UniformFloat<f32> (rand 0.8.5).
struct UniformF32 {
    float low, scale;
};
FG_HD UniformF32 uniform_f32_new(float low, float high) {
    const float max_rand = bits_f32(0x3F800000u | (0xFFFFFFFFu >> 9)) - 1.0f;  // 1 - 2^-23, exact
    float scale = FG_FSUB(high, low);
    for (int guard = 0; guard < 64; guard++) {
        float t = FG_FADD(FG_FMUL(scale, max_rand), low);
        if (!(t >= high)) break;
        scale = bits_f32(f32_bits(scale) - 1u);
    }
    UniformF32 u = {low, scale};
    return u;
}
// One sample from one raw next_u64 draw (next_u32 = high half; 23 high bits of that).
FG_HD float uniform_f32_from(const UniformF32 &u, uint64_t raw) {
    uint32_t m = (uint32_t)(raw >> 41);
    float v01 = FG_FSUB(bits_f32(m | 0x3F800000u), 1.0f);
    return FG_FADD(FG_FMUL(v01, u.scale), u.low);
}

// rand_distr::utils::log_gamma: Numerical Recipes' gammln (Lanczos, g = 5, six terms).
FG_HD double log_gamma(double x) {
    const double c0 = 76.18009172947146, c1 = -86.50532032941677, c2 = 24.01409824083091,
                 c3 = -1.231739572450155, c4 = 0.1208650973866179e-2, c5 = -0.5395239384953e-5;
    double tmp = FG_DADD(x, 5.5);
    double lg = FG_DSUB(FG_DMUL(FG_DADD(x, 0.5), log(tmp)), tmp);
    double a = 1.000000000190015;
    double den = x;
    den = FG_DADD(den, 1.0); a = FG_DADD(a, FG_DDIV(c0, den));
    den = FG_DADD(den, 1.0); a = FG_DADD(a, FG_DDIV(c1, den));
    den = FG_DADD(den, 1.0); a = FG_DADD(a, FG_DDIV(c2, den));
    den = FG_DADD(den, 1.0); a = FG_DADD(a, FG_DDIV(c3, den));
    den = FG_DADD(den, 1.0); a = FG_DADD(a, FG_DDIV(c4, den));
    den = FG_DADD(den, 1.0); a = FG_DADD(a, FG_DDIV(c5, den));
    return FG_DADD(lg, log(FG_DDIV(FG_DMUL(2.5066282746310005, a), x)));
}

// Poisson::new (rand_distr 0.4.3).
struct PoissonParams {
    double lambda, exp_lambda, log_lambda, sqrt_2lambda, magic_val;
};
FG_HD PoissonParams poisson_new(double lambda) {
    PoissonParams p;
    p.lambda = lambda;
    p.log_lambda = log(lambda);
    p.exp_lambda = exp(-lambda);
    p.sqrt_2lambda = sqrt(FG_DMUL(2.0, lambda));
    p.magic_val = FG_DSUB(FG_DMUL(lambda, p.log_lambda), log_gamma(FG_DADD(1.0, lambda)));
    return p;
}

// Knuth continuation: p already holds the first uniform and exceeds exp_lambda; returns the count
// (the sampler's f64 `result` counter is an exact small integer, kept here as an integer).  p and
// exp_lambda are positive doubles, whose bit patterns order like their values, so the comparison is
// an integer one.  The draw consumes exactly count + 1 uniforms.
template <class Rng>
FG_HD uint32_t poisson_knuth_tail(double p, double exp_lambda, Rng &rng) {
    const uint64_t e = f64_bits(exp_lambda);
    uint32_t count = 1;
    p = FG_DMUL(p, std_f64_from(rng.next()));
    while (f64_bits(p) > e) {
        p = FG_DMUL(p, std_f64_from(rng.next()));
        count++;
    }
    return count;
}

// Poisson::sample, rejection branch (lambda >= 12).
template <class Rng>
FG_HD uint32_t poisson_rejection(const PoissonParams &P, Rng &rng) {
    const double kPi = 3.14159265358979323846264338327950288;
    double result, comp_dev;
    for (;;) {
        for (;;) {
            double x = std_f64_from(rng.next());
            comp_dev = tan(FG_DMUL(kPi, x));
            comp_dev = FG_DADD(0.0, FG_DMUL(1.0, comp_dev));  // Cauchy(median 0, scale 1)
            result = FG_DADD(FG_DMUL(P.sqrt_2lambda, comp_dev), P.lambda);
            if (result >= 0.0) break;
        }
        result = floor(result);
        double arg = FG_DSUB(FG_DSUB(FG_DMUL(result, P.log_lambda), log_gamma(FG_DADD(1.0, result))), P.magic_val);
        double check = FG_DMUL(FG_DMUL(0.9, FG_DADD(1.0, FG_DMUL(comp_dev, comp_dev))), exp(arg));
        if (std_f64_from(rng.next()) <= check) break;
    }
    return result >= 4294967295.0 ? 0xFFFFFFFFu : (uint32_t)result;
}

// Poisson::sample cast with `as u32`.
template <class Rng>
FG_HD uint32_t poisson_sample(const PoissonParams &P, Rng &rng) {
    if (P.lambda < 12.0) {
        double p = std_f64_from(rng.next());
        if (!(p > P.exp_lambda)) return 0;
        return poisson_knuth_tail(p, P.exp_lambda, rng);
    }
    return poisson_rejection(P, rng);
}

// 256-layer ziggurat tables.
#ifdef __CUDACC__
static __device__ const double g_zig_x[257] = FG_ZIG_NORM_X_INIT;
static __device__ const double g_zig_f[257] = FG_ZIG_NORM_F_INIT;
#endif
static const double h_zig_x[257] = FG_ZIG_NORM_X_INIT;
static const double h_zig_f[257] = FG_ZIG_NORM_F_INIT;

FG_HD double zig_x(unsigned i) {
#ifdef __CUDA_ARCH__
    return __ldg(&g_zig_x[i]);
#else
    return h_zig_x[i];
#endif
}
FG_HD double zig_f(unsigned i) {
#ifdef __CUDA_ARCH__
    return __ldg(&g_zig_f[i]);
#else
    return h_zig_f[i];
#endif
}

// StandardNormal for f64 (rand_distr 0.4.3 ziggurat, symmetric, 256 layers).
template <class Rng>
FG_HD double std_normal(Rng &rng) {
    for (;;) {
        uint64_t bits = rng.next();
        unsigned i = (unsigned)(bits & 0xffu);
        // u = (2 + m*2^-51) - 3 for the 52-bit m = bits >> 12, i.e. exactly (m - 2^51) * 2^-51,
        // built from integer operations (the subtraction is exact in f64).
        double u = i51_scaled((int64_t)(bits >> 12) - (int64_t)(1ull << 51));
        double x = FG_DMUL(u, zig_x(i));
        // |x| < x_tab[i+1]: both non-negative doubles, so their bit patterns order like the values.
        if ((f64_bits(x) & 0x7FFFFFFFFFFFFFFFull) < f64_bits(zig_x(i + 1))) return x;
        if (i == 0) {
            double xx = 1.0, yy = 0.0;
            while (FG_DMUL(-2.0, yy) < FG_DMUL(xx, xx)) {
                double x_ = open01_from(rng.next());
                double y_ = open01_from(rng.next());
                xx = FG_DDIV(log(x_), FG_ZIG_NORM_R);
                yy = log(y_);
            }
            return (u < 0.0) ? FG_DSUB(xx, FG_ZIG_NORM_R) : FG_DSUB(FG_ZIG_NORM_R, xx);
        }
        double pdf = exp(FG_DDIV(FG_DMUL(-x, x), 2.0));
        double fi1 = zig_f(i + 1);
        if (FG_DADD(fi1, FG_DMUL(FG_DSUB(zig_f(i), fi1), std_f64_from(rng.next()))) < pdf) return x;
    }
}

// Normal::sample = mean + sd * z.
template <class Rng>
FG_HD double normal_sample(double mean, double sd, Rng &rng) {
    return FG_DADD(mean, FG_DMUL(sd, std_normal(rng)));
}

// ------------------------------------------------------------------ exp(t) rounded to f32
// LogNormal::sample(...) as f32 (src/model.rs:141-142) is RN_f32(exp(t)) of an f64 exp.  FP64
// throughput is a small fraction of FP32 on this part, so exp(t) is evaluated in double-float
// arithmetic on the FP32 pipes, by a table-driven method in the manner of P. T. P. Tang ("Table-driven
// implementation of the exponential function in IEEE floating-point arithmetic", ACM TOMS 15(2),
// 1989): a Cody-Waite reduction by ln 2 split into three parts, a second reduction against a table of
// exp(j/64), and a short polynomial:
//   t = th + tm + tt exactly (three floats cut from t's 53-bit significand);
//   r = t - k*ln2 with ln2 = L1 + L2 + L3 (L1 has 12 significant bits, so k*L1 is exact);
//   exp(r) = T[j] * exp(s), s = r - j/64, T[j] = exp(j/64) as a float pair (exp_table.h);
//   exp(s) = 1 + s + s^2/2 (double-float) + s^3/6 + ... + s^6/720 (float tail).
// The double-float result carries exp(t) to about 2^-43 relative.  When it lies within 2^-40 of an
// f32 rounding midpoint the FP64 exp decides instead; otherwise RN_f32 of the double-float value
// equals RN_f32 of any f64 exp within 2^-50 of the true value.
#include "exp_table.h"
#ifndef FG_EXP_FALLBACK_HOOK
#define FG_EXP_FALLBACK_HOOK()  // counted by the native host checker in tests/native
#endif

#ifdef __CUDACC__
static __device__ const float2 g_exp64[49] = FG_EXP64_TABLE_INIT;
#endif
struct FgFloat2 { float x, y; };
static const FgFloat2 h_exp64[49] = FG_EXP64_TABLE_INIT;

FG_HD float ff_fma(float a, float b, float c) {
#ifdef __CUDA_ARCH__
    return __fmaf_rn(a, b, c);
#else
    return fmaf(a, b, c);
#endif
}
FG_HD void ff_two_sum(float a, float b, float &s, float &e) {
    s = FG_FADD(a, b);
    float bb = FG_FSUB(s, a);
    e = FG_FADD(FG_FSUB(a, FG_FSUB(s, bb)), FG_FSUB(b, bb));
}
FG_HD void ff_fast_two_sum(float a, float b, float &s, float &e) {
    s = FG_FADD(a, b);
    e = FG_FSUB(b, FG_FSUB(s, a));
}
FG_HD float pow2f(int e) { return bits_f32((uint32_t)(e + 127) << 23); }  // e in [-126, 127]

FG_HD float exp_f64_to_f32(double t) {
    const uint64_t b = f64_bits(t);
    const uint32_t E = (uint32_t)(b >> 52) & 0x7FFu;
    if (E < 1023u - 30u) return 1.0f;                // |t| < 2^-30: exp(t) rounds to 1
    if (E >= 1023u + 4u) {                           // |t| >= 16, inf, nan
        FG_EXP_FALLBACK_HOOK();
        return (float)exp(t);
    }
    const uint64_t m = (b & 0x000FFFFFFFFFFFFFull) | 0x0010000000000000ull;  // t = +-m * 2^(E-1075)
    const uint32_t neg = (uint32_t)(b >> 63) << 31;
    const int e0 = (int)E - 1075;                    // in [-82, -49]
    const float th = bits_f32(neg | ((E - 896u) << 23) | ((uint32_t)(m >> 29) & 0x7FFFFFu));
    const float tm = bits_f32(f32_bits((float)(uint32_t)((m >> 5) & 0xFFFFFFu) * pow2f(e0 + 5)) | neg);
    const float tt = bits_f32(f32_bits((float)(uint32_t)(m & 31u) * pow2f(e0)) | neg);

    const float L1 = 0.693115234375f, L2 = 3.1946183e-05f, L3 = 1.646595e-12f;
    const float kf = rintf(FG_FMUL(th, 1.44269504f));
    const float a = FG_FSUB(th, FG_FMUL(kf, L1));    // exact (Sterbenz; k*L1 exact)
    const float p2h = FG_FMUL(kf, L2);
    const float p2l = ff_fma(kf, L2, -p2h);
    float sh, sl, e2;
    ff_two_sum(a, -p2h, sh, sl);
    ff_two_sum(sh, tm, sh, e2);
    sl = FG_FADD(FG_FADD(sl, e2), FG_FSUB(FG_FSUB(tt, p2l), FG_FMUL(kf, L3)));
    ff_fast_two_sum(sh, sl, sh, sl);

    const float jf = rintf(FG_FMUL(sh, 64.0f));      // |j| <= 23
    const int j = (int)jf;
    const float s = FG_FSUB(sh, FG_FMUL(jf, 0.015625f));  // exact
    const float q = FG_FMUL(s, s);
    const float ql = ff_fma(s, s, -q);
    float tail = FG_FADD(0.00833333377f, FG_FMUL(s, 0.00138888892f));
    tail = FG_FADD(0.0416666679f, FG_FMUL(s, tail));
    tail = FG_FADD(0.166666672f, FG_FMUL(s, tail));
    tail = FG_FMUL(FG_FMUL(s, q), tail);             // s^3/6 + s^4/24 + s^5/120 + s^6/720
    tail = FG_FADD(tail, FG_FMUL(s, sl));            // cross term of (s + sl)^2 / 2
    float a1, a1l;
    ff_two_sum(s, FG_FMUL(q, 0.5f), a1, a1l);
    a1l = FG_FADD(a1l, FG_FADD(sl, FG_FADD(FG_FMUL(ql, 0.5f), tail)));
    float b1, b1l;
    ff_two_sum(1.0f, a1, b1, b1l);
    b1l = FG_FADD(b1l, a1l);
    ff_fast_two_sum(b1, b1l, b1, b1l);
#ifdef __CUDA_ARCH__
    const float2 T = g_exp64[j + 24];
#else
    const FgFloat2 T = h_exp64[j + 24];
#endif
    float yh = FG_FMUL(T.x, b1);
    float yl = ff_fma(T.x, b1, -yh);
    yl = FG_FADD(yl, FG_FADD(FG_FMUL(T.x, b1l), FG_FMUL(T.y, b1)));
    ff_fast_two_sum(yh, yl, yh, yl);
    const float P = pow2f((int)kf);                  // |k| <= 23
    const float f = FG_FMUL(yh, P), fl = FG_FMUL(yl, P);
    const uint32_t fb = f32_bits(f);
    const float up = FG_FSUB(bits_f32(fb + 1u), f), dn = FG_FSUB(f, bits_f32(fb - 1u));
    const float half = fl >= 0.0f ? FG_FMUL(0.5f, up) : FG_FMUL(0.5f, dn);
    const float dist = fabsf(FG_FSUB(fabsf(fl), half));
    if (!(dist > FG_FMUL(f, 9.09494702e-13f)) || !(fabsf(fl) <= half)) {  // within 2^-40 of a midpoint
        FG_EXP_FALLBACK_HOOK();
        return (float)exp(t);
    }
    return f;
}

// The lognormal radius draw: LogNormal::sample (rand_distr 0.4.3) cast to f32.
template <class Rng>
FG_HD float lognormal_radius_f32(double mu, double sigma, Rng &rng) {
    return exp_f64_to_f32(normal_sample(mu, sigma, rng));
}

// ChaCha12 keystream reader (StdRng), seeded through rand_core's PCG32 seed_from_u64.
struct ChaCha12 {
    uint32_t key[8];
    uint64_t block;
    uint32_t buf[16];
    int idx;
};
FG_HD uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
FG_HD void chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream, int rounds, uint32_t out[16]) {
    uint32_t s[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u, key[0], key[1], key[2], key[3],
                      key[4], key[5], key[6], key[7], (uint32_t)counter, (uint32_t)(counter >> 32),
                      (uint32_t)stream, (uint32_t)(stream >> 32)};
    uint32_t x[16];
    for (int i = 0; i < 16; i++) x[i] = s[i];
#define FG_QR(a, b, c, d)                                                     \
    x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 16);                            \
    x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 12);                            \
    x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 8);                             \
    x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 7);
    for (int r = 0; r < rounds; r += 2) {
        FG_QR(0, 4, 8, 12) FG_QR(1, 5, 9, 13) FG_QR(2, 6, 10, 14) FG_QR(3, 7, 11, 15)
        FG_QR(0, 5, 10, 15) FG_QR(1, 6, 11, 12) FG_QR(2, 7, 8, 13) FG_QR(3, 4, 9, 14)
    }
#undef FG_QR
    for (int i = 0; i < 16; i++) out[i] = x[i] + s[i];
}
FG_HD ChaCha12 chacha12_seed_from_u64(uint64_t state) {
    ChaCha12 c;
    c.key[0] = pcg_word<1>(state);
    c.key[1] = pcg_word<2>(state);
    c.key[2] = pcg_word<3>(state);
    c.key[3] = pcg_word<4>(state);
    c.key[4] = pcg_word<5>(state);
    c.key[5] = pcg_word<6>(state);
    c.key[6] = pcg_word<7>(state);
    c.key[7] = pcg_word<8>(state);
    c.block = 0;
    c.idx = 16;
    return c;
}
struct ChaChaStream {
    ChaCha12 c;
    FG_HD uint64_t next() {
        if (c.idx >= 16) {
            chacha_block(c.key, c.block++, 0, 12, c.buf);
            c.idx = 0;
        }
        uint64_t lo = c.buf[c.idx], hi = c.buf[c.idx + 1];
        c.idx += 2;
        return (hi << 32) | lo;
    }
};

}  // namespace fg
