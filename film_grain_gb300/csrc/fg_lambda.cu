// fg_lambda.cu -- the whole-image prelude on the device: the colour workspace split, normalize_plane
// and lambda_plane (src/color.rs:158-213, src/model.rs:228-265), bit-identical to the host versions.
//
// The crate computes lambda = min(-inv_e_pi_r2 * ln(max(1 - u, 1e-6)), 1e6) in f32 with f32::ln, the
// platform logf.  The device evaluates RN_f32(log((double)x)) and replaces it, on the inputs listed in
// the process's logf table (fg_host.cpp logf_table: where the platform logf and that value differ, or
// could under a last-ulp difference of the double log), by the platform logf's own result, so the
// device plane equals the host plane on every input.  Everything else is exact f32 arithmetic in the
// host code's order (--fmad=false, explicit round-to-nearest operations).
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/film_grain_gb300.h"
#include "fg_host.h"
#include "fg_internal.h"
#include "fg_kernels.cuh"
#include "fg_rng.cuh"

namespace fg {

constexpr float kLamEps = 1e-6f;    // src/model.rs:10
constexpr float kMaxLambda = 1.0e6f;  // src/model.rs:11

// f32::clamp: a NaN passes through with its bits (tested on the integer bits, so that no NaN-propagating
// min/max can replace its payload with the canonical NaN).
__device__ __forceinline__ float clampf_d(float x, float lo, float hi) {
    if ((__float_as_uint(x) & 0x7fffffffu) > 0x7f800000u) return x;
    if (x < lo) x = lo;  // comparisons, not min/max: -0.0 stays -0.0 as in f32::clamp
    if (x > hi) x = hi;
    return x;
}

// v / den as the host's f32 division gives it, NaN bits included: a NaN dividend comes back unchanged
// (x86 and Arm propagate the dividend's payload; CUDA's division returns its canonical NaN), and a NaN
// made by the division itself (inf / inf) is the host's default NaN, `host_nan`.
__device__ __forceinline__ float div_like_host(float v, float den, uint32_t host_nan) {
    if ((__float_as_uint(v) & 0x7fffffffu) > 0x7f800000u) return v;
    const float q = FG_FDIV(v, den);
    return (__float_as_uint(q) & 0x7fffffffu) > 0x7f800000u ? __uint_as_float(host_nan) : q;
}

// The platform logf on [1e-6, 1].
__device__ __forceinline__ float platform_logf(float x, const LogfTableDev &t) {
    float y = __double2float_rn(log((double)x));
    const uint32_t b = __float_as_uint(x);
    if (b >= t.lo_bits && b <= t.hi_bits) {
        const uint32_t k = (b - t.lo_bits) >> t.shift;
        uint32_t lo = __ldg(t.bucket_start + k), hi = __ldg(t.bucket_start + k + 1);
        while (lo < hi) {  // first key >= b
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(t.keys + mid) < b) lo = mid + 1;
            else hi = mid;
        }
        if (lo < __ldg(t.bucket_start + k + 1) && __ldg(t.keys + lo) == b) y = __uint_as_float(__ldg(t.vals + lo));
    }
    return y;
}

// Plane maxima as normalize_plane folds them (fold(0.0, f32::max): NaN ignored), as f32 bit patterns of
// non-negative values, so that atomicMax on the bits orders them like the values.
__device__ __forceinline__ void block_max_to(float m, unsigned int *dst) {
    m = m > 0.0f ? m : 0.0f;  // -0.0 and NaN-free start at +0.0
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wmax[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) wmax[warp] = m;
    __syncthreads();
    if (warp == 0) {
        m = lane < (int)(blockDim.x >> 5) ? wmax[lane] : 0.0f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0 && m > 0.0f) atomicMax(dst, __float_as_uint(m));
    }
    __syncthreads();
}

// load_luma_workspace / load_rgb_workspace (src/color.rs:158-213) from the cropped interleaved RGB:
// luma writes Y (clamped), Cb and Cr; RGB writes the three clamped channels; and the maxima of the
// planes that normalize_plane will see (Y, or R, G and B).
__global__ void split_max_kernel(const float *__restrict__ rgb, long long n, int luma, float *__restrict__ p0,
                                 float *__restrict__ p1, float *__restrict__ p2, unsigned int *__restrict__ maxbits) {
    const float YR = 0.2126f, YG = 0.7152f, YB = 0.0722f, CBD = 1.8556f, CRD = 1.5748f;
    float m0 = 0.0f, m1 = 0.0f, m2 = 0.0f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float r = clampf_d(rgb[3 * i], 0.0f, 1.0f), g = clampf_d(rgb[3 * i + 1], 0.0f, 1.0f),
                    b = clampf_d(rgb[3 * i + 2], 0.0f, 1.0f);
        if (luma) {
            const float l = FG_FADD(FG_FADD(FG_FMUL(YR, r), FG_FMUL(YG, g)), FG_FMUL(YB, b));
            p1[i] = FG_FDIV(FG_FSUB(b, l), CBD);
            p2[i] = FG_FDIV(FG_FSUB(r, l), CRD);
            const float y = clampf_d(l, 0.0f, 1.0f);
            p0[i] = y;
            m0 = fmaxf(m0, y);
        } else {
            p0[i] = r; p1[i] = g; p2[i] = b;
            m0 = fmaxf(m0, r); m1 = fmaxf(m1, g); m2 = fmaxf(m2, b);
        }
    }
    block_max_to(m0, maxbits);
    if (!luma) {
        block_max_to(m1, maxbits + 1);
        block_max_to(m2, maxbits + 2);
    }
}

// Plane maxima of planes that are already split (fg_normalize_plane / fg_lambda_from_plane on device
// memory).
__global__ void plane_max_kernel(const float *__restrict__ src, long long n, unsigned int *__restrict__ maxbits) {
    float m = 0.0f;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        m = fmaxf(m, src[i]);
    block_max_to(m, maxbits);
}

// normalize_plane's element (src/model.rs:237-247) followed, when `lambda` is set, by lambda_plane's
// (src/model.rs:255-263): plane c of `src` (n elements each) -> plane c of `dst`.
__global__ void normalize_lambda_kernel(const float *__restrict__ src, long long n, int nplanes,
                                        const unsigned int *__restrict__ maxbits, int normalize, int lambda,
                                        float inv_e_pi_r2, LogfTableDev t, uint32_t host_nan,
                                        float *__restrict__ dst) {
    const long long total = n * nplanes;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(q / n);
        float v = src[q];
        if (normalize) {
            const float mx = __uint_as_float(maxbits[c]);
            const bool already = mx <= FG_FADD(1.0f, kLamEps);
            float den = FG_FADD(mx, kLamEps);
            if (den < kLamEps) den = kLamEps;
            v = clampf_d(already ? v : div_like_host(v, den, host_nan), 0.0f, 1.0f - kLamEps);
        }
        if (lambda) {
            const float cl = clampf_d(v, 0.0f, 1.0f - kLamEps);
            const float safe = fmaxf(FG_FSUB(1.0f, cl), kLamEps);
            const float act = FG_FMUL(-inv_e_pi_r2, platform_logf(safe, t));
            v = fminf(act, kMaxLambda);
        }
        dst[q] = v;
    }
}

// ------------------------------------------------------------------ the logf table on each device
struct DevTable {
    LogfTableDev t;
    bool ready = false;
};
static std::mutex g_tab_mu;
static DevTable g_tab[128];

fg_status device_logf_table(LogfTableDev *out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
    if (dev < 0 || dev >= 128) return set_error(FG_ERR_UNSUPPORTED, "device ordinal out of range");
    const LogfTable &h = logf_table();  // built once per process, outside the lock
    std::lock_guard<std::mutex> lock(g_tab_mu);
    DevTable &d = g_tab[dev];
    if (!d.ready) {
        const size_t nb = h.bucket_start.size(), nk = h.keys.size();
        uint32_t *buf = nullptr;
        e = cudaMalloc(&buf, sizeof(uint32_t) * (nb + 2 * nk + 1));
        if (e != cudaSuccess) return cuda_error(e, "alloc logf table");
        e = cudaMemcpy(buf, h.bucket_start.data(), sizeof(uint32_t) * nb, cudaMemcpyHostToDevice);
        if (e == cudaSuccess && nk)
            e = cudaMemcpy(buf + nb, h.keys.data(), sizeof(uint32_t) * nk, cudaMemcpyHostToDevice);
        if (e == cudaSuccess && nk)
            e = cudaMemcpy(buf + nb + nk, h.vals.data(), sizeof(uint32_t) * nk, cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            cudaFree(buf);
            return cuda_error(e, "logf table H2D");
        }
        d.t.bucket_start = buf;
        d.t.keys = buf + nb;
        d.t.vals = buf + nb + nk;
        d.t.lo_bits = h.lo_bits;
        d.t.hi_bits = h.hi_bits;
        d.t.shift = h.shift;
        d.ready = true;
    }
    *out = d.t;
    return FG_OK;
}

// The NaN this host's f32 division makes from inf / inf (x86: the negative quiet NaN, Arm: the positive
// one), computed at run time on the host itself.
static uint32_t host_default_nan() {
    volatile float inf = INFINITY;
    const float q = inf / inf;
    uint32_t b;
    std::memcpy(&b, &q, 4);
    return b;
}

static unsigned grid_for(long long n) {
    long long g = (n + 255) / 256;
    return (unsigned)std::max<long long>(1, std::min<long long>(g, 152LL * 16));
}

fg_status enqueue_split_lambda(const float *d_rgb, long long n_in, int luma, float *d_planes, unsigned int *d_max,
                               float inv_e_pi_r2, float *d_lam, cudaStream_t s) {
    LogfTableDev t;
    fg_status st = device_logf_table(&t);
    if (st != FG_OK) return st;
    cudaError_t e = cudaMemsetAsync(d_max, 0, 3 * sizeof(unsigned int), s);
    if (e != cudaSuccess) return cuda_error(e, "clear plane maxima");
    split_max_kernel<<<grid_for(n_in), 256, 0, s>>>(d_rgb, n_in, luma, d_planes, d_planes + n_in, d_planes + 2 * n_in,
                                                      d_max);
    const int nplanes = luma ? 1 : 3;
    normalize_lambda_kernel<<<grid_for(n_in * nplanes), 256, 0, s>>>(d_planes, n_in, nplanes, d_max, 1, 1, inv_e_pi_r2,
                                                                     t, host_default_nan(), d_lam);
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_error(e, "lambda kernels");
    return FG_OK;
}

// normalize_plane / lambda_plane / both, on device memory (synchronous; the legacy default stream).
fg_status device_plane_pass(const float *src, int64_t n, int normalize, int lambda, float inv_e_pi_r2, float *dst,
                            float *max_out) {
    LogfTableDev t;
    std::memset(&t, 0, sizeof t);
    if (lambda) {
        fg_status st = device_logf_table(&t);
        if (st != FG_OK) return st;
    }
    unsigned int *d_max = nullptr;
    cudaError_t e = cudaMalloc(&d_max, sizeof(unsigned int));
    if (e != cudaSuccess) return cuda_error(e, "alloc plane maximum");
    e = cudaMemset(d_max, 0, sizeof(unsigned int));
    if (e == cudaSuccess && normalize) {
        plane_max_kernel<<<grid_for(n), 256>>>(src, n, d_max);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) {
        normalize_lambda_kernel<<<grid_for(n), 256>>>(src, n, 1, d_max, normalize, lambda, inv_e_pi_r2, t,
                                                      host_default_nan(), dst);
        e = cudaGetLastError();
    }
    unsigned int mb = 0;
    if (e == cudaSuccess) e = cudaMemcpy(&mb, d_max, sizeof mb, cudaMemcpyDeviceToHost);
    cudaFree(d_max);
    if (e != cudaSuccess) return cuda_error(e, "plane pass");
    if (max_out) std::memcpy(max_out, &mb, sizeof mb);
    return FG_OK;
}

}  // namespace fg
