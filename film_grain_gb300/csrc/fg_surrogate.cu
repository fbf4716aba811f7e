// fg_surrogate.cu -- the learned stand-in for the MC integrator: a residual 3x3-conv network.
//
// Layers (all 3x3, zero padding; activations NHWC bf16; weights [cout][tap][cin] bf16; f32 accumulation):
//   x   = (u, N(0,1) noise, radius map, 0 ...)        16 channels (3 used)
//   h0  = relu(conv_in(x) + b_in)                     16 -> 32
//   h_l = h_{l-1} + relu(conv_l(h_{l-1}) + b_l)       32 -> 32, l = 1..L
//   y   = u + conv_out(h_L) + b_out                   32 -> 1 (8 computed channels, channel 0 kept), f32
// Every conv is an implicit GEMM on the tensor cores (mma.sync m16n8k16, bf16 x bf16 -> f32): a CTA owns
// an 8 x 32 pixel tile, stages the haloed input tile and all weights in shared memory, and each of its 8
// warps computes one 32-pixel tile row for every output channel.  The backward pass reuses the forward
// kernel for the data gradient (weights flipped and transposed) and has a persistent weight-gradient
// kernel in which pixels are the reduction dimension.  No bit-exactness constraint applies here, so this
// unit is compiled with FMA contraction.
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>

#include "../../include/film_grain_gb300.h"
#include "fg_host.h"
#include "fg_internal.h"

namespace fg {

typedef __nv_bfloat16 bf16;

constexpr int kSgTH = 8, kSgTW = 32;  // output tile (rows x cols)
constexpr int kSgThreads = 256;       // 8 warps, one tile row each
constexpr int kSgHH = kSgTH + 2, kSgHW = kSgTW + 2;
constexpr int kSgNPix = kSgTH * kSgTW;

__device__ __forceinline__ uint32_t ld_u32(const bf16 *p) { return *reinterpret_cast<const uint32_t *>(p); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// Epilogue modes of the forward kernel.
enum SgMode {
    kSgRelu = 0,      // out = relu(z + b)
    kSgResidual = 1,  // r = relu(z + b); out = res + r; r is also stored when aux != null (ReLU mask)
    kSgOutput = 2,    // out_f32 = res_f32 + z + b (channel 0 only)
    kSgLinearAdd = 3, // out = res + z                   (data gradient through a residual layer)
    kSgLinear = 4     // out = z                         (data gradient of the output conv)
};

struct SgConvArgs {
    const bf16 *in;       // [nb][H][W][in_cstride]
    const bf16 *w;        // [COUT][9][CIN]
    const float *bias;    // [COUT]
    const bf16 *res;      // [nb][H][W][COUT]
    const float *res_f32; // [nb][H][W]
    bf16 *out;            // [nb][H][W][COUT]
    bf16 *aux;            // [nb][H][W][COUT] or null
    float *out_f32;       // [nb][H][W]
    int H, W, in_cstride, tiles_x, tiles_per_img;
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem, bool valid) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(valid ? 16 : 0));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
__device__ __forceinline__ void ldsm_x4(uint32_t (&r)[4], const bf16 *smem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(sa));
}
__device__ __forceinline__ void ldsm_x2(uint32_t (&r)[2], const bf16 *smem) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("ldmatrix.sync.aligned.m8n8.x2.shared.b16 {%0,%1}, [%2];\n" : "=r"(r[0]), "=r"(r[1]) : "r"(sa));
}

// Shared-memory bytes of the conv kernel: the weights plus two input-tile stages.
template <int CIN, int COUT>
constexpr int sg_conv_smem_bytes() {
    return (COUT * (9 * CIN + 8) + 2 * kSgHH * kSgHW * (CIN + 8)) * 2;
}

// 3x3 conv of CIN channels to COUT channels over all tiles of the batch.  Persistent: a CTA loads the
// weights once, then walks tiles with a grid stride, fetching the next tile's haloed input into the
// other shared-memory stage with cp.async (zero-filled outside the image) while the tensor cores work
// on the current one.  Fragments come from ldmatrix; the element strides (CIN + 8 per pixel, 9*CIN + 8
// per weight row) put the 8 rows of every ldmatrix phase in disjoint banks.
template <int CIN, int COUT, int MODE>
__global__ void __launch_bounds__(kSgThreads) sg_conv_fwd(const __grid_constant__ SgConvArgs a, int total_tiles) {
    constexpr int PS = CIN + 8;
    constexpr int K = 9 * CIN;
    constexpr int WS = K + 8;
    constexpr int NT = COUT / 8;
    constexpr int STAGE = kSgHH * kSgHW * PS;
    extern __shared__ __align__(16) unsigned char sg_smem[];
    bf16 *s_w = reinterpret_cast<bf16 *>(sg_smem);
    bf16 *s_stage = s_w + COUT * WS;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int H = a.H, W = a.W;

    constexpr int K8 = K / 8;
    for (int e = tid; e < COUT * K8; e += kSgThreads) {
        const int k8 = e % K8, n = e / K8;
        cp_async16(&s_w[n * WS + 8 * k8], a.w + (size_t)n * K + 8 * k8, true);
    }
    auto load_tile = [&](int t, bf16 *dst) {
        const int img = t / a.tiles_per_img, tt = t - img * a.tiles_per_img;
        const int y0 = (tt / a.tiles_x) * kSgTH, x0 = (tt % a.tiles_x) * kSgTW;
        const size_t img_off = (size_t)img * H * W;
        constexpr int C8 = CIN / 8;
        for (int e = tid; e < kSgHH * kSgHW * C8; e += kSgThreads) {
            const int c8 = e % C8, px = e / C8;
            const int hx = px % kSgHW, hy = px / kSgHW;
            const int gy = y0 + hy - 1, gx = x0 + hx - 1;
            const bool ok = gy >= 0 && gy < H && gx >= 0 && gx < W;
            const bf16 *src = ok ? a.in + (img_off + (size_t)gy * W + gx) * a.in_cstride + 8 * c8 : a.in;
            cp_async16(&dst[px * PS + 8 * c8], src, ok);
        }
    };
    int t = blockIdx.x;
    if (t < total_tiles) load_tile(t, s_stage);
    cp_async_commit();  // the weights and the first tile

    // ldmatrix lane addressing: A rows (pixels) 0-15 and k halves; B rows (output channels) and k halves
    const int a_row = (lane & 7) + ((lane >> 3) & 1) * 8, a_k = (lane >> 4) * 8;
    const int b_n = (lane & 7) + (lane >> 4) * 8, b_k = ((lane >> 3) & 1) * 8;
    const int g = lane >> 2, q = lane & 3;
    // this lane's bias pairs, and whether the residual is the conv's own input (then it is read from the
    // staged tile instead of global memory)
    float bias0[NT], bias1[NT];
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
        const bool used = MODE == kSgRelu || MODE == kSgResidual || (MODE == kSgOutput && nt == 0);
        bias0[nt] = used ? a.bias[8 * nt + 2 * q] : 0.0f;
        bias1[nt] = used && MODE != kSgOutput ? a.bias[8 * nt + 2 * q + 1] : 0.0f;
    }
    const bool res_staged = (MODE == kSgResidual || MODE == kSgLinearAdd) && a.res == a.in && a.in_cstride == COUT &&
                            CIN == COUT;
    int stage = 0;
    for (; t < total_tiles; t += gridDim.x) {
        if (t + (int)gridDim.x < total_tiles) load_tile(t + gridDim.x, s_stage + (stage ^ 1) * STAGE);
        cp_async_commit();
        cp_async_wait<1>();  // everything but the prefetch just issued has landed
        __syncthreads();
        const bf16 *s_in = s_stage + stage * STAGE;

        float acc[2][NT][4];
#pragma unroll
        for (int mt = 0; mt < 2; mt++)
#pragma unroll
            for (int nt = 0; nt < NT; nt++)
#pragma unroll
                for (int r = 0; r < 4; r++) acc[mt][nt][r] = 0.0f;
#pragma unroll
        for (int tap = 0; tap < 9; tap++) {
            const int ky = tap / 3, kx = tap % 3;
#pragma unroll
            for (int cb = 0; cb < CIN; cb += 16) {
                const int kbase = tap * CIN + cb;
                uint32_t bfr[NT][2];
                if constexpr (NT >= 2) {
#pragma unroll
                    for (int np = 0; np < NT; np += 2) {
                        uint32_t r[4];
                        ldsm_x4(r, &s_w[(np * 8 + b_n) * WS + kbase + b_k]);
                        bfr[np][0] = r[0];
                        bfr[np][1] = r[1];
                        bfr[np + 1][0] = r[2];
                        bfr[np + 1][1] = r[3];
                    }
                } else {
                    uint32_t r[2];
                    ldsm_x2(r, &s_w[(lane & 7) * WS + kbase + b_k]);
                    bfr[0][0] = r[0];
                    bfr[0][1] = r[1];
                }
#pragma unroll
                for (int mt = 0; mt < 2; mt++) {
                    uint32_t af[4];
                    ldsm_x4(af, &s_in[((warp + ky) * kSgHW + (16 * mt + a_row + kx)) * PS + cb + a_k]);
#pragma unroll
                    for (int nt = 0; nt < NT; nt++) mma_bf16(acc[mt][nt], af[0], af[1], af[2], af[3], bfr[nt][0], bfr[nt][1]);
                }
            }
        }

        // epilogue: acc[mt][nt][r] is (pixel 16*mt + g + 8*(r>>1), channel 8*nt + 2*q + (r&1))
        const int img = t / a.tiles_per_img, tt = t - img * a.tiles_per_img;
        const int oy = (tt / a.tiles_x) * kSgTH + warp, x0 = (tt % a.tiles_x) * kSgTW;
        const size_t img_off = (size_t)img * H * W;
        if (oy < H) {
#pragma unroll
            for (int mt = 0; mt < 2; mt++) {
#pragma unroll
                for (int half = 0; half < 2; half++) {
                    const int ox = x0 + 16 * mt + g + 8 * half;
                    if (ox >= W) continue;
                    const size_t p = img_off + (size_t)oy * W + ox;
                    if constexpr (MODE == kSgOutput) {
                        if (q == 0) a.out_f32[p] = a.res_f32[p] + acc[mt][0][2 * half] + bias0[0];
                    } else {
                        // the output pixel's position in the staged (haloed) tile
                        const bf16 *srow = &s_in[((warp + 1) * kSgHW + (16 * mt + g + 8 * half + 1)) * PS];
#pragma unroll
                        for (int nt = 0; nt < NT; nt++) {
                            const int n = 8 * nt + 2 * q;
                            float z0 = acc[mt][nt][2 * half], z1 = acc[mt][nt][2 * half + 1];
                            if (MODE == kSgRelu || MODE == kSgResidual) {
                                z0 = fmaxf(z0 + bias0[nt], 0.0f);
                                z1 = fmaxf(z1 + bias1[nt], 0.0f);
                            }
                            if (MODE == kSgResidual && a.aux)
                                *reinterpret_cast<__nv_bfloat162 *>(&a.aux[p * COUT + n]) = __floats2bfloat162_rn(z0, z1);
                            if (MODE == kSgResidual || MODE == kSgLinearAdd) {
                                const __nv_bfloat162 rv = res_staged
                                                              ? *reinterpret_cast<const __nv_bfloat162 *>(&srow[n])
                                                              : *reinterpret_cast<const __nv_bfloat162 *>(&a.res[p * COUT + n]);
                                z0 += __bfloat162float(rv.x);
                                z1 += __bfloat162float(rv.y);
                            }
                            *reinterpret_cast<__nv_bfloat162 *>(&a.out[p * COUT + n]) = __floats2bfloat162_rn(z0, z1);
                        }
                    }
                }
            }
        }
        __syncthreads();  // this stage is refilled by the next iteration's prefetch
        stage ^= 1;
    }
    cp_async_wait<0>();
}

// Weight gradient of a 3x3 conv:
//   dW[co][tap][ci] += sum_p g[p][co] * x[p + shift(tap)][ci],   db[co] += sum_p g[p][co].
// GEMM with M = COUT (rows co), N = 9*CIN (columns (tap, ci)), K = pixels.  Persistent: a CTA walks tiles
// with a grid stride and keeps its partial sums in registers; warp w owns the column tiles w, w+8, ...
// The operands are staged channel-major ([co][pixel], [ci][halo pixel]) with row strides of 4 and 20
// banks mod 32, so the 8 row groups of a fragment load hit disjoint bank quadruples.
template <int CIN, int COUT>
__global__ void __launch_bounds__(kSgThreads) sg_conv_wgrad(const bf16 *__restrict__ gout, int g_cstride,
                                                           const bf16 *__restrict__ x, int x_cstride, float *__restrict__ dw,
                                                           float *__restrict__ db, int nb, int H, int W, int tiles_x,
                                                           int tiles_per_img) {
    constexpr int GS = kSgNPix + 8;  // 264 bf16 = 132 words
    constexpr int XS = 360;          // >= 10*34; 180 words
    constexpr int NCOL = 9 * CIN;
    constexpr int MT = (COUT + 15) / 16;
    constexpr int NT_ALL = NCOL / 8;
    constexpr int NTW = (NT_ALL + 7) / 8;
    __shared__ __align__(16) bf16 s_g[MT * 16 * GS];
    __shared__ __align__(16) bf16 s_x[CIN * XS];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int g = lane >> 2, q = lane & 3;
    const long long total = (long long)nb * tiles_per_img;

    float acc[NTW][MT][4];
#pragma unroll
    for (int j = 0; j < NTW; j++)
#pragma unroll
        for (int mt = 0; mt < MT; mt++)
#pragma unroll
            for (int r = 0; r < 4; r++) acc[j][mt][r] = 0.0f;
    float bsum = 0.0f;

    for (long long tile = blockIdx.x; tile < total; tile += gridDim.x) {
        const int img = (int)(tile / tiles_per_img);
        const int t = (int)(tile - (long long)img * tiles_per_img);
        const int y0 = (t / tiles_x) * kSgTH, x0 = (t % tiles_x) * kSgTW;
        const size_t img_off = (size_t)img * H * W;
        for (int e = tid; e < MT * 16 * kSgNPix; e += kSgThreads) {
            const int co = e % (MT * 16), px = e / (MT * 16);
            const int gy = y0 + px / kSgTW, gx = x0 + px % kSgTW;
            bf16 v = __float2bfloat16(0.0f);
            if (co < COUT && gy < H && gx < W) v = gout[(img_off + (size_t)gy * W + gx) * g_cstride + co];
            s_g[co * GS + px] = v;
        }
        for (int e = tid; e < CIN * kSgHH * kSgHW; e += kSgThreads) {
            const int ci = e % CIN, px = e / CIN;
            const int gy = y0 + px / kSgHW - 1, gx = x0 + px % kSgHW - 1;
            bf16 v = __float2bfloat16(0.0f);
            if (gy >= 0 && gy < H && gx >= 0 && gx < W) v = x[(img_off + (size_t)gy * W + gx) * x_cstride + ci];
            s_x[ci * XS + px] = v;
        }
        __syncthreads();
        if (tid < COUT) {
            for (int px = 0; px < kSgNPix; px++) bsum += __bfloat162float(s_g[tid * GS + px]);
        }
#pragma unroll
        for (int j = 0; j < NTW; j++) {
            const int nt = warp + 8 * j;
            if (nt >= NT_ALL) break;
            const int col = nt * 8 + g;  // this lane's B column (tap, ci)
            const int tap = col / CIN, ci = col - tap * CIN;
            const int ky = tap / 3, kx = tap - 3 * ky;
            const bf16 *xb = &s_x[ci * XS + ky * kSgHW + kx];
#pragma unroll 4
            for (int kb = 0; kb < kSgNPix; kb += 16) {
                // B[k = pixel][n = col]; the pixel pairs (p0, p0+1) and (p0+8, p0+9) stay in one tile row
                const int p0 = kb + 2 * q, p1 = p0 + 8;
                const int i0 = (p0 / kSgTW) * kSgHW + p0 % kSgTW, i1 = (p1 / kSgTW) * kSgHW + p1 % kSgTW;
                const uint32_t b0 = (uint32_t)__bfloat16_as_ushort(xb[i0]) | ((uint32_t)__bfloat16_as_ushort(xb[i0 + 1]) << 16);
                const uint32_t b1 = (uint32_t)__bfloat16_as_ushort(xb[i1]) | ((uint32_t)__bfloat16_as_ushort(xb[i1 + 1]) << 16);
#pragma unroll
                for (int mt = 0; mt < MT; mt++) {
                    const bf16 *ga = &s_g[(16 * mt + g) * GS + kb + 2 * q];
                    mma_bf16(acc[j][mt], ld_u32(ga), ld_u32(ga + 8 * GS), ld_u32(ga + 8), ld_u32(ga + 8 * GS + 8), b0, b1);
                }
            }
        }
        __syncthreads();
    }
    if (tid < COUT) atomicAdd(&db[tid], bsum);
#pragma unroll
    for (int j = 0; j < NTW; j++) {
        const int nt = warp + 8 * j;
        if (nt >= NT_ALL) break;
#pragma unroll
        for (int mt = 0; mt < MT; mt++) {
#pragma unroll
            for (int r = 0; r < 4; r++) {
                const int co = 16 * mt + g + 8 * (r >> 1);
                const int cc = nt * 8 + 2 * q + (r & 1);
                if (co < COUT) atomicAdd(&dw[(size_t)co * NCOL + cc], acc[j][mt][r]);
            }
        }
    }
}

// g = dh where the stored ReLU output is positive, else 0 (the backward of relu; NHWC, n elements)
__global__ void sg_mask_grad(const bf16 *__restrict__ dh, const bf16 *__restrict__ relu, bf16 *__restrict__ g,
                             long long n) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) g[i] = __bfloat162float(relu[i]) > 0.0f ? dh[i] : __float2bfloat16(0.0f);
}

// W[cout][tap][cin] -> W'[cin_pad][8 - tap][cout_pad], the weights of the data-gradient conv
__global__ void sg_flip_weights(const bf16 *__restrict__ w, bf16 *__restrict__ wt, int cout, int cin, int cout_pad,
                                int cin_pad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= cin_pad * 9 * cout_pad) return;
    const int co = i % cout_pad, tap = (i / cout_pad) % 9, ci = i / (9 * cout_pad);
    bf16 v = __float2bfloat16(0.0f);
    if (co < cout && ci < cin) v = w[((size_t)co * 9 + (8 - tap)) * cin + ci];
    wt[i] = v;
}

// Adam (Kingma & Ba 2015) with decoupled per-parameter weight decay (Loshchilov & Hutter 2019, AdamW)
// on f32 master weights; also writes the bf16 copy the conv kernels read and, when ema is not null, the
// exponential moving average of the weights (ema = d * ema + (1 - d) * w).
__global__ void sg_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                        const float *__restrict__ grad, const float *__restrict__ decay, bf16 *__restrict__ w_bf16,
                        float *__restrict__ ema, float ema_decay, long long n, float lr, float beta1, float beta2,
                        float eps, float bc1, float bc2) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = grad[i];
    const float mi = beta1 * m[i] + (1.0f - beta1) * gi;
    const float vi = beta2 * v[i] + (1.0f - beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float wd = decay ? decay[i] : 0.0f;
    const float wi = w[i] - lr * ((mi / bc1) / (sqrtf(vi / bc2) + eps) + wd * w[i]);
    w[i] = wi;
    if (w_bf16) w_bf16[i] = __float2bfloat16(wi);
    if (ema) ema[i] = ema_decay * ema[i] + (1.0f - ema_decay) * wi;
}

__device__ __forceinline__ uint64_t sg_mix64(uint64_t z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// The network input: (u, N(0,1) noise, radius * radius_scale, 0 x 13) per pixel.  The noise is a
// Box-Muller transform of two 24-bit uniforms hashed (SplitMix64 finaliser) from the seed and the global
// pixel index, so a batch's noise field depends only on (seed, pixel).
__global__ void sg_make_input(const float *__restrict__ u, const float *__restrict__ radius, float radius_scale,
                              uint64_t seed, bf16 *__restrict__ x, long long n_px, long long px_per_img) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_px) return;
    const uint64_t h = sg_mix64(seed + 0x9E3779B97F4A7C15ull * (uint64_t)(i + 1));
    const float u1 = ((float)(h >> 40) + 0.5f) * (1.0f / 16777216.0f);
    const float u2 = ((float)((h >> 8) & 0xFFFFFFu) + 0.5f) * (1.0f / 16777216.0f);
    const float nz = sqrtf(-2.0f * logf(u1)) * cospif(2.0f * u2);
    const float r = radius[i / px_per_img] * radius_scale;
    __align__(16) bf16 v[16];
#pragma unroll
    for (int c = 0; c < 16; c++) v[c] = __float2bfloat16(0.0f);
    v[0] = __float2bfloat16(u[i]);
    v[1] = __float2bfloat16(nz);
    v[2] = __float2bfloat16(r);
    uint4 *dst = reinterpret_cast<uint4 *>(x + i * 16);
    dst[0] = reinterpret_cast<const uint4 *>(v)[0];
    dst[1] = reinterpret_cast<const uint4 *>(v)[1];
}

// Mean squared error: dy16[p] = (scale * (y - t), 0 x 15) and loss += sum (y - t)^2.
__global__ void sg_mse_grad(const float *__restrict__ y, const float *__restrict__ t, bf16 *__restrict__ dy16,
                            float *__restrict__ loss, long long n, float scale) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    float e2 = 0.0f;
    if (i < n) {
        const float e = y[i] - t[i];
        e2 = e * e;
        __align__(16) bf16 v[16];
#pragma unroll
        for (int c = 0; c < 16; c++) v[c] = __float2bfloat16(0.0f);
        v[0] = __float2bfloat16(scale * e);
        uint4 *dst = reinterpret_cast<uint4 *>(dy16 + i * 16);
        dst[0] = reinterpret_cast<const uint4 *>(v)[0];
        dst[1] = reinterpret_cast<const uint4 *>(v)[1];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) e2 += __shfl_xor_sync(0xffffffffu, e2, o);
    __shared__ float s[8];
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = e2;
    __syncthreads();
    if (threadIdx.x == 0) {
        float tot = 0.0f;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) tot += s[w];
        atomicAdd(loss, tot);
    }
}

static SgConvArgs conv_args(const void *in, const void *w, const float *bias, const void *res, const float *res_f32,
                            void *out, void *aux, float *out_f32, int H, int W, int in_cstride) {
    SgConvArgs a;
    a.in = static_cast<const bf16 *>(in);
    a.w = static_cast<const bf16 *>(w);
    a.bias = bias;
    a.res = static_cast<const bf16 *>(res);
    a.res_f32 = res_f32;
    a.out = static_cast<bf16 *>(out);
    a.aux = static_cast<bf16 *>(aux);
    a.out_f32 = out_f32;
    a.H = H;
    a.W = W;
    a.in_cstride = in_cstride;
    a.tiles_x = (W + kSgTW - 1) / kSgTW;
    a.tiles_per_img = a.tiles_x * ((H + kSgTH - 1) / kSgTH);
    return a;
}

template <int CIN, int COUT, int MODE>
static cudaError_t launch_conv_t(const SgConvArgs &a, int total, cudaStream_t s) {
    constexpr int smem = sg_conv_smem_bytes<CIN, COUT>();
    auto k = sg_conv_fwd<CIN, COUT, MODE>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    int dev = 0, sms = 0, per_sm = 0;
    if (e == cudaSuccess) e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kSgThreads, smem);
    if (e != cudaSuccess) return e;
    const int grid = std::max(1, std::min(total, sms * std::max(1, per_sm)));
    k<<<grid, kSgThreads, smem, s>>>(a, total);
    return cudaGetLastError();
}

// fg_sg_tc.cu: the residual conv on the tcgen05 tensor cores (TMA-staged rows, accumulator in tensor
// memory); cudaErrorNotSupported when its preconditions fail.
cudaError_t launch_sg_conv32_tc(const void *in, const void *w, const float *bias, void *out, void *aux, int nb, int H,
                                int W, cudaStream_t s);

static fg_status launch_conv(int32_t kind, const SgConvArgs &a, int nb, cudaStream_t s) {
    const long long blocks = (long long)nb * a.tiles_per_img;
    if (blocks > 0x7FFFFFFFll) return set_error(FG_ERR_UNSUPPORTED, "surrogate batch too large");
    const int total = (int)blocks;
    cudaError_t e;
    switch (kind) {
    case FG_SG_CONV_INPUT: e = launch_conv_t<16, 32, kSgRelu>(a, total, s); break;
    case FG_SG_CONV_RESIDUAL:
        // the residual is the conv's own input (every residual layer of the network): tensor cores
        e = a.res == a.in && a.in_cstride == 32
                ? launch_sg_conv32_tc(a.in, a.w, a.bias, a.out, a.aux, nb, a.H, a.W, s)
                : cudaErrorNotSupported;
        if (e == cudaErrorNotSupported) {
            cudaGetLastError();
            e = launch_conv_t<32, 32, kSgResidual>(a, total, s);
        }
        break;
    case FG_SG_CONV_OUTPUT: e = launch_conv_t<32, 8, kSgOutput>(a, total, s); break;
    case FG_SG_CONV_DGRAD_RESIDUAL: e = launch_conv_t<32, 32, kSgLinearAdd>(a, total, s); break;
    case FG_SG_CONV_DGRAD_OUTPUT: e = launch_conv_t<16, 32, kSgLinear>(a, total, s); break;
    default: return set_error(FG_ERR_INVALID, "unknown surrogate conv kind");
    }
    return e == cudaSuccess ? FG_OK : cuda_error(e, "surrogate conv launch");
}

static bool aligned16(const void *p) { return p == nullptr || ((uintptr_t)p & 15u) == 0; }

}  // namespace fg

using namespace fg;

extern "C" {

FG_API fg_status fg_sg_conv_forward(int32_t kind, const void *in, int32_t in_cstride, const void *w, const float *bias,
                                    const void *res, const float *res_f32, void *out, void *aux, float *out_f32,
                                    int32_t nb, int32_t height, int32_t width, void *stream) {
    if (nb <= 0 || height <= 0 || width <= 0) return set_error(FG_ERR_INVALID, "empty surrogate batch");
    if (!in || !w || !aligned16(in) || !aligned16(w) || (in_cstride % 8) != 0)
        return set_error(FG_ERR_INVALID, "surrogate conv: input and weights must be 16-byte aligned");
    if (kind < FG_SG_CONV_INPUT || kind > FG_SG_CONV_DGRAD_OUTPUT)
        return set_error(FG_ERR_INVALID, "unknown surrogate conv kind");
    const bool f32_out = kind == FG_SG_CONV_OUTPUT;
    if ((!f32_out && !out) || (f32_out && (!out_f32 || !res_f32 || !bias)) ||
        ((kind == FG_SG_CONV_INPUT || kind == FG_SG_CONV_RESIDUAL) && !bias) ||
        ((kind == FG_SG_CONV_RESIDUAL || kind == FG_SG_CONV_DGRAD_RESIDUAL) && !res))
        return set_error(FG_ERR_INVALID, "surrogate conv: missing buffer");
    const int need_c = (kind == FG_SG_CONV_INPUT || kind == FG_SG_CONV_DGRAD_OUTPUT) ? 16 : 32;
    if (in_cstride < need_c) return set_error(FG_ERR_INVALID, "surrogate conv: input channel stride too small");
    const SgConvArgs a = conv_args(in, w, bias, res, res_f32, out, aux, out_f32, height, width, in_cstride);
    return launch_conv(kind, a, nb, (cudaStream_t)stream);
}

FG_API fg_status fg_sg_conv_wgrad(int32_t kind, const void *gout, int32_t g_cstride, const void *x, int32_t x_cstride,
                                  float *dw, float *db, int32_t nb, int32_t height, int32_t width, void *stream) {
    if (nb <= 0 || height <= 0 || width <= 0 || !gout || !x || !dw || !db)
        return set_error(FG_ERR_INVALID, "surrogate wgrad: bad arguments");
    const int tiles_x = (width + kSgTW - 1) / kSgTW;
    const int tiles_per_img = tiles_x * ((height + kSgTH - 1) / kSgTH);
    const long long total = (long long)nb * tiles_per_img;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return cuda_error(e, "surrogate wgrad: device query");
    const unsigned grid = (unsigned)std::max(1ll, std::min(total, (long long)std::max(1, sms) * 4));
    cudaStream_t s = (cudaStream_t)stream;
    auto G = static_cast<const bf16 *>(gout);
    auto X = static_cast<const bf16 *>(x);
    switch (kind) {
    case FG_SG_CONV_INPUT:
        if (g_cstride < 32 || x_cstride < 16) return set_error(FG_ERR_INVALID, "surrogate wgrad: channel stride");
        sg_conv_wgrad<16, 32><<<grid, kSgThreads, 0, s>>>(G, g_cstride, X, x_cstride, dw, db, nb, height, width, tiles_x,
                                                          tiles_per_img);
        break;
    case FG_SG_CONV_RESIDUAL:
        if (g_cstride < 32 || x_cstride < 32) return set_error(FG_ERR_INVALID, "surrogate wgrad: channel stride");
        sg_conv_wgrad<32, 32><<<grid, kSgThreads, 0, s>>>(G, g_cstride, X, x_cstride, dw, db, nb, height, width, tiles_x,
                                                          tiles_per_img);
        break;
    case FG_SG_CONV_OUTPUT:
        if (g_cstride < 8 || x_cstride < 32) return set_error(FG_ERR_INVALID, "surrogate wgrad: channel stride");
        sg_conv_wgrad<32, 8><<<grid, kSgThreads, 0, s>>>(G, g_cstride, X, x_cstride, dw, db, nb, height, width, tiles_x,
                                                         tiles_per_img);
        break;
    default:
        return set_error(FG_ERR_INVALID, "surrogate wgrad: unknown conv kind");
    }
    e = cudaGetLastError();
    return e == cudaSuccess ? FG_OK : cuda_error(e, "surrogate wgrad launch");
}

FG_API fg_status fg_sg_mask_grad(const void *dh, const void *relu, void *g, int64_t n, void *stream) {
    if (n <= 0) return FG_OK;
    if (!dh || !relu || !g) return set_error(FG_ERR_INVALID, "surrogate mask: null pointer");
    sg_mask_grad<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        static_cast<const bf16 *>(dh), static_cast<const bf16 *>(relu), static_cast<bf16 *>(g), n);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FG_OK : cuda_error(e, "surrogate mask launch");
}

FG_API fg_status fg_sg_flip_weights(const void *w, void *wt, int32_t cout, int32_t cin, int32_t cout_pad,
                                    int32_t cin_pad, void *stream) {
    if (!w || !wt || cout <= 0 || cin <= 0 || cout_pad < cout || cin_pad < cin)
        return set_error(FG_ERR_INVALID, "surrogate flip: bad arguments");
    const int n = cin_pad * 9 * cout_pad;
    sg_flip_weights<<<(n + 255) / 256, 256, 0, (cudaStream_t)stream>>>(static_cast<const bf16 *>(w),
                                                                      static_cast<bf16 *>(wt), cout, cin, cout_pad,
                                                                      cin_pad);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FG_OK : cuda_error(e, "surrogate flip launch");
}

FG_API fg_status fg_sg_adam(float *w, float *m, float *v, const float *grad, const float *decay, void *w_bf16,
                            float *ema, float ema_decay, int64_t n, float lr, float beta1, float beta2, float eps,
                            int32_t step, void *stream) {
    if (n <= 0 || step <= 0 || !w || !m || !v || !grad) return set_error(FG_ERR_INVALID, "surrogate adam: bad arguments");
    const float bc1 = 1.0f - powf(beta1, (float)step), bc2 = 1.0f - powf(beta2, (float)step);
    sg_adam<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(
        w, m, v, grad, decay, static_cast<bf16 *>(w_bf16), ema, ema_decay, n, lr, beta1, beta2, eps, bc1, bc2);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FG_OK : cuda_error(e, "surrogate adam launch");
}

FG_API fg_status fg_sg_make_input(const float *u, const float *radius, float radius_scale, uint64_t seed, void *x,
                                  int32_t nb, int32_t height, int32_t width, void *stream) {
    if (nb <= 0 || height <= 0 || width <= 0 || !u || !radius || !x || !aligned16(x))
        return set_error(FG_ERR_INVALID, "surrogate input: bad arguments");
    const long long px_img = (long long)height * width, n = px_img * nb;
    sg_make_input<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(u, radius, radius_scale, seed,
                                                                                static_cast<bf16 *>(x), n, px_img);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FG_OK : cuda_error(e, "surrogate input launch");
}

FG_API fg_status fg_sg_mse_grad(const float *y, const float *target, void *dy16, float *loss_sum, int64_t n,
                                float scale, void *stream) {
    if (n <= 0 || !y || !target || !dy16 || !loss_sum || !aligned16(dy16))
        return set_error(FG_ERR_INVALID, "surrogate loss: bad arguments");
    sg_mse_grad<<<(unsigned)((n + 255) / 256), 256, 0, (cudaStream_t)stream>>>(y, target, static_cast<bf16 *>(dy16),
                                                                              loss_sum, n, scale);
    const cudaError_t e = cudaGetLastError();
    return e == cudaSuccess ? FG_OK : cuda_error(e, "surrogate loss launch");
}

FG_API size_t fg_sg_infer_workspace_bytes(int32_t nb, int32_t height, int32_t width) {
    if (nb <= 0 || height <= 0 || width <= 0) return 0;
    const size_t px = (size_t)nb * height * width;
    return px * (16 + 32 + 32) * sizeof(uint16_t) + 256;
}

FG_API fg_status fg_sg_infer(const fg_sg_net *net, const float *u, const float *radius, uint64_t seed, float *out,
                             int32_t nb, int32_t height, int32_t width, void *workspace, size_t workspace_bytes,
                             void *stream) {
    if (!net || !u || !radius || !out || !workspace) return set_error(FG_ERR_INVALID, "surrogate infer: null pointer");
    if (nb <= 0 || height <= 0 || width <= 0) return set_error(FG_ERR_INVALID, "surrogate infer: empty batch");
    if (net->n_res < 0 || net->n_res > 64 || !net->w_in || !net->b_in || !net->w_out || !net->b_out ||
        (net->n_res > 0 && (!net->w_res || !net->b_res)) || !aligned16(net->w_in) || !aligned16(net->w_res) ||
        !aligned16(net->w_out))
        return set_error(FG_ERR_INVALID, "surrogate infer: incomplete or misaligned network");
    if (workspace_bytes < fg_sg_infer_workspace_bytes(nb, height, width))
        return set_error(FG_ERR_INVALID, "surrogate infer: workspace too small");
    cudaStream_t s = (cudaStream_t)stream;
    const size_t px = (size_t)nb * height * width;
    const uintptr_t base = ((uintptr_t)workspace + 255) & ~(uintptr_t)255;
    bf16 *x = reinterpret_cast<bf16 *>(base);
    bf16 *h0 = x + px * 16;
    bf16 *h1 = h0 + px * 32;
    fg_status st = fg_sg_make_input(u, radius, net->radius_scale, seed, x, nb, height, width, stream);
    if (st != FG_OK) return st;
    st = launch_conv(FG_SG_CONV_INPUT,
                     conv_args(x, net->w_in, net->b_in, nullptr, nullptr, h0, nullptr, nullptr, height, width, 16), nb, s);
    const bf16 *w_res = static_cast<const bf16 *>(net->w_res);
    for (int l = 0; l < net->n_res && st == FG_OK; l++) {
        st = launch_conv(FG_SG_CONV_RESIDUAL,
                         conv_args(h0, w_res + (size_t)l * 32 * 9 * 32, net->b_res + 32 * l, h0, nullptr, h1, nullptr,
                                   nullptr, height, width, 32), nb, s);
        std::swap(h0, h1);
    }
    if (st != FG_OK) return st;
    return launch_conv(FG_SG_CONV_OUTPUT,
                       conv_args(h0, net->w_out, net->b_out, nullptr, u, nullptr, nullptr, out, height, width, 32), nb, s);
}

}  // extern "C"
