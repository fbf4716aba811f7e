// fg_sg_tc.cu -- the surrogate's 32 -> 32 residual conv on the fifth-generation tensor cores.
//
// h' = h + relu(conv3x3(h) + b), NHWC bf16 activations with 32 channels, weights [cout 32][tap 9][cin 32]
// bf16, f32 accumulation.  An implicit GEMM with M = 128 output pixels (one row segment), N = 32 output channels,
// K = 9 taps x 32 input channels, issued as 18 tcgen05.mma (kind::f16, M 128, N 32, K 16) by one thread,
// the accumulator in tensor memory (32 columns).
//
// A CTA (128 threads) owns 128 columns of kTcRows consecutive rows of one image.  Its input rows (the
// 130-pixel halo row: columns x0 - 1 .. x0 + 128) arrive by TMA (cp.async.bulk.tensor, one box per
// 8-channel chunk, zero-filled outside the image) into a ring of four row slots, each laid out
// chunk-major: chunk c of a row holds its 130 pixels' channels 8c .. 8c + 7 at 16 bytes per pixel.  That
// is the tensor cores' K-major no-swizzle layout read with 8-pixel core matrices 128 bytes apart (the
// descriptor's stride offset) and 8-channel chunks one chunk apart (its leading offset), so the A operand
// of tap (ky, kx) is the row slot of input row y + ky - 1 started kx pixels in: no data moves per tap.
// The weights sit in the same layout ([k chunk 36][cout 32][8]) for the whole CTA.  The next row's TMA
// overlaps the current row's MMAs and epilogue; the epilogue reads the accumulator back with
// tcgen05.ld (warp w: pixels 32w .. 32w + 31, one pixel's 32 channels per thread), adds bias, applies
// the ReLU, adds the residual (the input row's centre pixel, already in shared memory) and stores 64
// bytes per pixel.
//
// Every wait on an mbarrier is bounded; a wait that runs out records the fact in g_sg_tc_timeout,
// writes NaN outputs for the rest of the CTA's rows, waits (bounded) for its own copies and MMAs, frees
// its tensor memory and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>
#include <stdint.h>

#include <mutex>

#include "fg_internal.h"

namespace fg {

typedef __nv_bfloat16 bf16;

constexpr int kTcPx = 128;                    // output pixels of one row tile (the MMA's M)
constexpr int kTcHalo = kTcPx + 2;            // input pixels of one halo row
constexpr int kTcChunkBytes = 2176;           // one 8-channel chunk of a halo row: 130 x 16 B, to 128 B
constexpr int kTcBoxBytes = kTcHalo * 16;     // bytes one TMA box writes
constexpr int kTcRowBytes = 4 * kTcChunkBytes;
constexpr int kTcSlots = 4;
constexpr int kTcWOff = kTcSlots * kTcRowBytes;  // 34816
constexpr int kTcWBytes = 36 * 32 * 16;          // 18432
constexpr int kTcBarOff = kTcWOff + kTcWBytes;   // 53248
constexpr int kTcSmem = kTcBarOff + 64;
constexpr int kTcRows = 16;                   // output rows per CTA
constexpr int kTcThreads = 128;
constexpr uint32_t kTcTmemCols = 32;
// SM cycles a wait on an mbarrier may take before it gives up (about a second)
constexpr long long kTcWaitCycles = 2000000000ll;

__device__ int g_sg_tc_timeout;

// Instruction descriptor of tcgen05.mma kind::f16: D f32 (bits 4-5 = 1), A and B bf16 (bits 7-9 and
// 10-12 = 1), both K-major (bits 15, 16 = 0), N >> 3 at bit 17, M >> 4 at bit 24.
constexpr uint32_t kTcIdesc = (1u << 4) | (1u << 7) | (1u << 10) | ((32u >> 3) << 17) | ((128u >> 4) << 24);

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Shared-memory matrix descriptor, no swizzle: start address, leading (K-direction core-matrix) byte
// offset, stride (M/N-direction core-matrix) byte offset, each >> 4; descriptor version 1 at bit 46.
__device__ __forceinline__ uint64_t tc_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(bar), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}
// Bounded wait for the completion of the phase with the given parity (non-blocking polls against the
// SM clock); false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
    const long long t0 = clock64();
    for (;;) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
        if (clock64() - t0 > kTcWaitCycles) return false;
    }
}

// One halo row (input row y, all 32 channels) into row slot `slot`: four boxes of (8 channels, 1 chunk,
// 130 pixels, 1 row, 1 image) at x = x0 - 1.
__device__ __forceinline__ void tma_row(const CUtensorMap *tm, uint32_t sbase, int slot, int x0, int y, int img,
                                        uint32_t bar) {
    mbar_expect_tx(bar, 4 * kTcBoxBytes);
    const uint64_t desc = reinterpret_cast<uint64_t>(tm);
#pragma unroll
    for (int c = 0; c < 4; c++) {
        const uint32_t dst = sbase + (uint32_t)(slot * kTcRowBytes + c * kTcChunkBytes);
        asm volatile(
            "cp.async.bulk.tensor.5d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, "
            "%6}], [%7];\n" ::"r"(dst),
            "l"(desc), "r"(0), "r"(c), "r"(x0 - 1), "r"(y), "r"(img), "r"(bar)
            : "memory");
    }
}

// out = in + relu(conv(in) + b); aux (when not null) = relu(conv(in) + b), the ReLU output training keeps
__global__ void __launch_bounds__(kTcThreads) sg_conv32_tc_kernel(const __grid_constant__ CUtensorMap tmap,
                                                                  const bf16 *__restrict__ w,
                                                                  const float *__restrict__ bias, bf16 *__restrict__ out,
                                                                  bf16 *__restrict__ aux, int H, int W, int tiles_x,
                                                                  int strips) {
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    int b = (int)blockIdx.x;
    const int tx = b % tiles_x;
    b /= tiles_x;
    const int strip = b % strips, img = b / strips;
    const int x0 = tx * kTcPx, y0 = strip * kTcRows;
    const int nrows = min(kTcRows, H - y0);
    const uint32_t sbase = smem_u32(tc_smem);
    const uint32_t bar0 = sbase + kTcBarOff, mma_bar = bar0 + 8 * kTcSlots, tmem_slot = mma_bar + 8;
    volatile int *s_abort = reinterpret_cast<volatile int *>(tc_smem + kTcBarOff + 8 * kTcSlots + 12);

    if (tid == 0) {
        for (int s = 0; s < kTcSlots; s++) mbar_init(bar0 + 8 * s, 1);
        mbar_init(mma_bar, 1);
        *s_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(tmem_slot),
                     "r"(kTcTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
    }
    // weights: element (n, k = tap * 32 + ci) to chunk k / 8, row n
    for (int e = tid; e < 32 * 36; e += kTcThreads) {
        const int n = e / 36, kc = e - n * 36;
        const uint4 v = *reinterpret_cast<const uint4 *>(w + n * 288 + kc * 8);
        *reinterpret_cast<uint4 *>(tc_smem + kTcWOff + (kc * 32 + n) * 16) = v;
    }
    float bv[32];
#pragma unroll
    for (int n = 0; n < 32; n++) bv[n] = bias[n];
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");  // the weights, for the tensor cores
    asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    const uint32_t tmem = *reinterpret_cast<volatile uint32_t *>(tc_smem + kTcBarOff + 8 * kTcSlots + 8);

    // input row i (i = 0 .. nrows + 1) is image row y0 - 1 + i, in slot i % 4; its barrier completes its
    // (i / 4)-th phase
    // (thread 0's bookkeeping, for a clean exit after a failed wait: the last row issued, the last row
    // whose barrier every thread saw complete, the MMA commits issued and waited for)
    int last_issued = -1, last_seen = -1, commits = 0, commits_seen = 0;
    if (tid == 0)
        for (int i = 0; i < 3; i++) tma_row(&tmap, sbase, i, x0, y0 - 1 + i, img, bar0 + 8 * i);
    last_issued = 2;

    bool ok = true;
    int r = 0;
    for (; r < nrows; r++) {
        if (tid == 0 && r + 3 <= nrows + 1) {
            const int i = r + 3;
            tma_row(&tmap, sbase, i % kTcSlots, x0, y0 - 1 + i, img, bar0 + 8 * (i % kTcSlots));
            last_issued = i;
        }
        for (int i = (r == 0 ? 0 : r + 2); i <= r + 2; i++) {
            if (mbar_wait(bar0 + 8 * (i % kTcSlots), (uint32_t)((i / kTcSlots) & 1))) last_seen = i;
            else *s_abort = 1;
        }
        if (tid == 0 && !*s_abort) {
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
            for (int tap = 0; tap < 9; tap++) {
                const int ky = tap / 3, kx = tap - 3 * ky;
                const uint32_t arow = sbase + (uint32_t)(((r + ky) % kTcSlots) * kTcRowBytes + kx * 16);
#pragma unroll
                for (int j = 0; j < 2; j++) {
                    const uint64_t ad = tc_desc(arow + (uint32_t)(2 * j * kTcChunkBytes), kTcChunkBytes, 128);
                    const uint64_t bd = tc_desc(sbase + (uint32_t)(kTcWOff + (tap * 4 + 2 * j) * 512), 512, 128);
                    const uint32_t acc = (tap | j) != 0 ? 1u : 0u;
                    asm volatile(
                        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
                        "l"(ad), "l"(bd), "r"(kTcIdesc), "r"(acc)
                        : "memory");
                }
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(mma_bar)
                         : "memory");
            commits++;
        }
        __syncthreads();  // every thread has seen the rows (or the abort) before anyone tests the flag
        if (*s_abort) {
            ok = false;
            break;
        }
        if (mbar_wait(mma_bar, (uint32_t)(r & 1))) commits_seen = r + 1;
        else *s_abort = 1;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        uint32_t v[32];
        asm volatile(
            "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
            "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n"
            : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
              "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
              "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
              "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
            : "r"(tmem + ((uint32_t)(warp * 32) << 16)));
        asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
        const int m = warp * 32 + lane, x = x0 + m, y = y0 + r;
        if (x < W) {
            const bool bad = *s_abort != 0;
            const unsigned char *rp = tc_smem + ((r + 1) % kTcSlots) * kTcRowBytes + (m + 1) * 16;
            const size_t p = ((size_t)img * H + y) * W + x;
#pragma unroll
            for (int c = 0; c < 4; c++) {
                const uint4 rv = *reinterpret_cast<const uint4 *>(rp + c * kTcChunkBytes);
                const __nv_bfloat162 *r2 = reinterpret_cast<const __nv_bfloat162 *>(&rv);
                uint4 ov, av;
                __nv_bfloat162 *o2 = reinterpret_cast<__nv_bfloat162 *>(&ov);
                __nv_bfloat162 *a2 = reinterpret_cast<__nv_bfloat162 *>(&av);
#pragma unroll
                for (int q = 0; q < 4; q++) {
                    const int n = 8 * c + 2 * q;
                    float z0 = __uint_as_float(v[n]), z1 = __uint_as_float(v[n + 1]);
                    z0 = fmaxf(z0 + bv[n], 0.0f);
                    z1 = fmaxf(z1 + bv[n + 1], 0.0f);
                    a2[q] = __floats2bfloat162_rn(z0, z1);
                    const float2 rf = __bfloat1622float2(r2[q]);
                    z0 += rf.x;
                    z1 += rf.y;
                    if (bad) z0 = z1 = __int_as_float(0x7fc00000);
                    o2[q] = __floats2bfloat162_rn(z0, z1);
                }
                *reinterpret_cast<uint4 *>(out + p * 32 + 8 * c) = ov;
                if (aux) *reinterpret_cast<uint4 *>(aux + p * 32 + 8 * c) = av;
            }
        }
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        __syncthreads();  // the accumulator and the oldest row slot are free again
        if (*s_abort) {
            ok = false;
            r++;
            break;
        }
    }
    if (!ok) {
        if (tid == 0) atomicExch(&g_sg_tc_timeout, 1);
        // rows this CTA still owns: NaN, so that a failed launch cannot pass for a result
        for (int rr = r; rr < nrows; rr++) {
            const int x = x0 + tid;
            if (x < W) {
                const size_t p = ((size_t)img * H + y0 + rr) * W + x;
                const uint4 nan4 = make_uint4(0x7fc07fc0u, 0x7fc07fc0u, 0x7fc07fc0u, 0x7fc07fc0u);
                for (int c = 0; c < 4; c++) *reinterpret_cast<uint4 *>(out + p * 32 + 8 * c) = nan4;
            }
        }
        // the copies and MMAs this CTA issued must land before its shared and tensor memory are released:
        // the rows issued but not yet seen (at most the two newest; each slot holds one), and the last
        // commit when it was not waited for
        if (tid == 0) {
            for (int i = max(last_seen + 1, last_issued - 1); i <= last_issued; i++)
                (void)mbar_wait(bar0 + 8 * (i % kTcSlots), (uint32_t)((i / kTcSlots) & 1));
            if (commits > commits_seen) (void)mbar_wait(mma_bar, (uint32_t)((commits - 1) & 1));
        }
        __syncthreads();
    }
    if (warp == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTcTmemCols)
                     : "memory");
    }
}

static PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static std::once_flag once;
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    std::call_once(once, [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
        else
            cudaGetLastError();
    });
    return fn;
}

// The residual conv on the tensor cores: out = in + relu(conv(in) + b) (aux = the ReLU output when not
// null), 32 channels per pixel, out distinct from in.  Returns cudaErrorNotSupported when the tensor
// map cannot be made (the caller's mma.sync kernel runs instead).
cudaError_t launch_sg_conv32_tc(const void *in, const void *w, const float *bias, void *out, void *aux, int nb, int H,
                                int W, cudaStream_t s) {
    if (nb <= 0 || H <= 0 || W <= 0) return cudaSuccess;
    if ((reinterpret_cast<uintptr_t>(in) & 15u) || (reinterpret_cast<uintptr_t>(w) & 15u) ||
        (reinterpret_cast<uintptr_t>(out) & 15u) || (reinterpret_cast<uintptr_t>(aux) & 15u) || in == out)
        return cudaErrorNotSupported;
    PFN_cuTensorMapEncodeTiled_v12000 encode = tensor_map_encoder();
    if (!encode) return cudaErrorNotSupported;
    CUtensorMap tm;
    const cuuint64_t dims[5] = {8, 4, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)nb};
    const cuuint64_t strides[4] = {16, 64, (cuuint64_t)W * 64, (cuuint64_t)H * W * 64};
    const cuuint32_t box[5] = {8, 1, (cuuint32_t)kTcHalo, 1, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    if (encode(&tm, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<void *>(in), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return cudaErrorNotSupported;
    const int tiles_x = (W + kTcPx - 1) / kTcPx, strips = (H + kTcRows - 1) / kTcRows;
    const long long grid = (long long)tiles_x * strips * nb;
    if (grid > 0x7FFFFFFFll) return cudaErrorNotSupported;
    const cudaError_t e = cudaFuncSetAttribute(sg_conv32_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kTcSmem);
    if (e != cudaSuccess) return e;
    sg_conv32_tc_kernel<<<(unsigned)grid, kTcThreads, kTcSmem, s>>>(tm, static_cast<const bf16 *>(w), bias,
                                                                      static_cast<bf16 *>(out), static_cast<bf16 *>(aux),
                                                                      H, W, tiles_x, strips);
    return cudaGetLastError();
}

// Whether a tensor-core conv ran out of an mbarrier wait since the last call (and clears the flag).
int sg_conv32_tc_timeouts() {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_sg_tc_timeout, sizeof v) != cudaSuccess) {
        cudaGetLastError();
        return -1;
    }
    const int z = 0;
    cudaMemcpyToSymbol(g_sg_tc_timeout, &z, sizeof z);
    return v;
}

}  // namespace fg
