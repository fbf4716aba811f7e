// fg_kernels.cuh -- launch descriptors shared by the kernels and the C-ABI layer.
#pragma once
#include <stdint.h>
#include <cuda_runtime.h>

namespace fg {

// Per input pixel: the Poisson set-up of a pixel-wise cell whose lambda lookup lands on the pixel
// (src/pixelwise.rs:69-82).  `thresh` turns the first Knuth comparison into an integer test on the
// first draw's 53-bit value v: U1 = v * 2^-53 > exp_lambda  <=>  v > floor(exp_lambda * 2^53), so
// v <= thresh means q = 0.  thresh = INT64_MAX means "no grains" (lambda <= 0 or
// lambda*delta*delta <= 0, the cell is skipped without drawing); thresh = -1 marks the rejection
// regime (lambda*delta^2 >= 12), where exp_lambda holds -expected.
struct __align__(16) CellParam {
    long long thresh;
    double exp_lambda;
};

// Shared-memory capacities of the pixel-wise tile kernel.
constexpr int kPwCellMax = 8192;   // staged window cells
// Shared-memory configurations of the pixel-wise block: lean CTAs (256 threads, 4 per SM) take every
// block first and defer the dense ones; fat CTAs (512 threads, 2 per SM) take the deferred blocks
// (and every block of the batched and allocation-free paths).
struct PwLean {
    static constexpr int kThreads = 256, kCtasPerSm = 4, kGrainMax = 1024, kListMax = 2048;
    static constexpr bool kDefers = true;
};
struct PwFat {
    static constexpr int kThreads = 512, kCtasPerSm = 2, kGrainMax = 4096, kListMax = 8192;
    static constexpr bool kDefers = false;
};
constexpr int kPwEdgeMax = 128;    // window cells per axis
constexpr int kPwKChunk = 256;     // offsets per sample-assignment chunk
constexpr int kPwFootMax = 1024;   // per-block output-pixel counters
constexpr int kPwMaxLevel = 3;     // block subdivision depth on grain overflow
// Pixel-wise diagnostic counters (PixelwiseArgs::diag): [0] samples evaluated on the per-sample path,
// [1] blocks without a staged window, [2] block subdivisions, [3] blocks run, [4] sparse blocks whose
// samples ran sample-major, [5] sparse blocks that ran grain-major.
constexpr int kPwDiagWords = 6;
// A block regenerates per sample (no staging) when its samples' reach, in cells, is below
// kPwRegenSparse x its window's cells, or below kPwRegenOverflow x them once the window overflows
// with more than kPwRegenDense of its cells non-empty.
constexpr float kPwRegenSparse = 1.0f;
constexpr float kPwRegenOverflow = 4.0f;
constexpr float kPwRegenDense = 0.4f;
// The per-sample kernel replaces the block kernel for a whole plane when an interior root block's
// samples reach fewer than kPwRegenKernel x its window's cells (and a sample's range fits 64 cells).
constexpr int kPwRegenThreads = 256;
constexpr float kPwRegenKernel = 1.5f;
// Forms of the per-sample kernel by a warp's expected grains per cell (λδ²), from timings of uniform
// planes (r 0.025-0.1, N 16-256): lane-major dealing up to 0.3, rank-major dealing up to 1.1 (u 0.7:
// 11 % faster, u 0.9: 27 % faster than its neighbours), the flattened loop above (u 0.99).
constexpr float kPwRegenRankLd = 0.3f;
constexpr float kPwRegenFlatLd = 1.1f;

// In-launch cancellation: `cancel` is null or two words of mapped pinned host memory.  Word 0 is set
// by the library's host watcher once the caller's cancel flag turns non-zero; the persistent passes
// read it once per work item they pull (the block passes once per block) and stop, and a CTA that
// stops on it sets word 1.
#ifdef __CUDACC__
__device__ __forceinline__ bool cancel_requested(int *cancel) {
    if (!cancel || *(volatile int *)cancel == 0) return false;
    *(volatile int *)(cancel + 1) = 1;
    return true;
}
#endif

struct PixelwiseArgs {
    const float *lam;           // in_w x in_h
    const CellParam *cells;     // in_w x in_h
    const float2 *offs;         // offsets_input [n]
    float *out;                 // out_w x out_h, accumulates hit counts (pre-zeroed)
    unsigned long long *diag;   // [4] counters: regenerated samples, unstaged blocks, subdivisions, blocks
    int in_w, in_h, out_w, out_h;
    int n;
    float rm, delta, inv_zoom, zoom;
    float regen_cells;          // mean cells one sample's own loop visits: (2 rm / delta + 1)^2
    float bsize, inv_bsize;     // block edge in input pixels (power of two) and its inverse
    int bx0, by0, nbx;          // block-grid origin and width
    float offx_min, offx_max, offy_min, offy_max;
    unsigned long long seed;
    int lognorm;
    float radius_mean;
    double log_mu, log_sigma;
    int *cancel;                // null, or the in-launch cancellation words (cancel_requested)
    // null, or the plane's emptiness bitmask (the sparse pass's first_draw_screen of every cell):
    // cells [cm_gi0, cm_gi0 + cm_gw) x [cm_gj0, cm_gj0 + 32 cm_ghw), word (c, k) = cellmask[k * cm_gw + c]
    // holding rows cm_gj0 + 32k .. + 31 of column cm_gi0 + c
    const unsigned int *cellmask;
    int cm_gi0, cm_gj0, cm_gw, cm_ghw;
};

constexpr int kGwBucketCount = 256;  // bucket index over the frac(offx)-sorted offsets

struct GrainwiseArgs {
    const float *lam;           // in_w x in_h
    const float4 *sorted_offs;  // [n] (frac(offy), offx, offy, k as int bits), ascending frac(offx)
    const int *bucket_start;    // [kGwBucketCount + 1]: first entry with frac(offx) >= b / kGwBucketCount
    unsigned int *gmask;        // out_w x out_h x words sample masks (zeroed before the launch)
    int in_w, in_h, out_w, out_h;
    int n, words;               // words = ceil(n/32)
    int tin_w, tin_h;           // input tile of one CTA
    int rmax_w, rmax_h;         // bound of the zoomed tile rectangle held in shared memory
    float rm, zoom;
    float offx_min, offx_max, offy_min, offy_max;
    float frac_eps;             // rounding margin of the candidate-offset intervals
    unsigned long long seed;
    int lognorm;
    float radius_mean;
    double log_mu, log_sigma;
    int *work;                  // null: one CTA per tile; else the tile scheduler's area (grainwise_work_ints)
    int parts;                  // CTAs per tile (>= 1; above 1 only for the bitmask variants)
    int *cancel;                // null, or the in-launch cancellation words (cancel_requested)
};

// popcount / colour epilogue of the grain-wise path.
struct GrainwiseEpilogueArgs {
    const unsigned int *gmask;  // planes x out_w x out_h x words
    float *out;                 // planes x out_w x out_h values (may be null)
    unsigned char *out_rgb8;    // null, or u8 RGB (mode 1 / 2)
    const float *cb, *cr;       // luma: chroma planes at input size
    int out_w, out_h, in_w, in_h;
    int n, words;
    int mode;                   // 0 values of one plane, 1 luma recombination, 2 pack of three planes
};

// Epilogue of the pixel-wise path: counts -> value (and optional colour packing).
struct EpilogueArgs {
    float *plane;               // counts in, values out (in place)
    int out_w, out_h, in_w, in_h;
    float inv_samples;
    unsigned char *out_rgb8;    // null: values only
    int mode;                   // 0 values, 1 luma recombine, 2 rgb pack (plane is channel 2)
    const float *cb, *cr;       // luma: chroma planes at input size
    const float *p0, *p1;       // rgb: rendered channels 0 and 1 (values)
};

// The platform-logf table on the device (fg_lambda.cu platform_logf).
struct LogfTableDev {
    const uint32_t *bucket_start, *keys, *vals;
    uint32_t lo_bits, hi_bits;
    int shift;
};

cudaError_t launch_cell_params(const float *lam, int in_w, int in_h, float delta, CellParam *cells, cudaStream_t s);
// defer: null (fat CTAs over every block) or a buffer of 2 + nbx*nby ints (lean pass, then fat CTAs
// over the deferred blocks).
// cellmask: null, or pixelwise_cellmask_bytes(a, nby) bytes for the sparse pass's plane bitmask (the
// plane then takes the sparse pass, else the lean pass).
cudaError_t launch_pixelwise(const PixelwiseArgs &a, int nby, int *defer, unsigned int *cellmask, cudaStream_t s);
// Scratch bytes of the sparse pass's plane bitmask for this plane; 0 when the plane does not take it.
size_t pixelwise_cellmask_bytes(const PixelwiseArgs &a, int nby);
// Whether a plane runs on the per-sample kernel instead of the block kernel, and its launch.
bool pixelwise_prefers_regen(const PixelwiseArgs &a);
cudaError_t launch_pixelwise_regen(const PixelwiseArgs &a, cudaStream_t s);
size_t pixelwise_smem_bytes();  // the fat configuration (the batched kernel's pixel-wise items)
cudaError_t launch_grainwise(const GrainwiseArgs &a, cudaStream_t s);
size_t grainwise_smem_bytes(const GrainwiseArgs &a);
int grainwise_tile_count(const GrainwiseArgs &a);
size_t grainwise_work_ints(const GrainwiseArgs &a);  // scheduler area: counter, pad, order[tiles], cost[tiles]
int grainwise_parts(const GrainwiseArgs &a, int sms);
cudaError_t launch_grainwise_epilogue(const GrainwiseEpilogueArgs &a, cudaStream_t s);
cudaError_t launch_epilogue(const EpilogueArgs &a, cudaStream_t s);
cudaError_t launch_rgb_pack(const float *p0, const float *p1, const float *p2, int n, unsigned char *out,
                            cudaStream_t s);

}  // namespace fg
