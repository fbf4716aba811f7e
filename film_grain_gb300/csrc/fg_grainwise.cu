// fg_grainwise.cu -- the grain-wise integrator (src/grainwise.rs:12-142) for sm_103a.
//
// The reference walks input pixels, draws Poisson(lambda) grains from each pixel's stream, and for
// every grain and offset k ORs bit k into the 64-bit sample masks of the output pixels whose centres
// fall in the offset disk (AtomicU64::fetch_or), then popcounts the masks.  Here one CTA owns an
// output tile and keeps its N-bit masks in shared memory (ceil(N/32) words per pixel).  It
// regenerates the grains of every input pixel whose offset disks can reach the tile (pixel streams
// are deterministic, so tiles never exchange grains), rasterises them with the reference's exact
// bounds() and centre test, and finishes with the popcount * (1/N) epilogue -- optionally fused
// with the luma colour recombination and u8 packing.
//
// Work organisation:
//   - each warp takes 32 footprint pixels at a time (one per lane, Poisson set-up in step) and
//     draws their grains one per lane per step; valid grains are compacted into a 64-entry warp
//     queue with a ballot, and every full batch of 32 is rasterised grain by grain by the whole warp;
//   - an offset can put a pixel centre inside a grain's disk only if frac(czx + offx) lies within
//     radius_out of 1/2 (and likewise for y).  For N <= 256 each lane turns both tests, widened by a
//     rounding margin and rounded out to 1/128 buckets, into a bitmask over the sample index (two
//     lookups per axis in per-tile sparse OR tables), ANDs them, and the set bits -- about 1.2x the
//     true candidates -- go through the warp's list to stage B.  For larger N the offsets are sorted
//     by frac(offx), the cyclic interval of the sorted table around frac(1/2 - czx) is flattened over
//     the lanes (stage A) and filtered by the y test.  Stage B runs the reference's exact bounds()
//     and centre tests on the pairs, one pair per lane;
//   - the lognormal radius is evaluated with the double-float exp (exp_f64_to_f32).
// Bits are set with shared-memory atomicOr; OR is idempotent and commutative, so the result does not
// depend on the order.
#include "fg_kernels.cuh"
#include "fg_rng.cuh"
#include "fg_color.cuh"
#include "fg_grainwise.cuh"
#include "fg_internal.h"

#include <algorithm>

namespace fg {

template <bool kSmall, int kVariant>
__global__ void __launch_bounds__(kGwThreads, 2) grainwise_kernel(const __grid_constant__ GrainwiseArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    grainwise_tile<kSmall, kVariant>(a, blockIdx.x, blockIdx.y, smem_raw, blockIdx.z, a.parts);
}

// Persistent form: CTAs pull tiles from the scheduler's list (a.work[2..], heaviest first) through the
// counter a.work[0] until the list is exhausted.
template <bool kSmall, int kVariant>
__global__ void __launch_bounds__(kGwThreads, 2) grainwise_persistent_kernel(const __grid_constant__ GrainwiseArgs a,
                                                                             int ntx, int ntiles) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_tile;
    const int parts = a.parts;
    for (;;) {
        if (threadIdx.x == 0) {
            const int i = atomicAdd(a.work, 1);  // item i: part i % parts of the (i / parts)-th tile
            s_tile = (i < ntiles * parts && !cancel_requested(a.cancel)) ? i : -1;
        }
        __syncthreads();
        const int i = s_tile;
        if (i < 0) break;
        const int t = a.work[2 + i / parts];
        grainwise_tile<kSmall, kVariant>(a, t % ntx, t / ntx, smem_raw, i % parts, parts);
        __syncthreads();
    }
}

// Expected cost of each input tile (one warp per tile): its grains (sum of lambda) plus a per-pixel
// set-up term.
__global__ void grainwise_costs_kernel(const float *__restrict__ lam, int in_w, int in_h, int tin_w, int tin_h, int ntx,
                                       int ntiles, float *__restrict__ cost) {
    const int tile = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (tile >= ntiles) return;
    const int x0 = (tile % ntx) * tin_w, y0 = (tile / ntx) * tin_h;
    const int w = min(x0 + tin_w, in_w) - x0, n = w * (min(y0 + tin_h, in_h) - y0);
    float sum = 0.0f;
    for (int i = lane; i < n; i += 32) sum += lam[(long long)(y0 + i / w) * in_w + x0 + i % w];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) cost[tile] = sum + 4.0f * (float)n;
}

// order[i] = the tile indices by descending cost: a bitonic sort in shared memory (one CTA) for up to
// kGwSortMax tiles; larger grids keep the natural order.
constexpr int kGwSortMax = 4096;
__global__ void __launch_bounds__(1024) grainwise_order_kernel(const float *__restrict__ cost, int ntiles,
                                                               int *__restrict__ order) {
    __shared__ float key[kGwSortMax];
    __shared__ int idx[kGwSortMax];
    const int tid = threadIdx.x;
    if (ntiles > kGwSortMax) {
        for (int i = tid; i < ntiles; i += blockDim.x) order[i] = i;
        return;
    }
    int n2 = 2;
    while (n2 < ntiles) n2 <<= 1;
    for (int i = tid; i < n2; i += blockDim.x) {
        key[i] = i < ntiles ? cost[i] : -1.0f;  // costs are >= 0: the padding sorts last
        idx[i] = i;
    }
    __syncthreads();
    for (int k = 2; k <= n2; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = tid; i < n2; i += blockDim.x) {
                const int ixj = i ^ j;
                if (ixj > i) {
                    const bool desc = (i & k) == 0;
                    if ((key[i] < key[ixj]) == desc) {
                        const float tk = key[i];
                        key[i] = key[ixj];
                        key[ixj] = tk;
                        const int ti = idx[i];
                        idx[i] = idx[ixj];
                        idx[ixj] = ti;
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int i = tid; i < ntiles; i += blockDim.x) order[i] = idx[i];
}

// popcount * (1/N) of the sample masks (src/grainwise.rs:114-122), fused with the colour output:
// mode 0 values only, 1 luma recombination + u8 (src/color.rs:75-96), 2 u8 pack of three planes
// whose masks are consecutive (src/color.rs:101-113).
__global__ void grainwise_epilogue_kernel(const GrainwiseEpilogueArgs a) {
    const long long n = (long long)a.out_w * a.out_h;
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float inv_samples = FG_FDIV(1.0f, (float)(a.n > 0 ? a.n : 1));
    float v[3];
    const int planes = a.mode == 2 ? 3 : 1;
    for (int c = 0; c < planes; c++) {
        const unsigned int *m = a.gmask + ((long long)c * n + i) * a.words;
        unsigned cnt = 0;
        for (int w = 0; w < a.words; w++) cnt += __popc(m[w]);
        v[c] = FG_FMUL((float)cnt, inv_samples);
        if (a.out) a.out[(long long)c * n + i] = v[c];
    }
    if (!a.out_rgb8) return;
    unsigned char *o = a.out_rgb8 + 3 * i;
    if (a.mode == 1) {
        const int ox = (int)(i % a.out_w), oy = (int)(i / a.out_w);
        float cbv, crv;
        if (a.in_w == a.out_w && a.in_h == a.out_h) {
            cbv = a.cb[i];
            crv = a.cr[i];
        } else {
            const float sxs = FG_FDIV((float)a.in_w, (float)a.out_w), sys = FG_FDIV((float)a.in_h, (float)a.out_h);
            const long long src = (long long)nearest_src(oy, sys, a.in_h) * a.in_w + nearest_src(ox, sxs, a.in_w);
            cbv = a.cb[src];
            crv = a.cr[src];
        }
        luma_rgb8(v[0], cbv, crv, o);
    } else if (a.mode == 2) {
        o[0] = to_u8(v[0]);
        o[1] = to_u8(v[1]);
        o[2] = to_u8(v[2]);
    }
}

size_t grainwise_smem_bytes(const GrainwiseArgs &a) { return grainwise_tile_smem_bytes(a); }

// The directed-rounding floor/ceil needs every bounds() argument within +-2^22.
// CTAs per tile for a stand-alone launch: enough work items to give every SM about eight, never so
// many that a part has fewer 32-pixel batches than the CTA has warps (bitmask variants only).
int grainwise_parts(const GrainwiseArgs &a, int sms) {
    if (grainwise_variant(a.n) == 0) return 1;
    const int ntiles = grainwise_tile_count(a);
    const int batches = (a.tin_w * a.tin_h + 31) / 32;
    const int want = (8 * sms + ntiles - 1) / std::max(1, ntiles);
    // each part keeps at least one 32-pixel batch per warp: fewer leave warps idle at the tile's end
    return std::max(1, std::min(std::max(1, batches / kGwWarps), want));
}

bool grainwise_small_coords(const GrainwiseArgs &a) {
    const float span = (float)max(a.out_w, a.out_h) +
                       fmaxf(fmaxf(-a.offx_min, a.offx_max), fmaxf(-a.offy_min, a.offy_max)) + a.rm * a.zoom + 4.0f;
    return span < 4194304.0f;
}

int grainwise_tile_count(const GrainwiseArgs &a) {
    return ((a.in_w + a.tin_w - 1) / a.tin_w) * ((a.in_h + a.tin_h - 1) / a.tin_h);
}

size_t grainwise_work_ints(const GrainwiseArgs &a) { return 2 + 2 * (size_t)grainwise_tile_count(a); }

cudaError_t launch_grainwise(const GrainwiseArgs &a, cudaStream_t s) {
    const size_t smem = grainwise_smem_bytes(a);
    const int ntx = (a.in_w + a.tin_w - 1) / a.tin_w, nty = (a.in_h + a.tin_h - 1) / a.tin_h;
    if (ntx <= 0 || nty <= 0) return cudaSuccess;
    const bool small = grainwise_small_coords(a);
    const int v = grainwise_variant(a.n);
    cudaError_t e;
    if (!a.work) {
        void (*k)(GrainwiseArgs);
        if (small) k = v == 4 ? grainwise_kernel<true, 4> : (v == 8 ? grainwise_kernel<true, 8> : grainwise_kernel<true, 0>);
        else k = v == 4 ? grainwise_kernel<false, 4> : (v == 8 ? grainwise_kernel<false, 8> : grainwise_kernel<false, 0>);
        e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        k<<<dim3(ntx, nty, std::max(1, a.parts)), kGwThreads, smem, s>>>(a);
        return cudaGetLastError();
    }
    // tile scheduler: costs from lambda, heaviest first, persistent CTAs
    const int ntiles = ntx * nty;
    float *cost = reinterpret_cast<float *>(a.work + 2 + ntiles);
    e = cudaMemsetAsync(a.work, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    grainwise_costs_kernel<<<(ntiles + 7) / 8, 256, 0, s>>>(a.lam, a.in_w, a.in_h, a.tin_w, a.tin_h, ntx, ntiles, cost);
    grainwise_order_kernel<<<1, 1024, 0, s>>>(cost, ntiles, a.work + 2);
    void (*k)(GrainwiseArgs, int, int);
    if (small)
        k = v == 4 ? grainwise_persistent_kernel<true, 4>
                   : (v == 8 ? grainwise_persistent_kernel<true, 8> : grainwise_persistent_kernel<true, 0>);
    else
        k = v == 4 ? grainwise_persistent_kernel<false, 4>
                   : (v == 8 ? grainwise_persistent_kernel<false, 8> : grainwise_persistent_kernel<false, 0>);
    e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0, per_sm = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kGwThreads, smem);
    if (e != cudaSuccess) return e;
    const int grid = std::max(1, std::min(ntiles * std::max(1, a.parts), sms * std::max(1, per_sm)));
    k<<<grid, kGwThreads, smem, s>>>(a, ntx, ntiles);
    return cudaGetLastError();
}

cudaError_t launch_grainwise_epilogue(const GrainwiseEpilogueArgs &a, cudaStream_t s) {
    const long long n = (long long)a.out_w * a.out_h;
    if (n <= 0) return cudaSuccess;
    grainwise_epilogue_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace fg
