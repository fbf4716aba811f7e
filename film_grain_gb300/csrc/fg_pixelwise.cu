// fg_pixelwise.cu -- the pixel-wise coverage estimator (src/pixelwise.rs:11-106) for sm_103a.
//
// The reference loops pixel -> offset sample -> cell -> grain and regenerates every cell's grains
// from its cell_rng each time a sample visits it.  A plane takes one of two kernels
// (pixelwise_prefers_regen): the per-sample kernel keeps that loop, one thread per output pixel
// (pixelwise_regen_pixels in fg_pixelwise.cuh), for planes whose samples reach fewer cells than a
// staged window would hold (small radii, few samples per pixel); the block kernels regroup the work by
// where the samples land: sample (pixel x,y; offset k) has the input-space point
//     xg = ((x + 0.5) * inv_zoom) - offsets_input[k][0]      (same f32 rounding as src/pixelwise.rs:34)
// and belongs to the block of input space [X0,X1) x [Y0,Y1) containing (xg, yg).  One CTA owns a
// block; it
//   A. hashes every cell of the block's window (the cells any owned sample can reach) once and
//      stores its grain count q (the Poisson draw of src/pixelwise.rs:77-82),
//   B. turns the counts into a row-major CSR prefix and regenerates the non-empty cells' grains
//      (centre, radius^2) into shared memory,
//   C. evaluates every owned sample: its exact cell range i0..i1 x j0..j1 (src/pixelwise.rs:55-58)
//      maps to one contiguous CSR interval per cell row; the sample is covered if any grain there
//      passes the reference's disk test dx*dx + dy*dy <= r*r (src/pixelwise.rs:96-99),
//   D. adds per-pixel hit counts (integers, exact in f32) into the output plane.
// Because a cell's grains depend only on (seed, i, j) and coverage is an OR over the grains of the
// sample's cells, the result equals the reference's early-exit loop bit for bit.  A block whose
// window holds more grains than shared memory splits into quadrants (up to kPwMaxLevel levels);
// border blocks (few owned samples), dense overflowing windows, samples whose cell range leaves the
// staged window (never expected) and leaf blocks that still overflow run the reference's per-sample
// regeneration instead, which is exact too.
#include <algorithm>
#include <cmath>

#include "fg_kernels.cuh"
#include "fg_rng.cuh"
#include "fg_color.cuh"
#include "fg_pixelwise.cuh"
#include "fg_pixelwise_sparse.cuh"

namespace fg {

// ------------------------------------------------------------------ per-pixel Poisson set-up
__global__ void cell_params_kernel(const float *__restrict__ lam, int n, float delta, CellParam *__restrict__ cells) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float l = lam[i];
    CellParam c;
    c.thresh = 0x7FFFFFFFFFFFFFFFll;
    c.exp_lambda = 0.0;
    if (l > 0.0f) {
        float expected = FG_FMUL(FG_FMUL(l, delta), delta);  // lambda_cell * delta * delta
        if (expected > 0.0f) {
            double e = (double)expected;
            if (e < 12.0) {
                double el = exp(-e);
                c.exp_lambda = el;
                c.thresh = (long long)FG_DMUL(el, 9007199254740992.0);  // floor(el * 2^53), exact scale
            } else {
                c.thresh = -1;
                c.exp_lambda = -e;
            }
        }
    }
    cells[i] = c;
}

cudaError_t launch_cell_params(const float *lam, int in_w, int in_h, float delta, CellParam *cells, cudaStream_t s) {
    int n = in_w * in_h;
    if (n <= 0) return cudaSuccess;
    cell_params_kernel<<<(n + 255) / 256, 256, 0, s>>>(lam, n, delta, cells);
    return cudaGetLastError();
}

size_t pixelwise_smem_bytes() { return sizeof(PwShared<PwFat>); }

// One CTA per root block (block-grid row-major from (bx0, by0)).  With a list (lean pass), the blocks
// left to fat CTAs are appended to it: list[0] = count, list[1..] = block indices.
template <class C>
__global__ void __launch_bounds__(C::kThreads, C::kCtasPerSm)
    pixelwise_kernel(const __grid_constant__ PixelwiseArgs a, int *__restrict__ list) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int id = (int)blockIdx.x;
    const bool deferred = pixelwise_block<C>(a, a.bx0 + (int)(blockIdx.x % (unsigned)a.nbx),
                                             a.by0 + (int)(blockIdx.x / (unsigned)a.nbx), smem_raw, list != nullptr);
    if (deferred && threadIdx.x == 0) list[1 + atomicAdd(list, 1)] = id;
}

// The sparse pass: one CTA per sparse block (grid row-major from (sbx0, sby0)); the fat-grid blocks it
// leaves are appended to the list (list[0] = count, list[1..] = fat-grid block indices).
__global__ void __launch_bounds__(PwSparse::kThreads, PwSparse::kCtasPerSm)
    pixelwise_sparse_kernel(const __grid_constant__ PixelwiseArgs a, const PwSparseGrid g, int nby,
                            int *__restrict__ list) {
    const int sbx = g.sbx0 + (int)(blockIdx.x % (unsigned)g.nsbx), sby = g.sby0 + (int)(blockIdx.x / (unsigned)g.nsbx);
    pixelwise_sparse_root(a, g, sbx, sby, nby, list);
}

// The offsets in ascending x (ties by index: a permutation even with NaNs), for the sparse pass's
// lanes (sparse_sample_pass); with gm_ent, also the grain-major form's table of the sorted offsets by
// phase bin (frac(o.x * zoom), frac(o.y * zoom)): entries bin-major (ties by sorted index), each
// entry's sorted index, and each bin's first entry (sparse_grain_pass).  One CTA of kPwKChunk threads;
// n <= kPwKChunk.
__device__ __forceinline__ unsigned offset_sort_key(float v) {
    const unsigned b = __float_as_uint(v);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);  // the float order as an unsigned order
}
__device__ __forceinline__ int offset_phase_bin(float v) {  // v = o * zoom
    constexpr int B = PwSparse::kGmBins;
    const float f = v - floorf(v);  // [0, 1]: 1 only when v is just below an integer
    return min((int)(f * (float)B), B - 1);
}
__global__ void __launch_bounds__(kPwKChunk) sort_offsets_kernel(const float2 *__restrict__ offs, int n, float zoom,
                                                                 float2 *__restrict__ sorted,
                                                                 float4 *__restrict__ gm_ent, int *__restrict__ gm_idx) {
    constexpr int B = PwSparse::kGmBins;
    __shared__ float2 s_sorted[kPwKChunk];
    __shared__ int s_bin[kPwKChunk];
    const int k = threadIdx.x;
    if (k < n) {
        const float2 o = offs[k];
        const unsigned key = offset_sort_key(o.x);
        int rank = 0;
        for (int j = 0; j < n; j++) {
            const unsigned kj = offset_sort_key(offs[j].x);
            rank += (kj < key || (kj == key && j < k)) ? 1 : 0;
        }
        sorted[rank] = o;
        s_sorted[rank] = o;
    }
    if (!gm_ent) return;  // uniform
    __syncthreads();
    float4 e = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    int bin = 0;
    if (k < n) {
        const float2 o = s_sorted[k];
        e = make_float4(o.x, o.y, o.x * zoom, o.y * zoom);
        bin = offset_phase_bin(e.w) * B + offset_phase_bin(e.z);
        s_bin[k] = bin;
    }
    __syncthreads();
    if (k < n) {
        int pos = 0;
        for (int j = 0; j < n; j++) pos += (s_bin[j] < bin || (s_bin[j] == bin && j < k)) ? 1 : 0;
        gm_ent[pos] = e;
        gm_idx[pos] = k;
    }
    for (int b = k; b <= B * B; b += blockDim.x) {
        int first = 0;
        for (int j = 0; j < n; j++) first += s_bin[j] < b ? 1 : 0;
        gm_idx[n + b] = first;
    }
}

// The plane's emptiness bitmask (pixelwise_sparse_block step 0): one thread per mask word.
__global__ void __launch_bounds__(256) cell_mask_kernel(const __grid_constant__ PixelwiseArgs a, const PwSparseGrid g,
                                                        unsigned int *__restrict__ cellmask) {
    const long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= (long long)g.gw * g.ghw) return;
    cell_mask_word(a, g, t, cellmask);
}

static int floor_div(int a, int b) { return a >= 0 ? a / b : -((-a + b - 1) / b); }

// The window bounds of pixelwise_sparse_block, by the same f32 operations.
static int window_lo(float X0, const PixelwiseArgs &a) { return (int)std::floor((X0 - a.rm) / a.delta); }
static int window_hi(float X1, const PixelwiseArgs &a) { return (int)std::floor((X1 + a.rm) / a.delta); }

// Largest plane bitmask the sparse pass allocates (larger planes take the lean pass).
constexpr double kCellMaskMaxBytes = 16.0 * (1ull << 30);

// The sparse pass's block grid: the largest edge of 4, 2 or 1 fat-grid blocks whose window fits its
// bitmask and whose grid still gives every CTA slot several blocks; false when no edge fits (or N is
// above one offset chunk), and the plane takes the lean pass instead.
static bool plan_sparse(const PixelwiseArgs &a, int nby, int sms, PwSparseGrid *g) {
    if (a.n > kPwKChunk || !(a.rm >= 0.0f)) return false;
    for (int R = 4; R >= 1; R >>= 1) {
        const float bs = a.bsize * (float)R;
        const double edge = std::floor(((double)bs + 2.0 * a.rm) / a.delta) + 3.0;
        const double wpr = (double)sparse_col_stride((int)std::ceil(edge / 32.0));
        if (edge > PwSparse::kRowsMax || wpr * edge > PwSparse::kMaskWords) continue;
        const int sbx0 = floor_div(a.bx0, R), sbx1 = floor_div(a.bx0 + a.nbx - 1, R);
        const int sby0 = floor_div(a.by0, R), sby1 = floor_div(a.by0 + nby - 1, R);
        const long long blocks = (long long)(sbx1 - sbx0 + 1) * (sby1 - sby0 + 1);
        if (R > 1 && blocks < 4LL * sms * PwSparse::kCtasPerSm) continue;
        g->bs = bs;
        g->ratio = R;
        g->sbx0 = sbx0; g->sby0 = sby0;
        g->nsbx = sbx1 - sbx0 + 1; g->nsby = sby1 - sby0 + 1;
        // the bitmask covers every block's window with a two-cell margin
        const int gi0 = window_lo((float)sbx0 * bs, a) - 2, gi1 = window_hi((float)(sbx1 + 1) * bs, a) + 2;
        const int gj0 = window_lo((float)sby0 * bs, a) - 2, gj1 = window_hi((float)(sby1 + 1) * bs, a) + 2;
        g->cellmask = nullptr;
        g->gm_ent = nullptr;
        g->gm_idx = nullptr;
        g->gm_eps = g->gm_grain_cost = g->gm_sample_cost = 0.0f;
        g->gm_noslow = 0;
        g->gi0 = gi0;
        g->gj0 = gj0;
        g->gw = gi1 - gi0 + 1;
        g->ghw = (gj1 - gj0 + 1 + 31) / 32 + 1;  // one more word row for the windows' shifted reads
        return (double)g->gw * g->ghw * 4.0 <= kCellMaskMaxBytes;
    }
    return false;
}

static int sm_count() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
                                                    cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return sms;
}

// The sparse pass's scratch, each part 16-byte aligned: the bitmask, the offsets sorted by x, the
// grain-major form's entries (float4) and its index (entry offsets, then bin starts).
static size_t align16(size_t b) { return (b + 15) & ~(size_t)15; }
static size_t sparse_mask_bytes(const PwSparseGrid &g) { return align16((size_t)g.gw * g.ghw * sizeof(unsigned int)); }
static size_t sparse_gm_ent_at(const PwSparseGrid &g, int n) {
    return sparse_mask_bytes(g) + align16((size_t)n * sizeof(float2));
}
static size_t sparse_gm_idx_at(const PwSparseGrid &g, int n) {
    return sparse_gm_ent_at(g, n) + (size_t)n * sizeof(float4);
}

size_t pixelwise_cellmask_bytes(const PixelwiseArgs &a, int nby) {
    if (pixelwise_prefers_regen(a)) return 0;
    PwSparseGrid g;
    const int sms = sm_count();  // without a device (planning only): the GB300's 152
    if (!plan_sparse(a, nby, sms > 0 ? sms : 152, &g)) return 0;
    const int bins = PwSparse::kGmBins * PwSparse::kGmBins;
    return sparse_gm_idx_at(g, a.n) + (size_t)(a.n + bins + 1) * sizeof(int);
}

// The grain-major form's plane conditions and cost model (sparse_grain_pass).  A grain reaches at most
// rm * zoom output pixels; the candidate pixel of an offset is exact while that reach plus the f32
// rounding of the pixel coordinates (eps: a few ulps of the largest coordinate) stays below half a
// pixel, and the rounding to an integer by adding 1.5 * 2^23 needs coordinates below 2^22.  Costs, in
// units fitted to timings of both forms (on the 4096^2 planes at r 0.025 log-normal N 256 grain-major
// is faster for every block; on the 256^2 ramp at r 0.12 N 64 it is slower for the dense blocks): a
// grain pays its set-up and, per candidate, a disk test and its share of the listed hits, for
// n (2 (r_mean zoom + eps) + 1/bins)^2 candidates on average; a sample pays the scan of its cell
// range's columns.
static bool plan_grain_major(const PixelwiseArgs &a, PwSparseGrid *g) {
    const double ext = std::max({std::fabs(a.offx_min), std::fabs(a.offx_max), std::fabs(a.offy_min),
                                 std::fabs(a.offy_max)});
    const double coord = (double)std::max(a.out_w, a.out_h) + ext * a.zoom + 2.0;
    const double eps = coord * 0x1p-21 + 0x1p-20;
    g->gm_eps = (float)eps;
    const double reach = (double)a.rm * a.zoom;
    if (!(coord < 0x1p21) || !(reach + eps <= 0.4)) return false;
    // a sample's range spans floor((xg + rm) / delta) - floor((xg - rm) / delta) cells: 2 rm / delta + 1
    // and the rounding of xg +- rm and of the divisions (a few ulps of the largest grid coordinate)
    const double grid = (double)std::max(a.out_w, a.out_h) * a.inv_zoom + ext + a.rm + 2.0;
    const double span = 2.0 * a.rm / a.delta + 1.0 + 8.0 * grid * 0x1p-23 / a.delta;
    g->gm_noslow = span <= 30.0 ? 1 : 0;
    const double band = 2.0 * ((double)a.radius_mean * a.zoom + eps) + 1.0 / PwSparse::kGmBins;
    g->gm_grain_cost = (float)(60.0 + 40.0 * a.n * band * band);
    g->gm_sample_cost = (float)(40.0 + 9.0 * (2.0 * a.rm / a.delta + 1.0));
    return true;
}

// The root blocks the lean pass deferred, in fat CTAs: persistent, each CTA taking the next listed
// block from the counter defer[-1] (the word before the list's count).
__global__ void __launch_bounds__(PwFat::kThreads, PwFat::kCtasPerSm)
    pixelwise_deferred_kernel(const __grid_constant__ PixelwiseArgs a, int *__restrict__ defer) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_id;
    const int n = defer[0];
    for (;;) {
        if (threadIdx.x == 0) {
            const int i = atomicAdd(defer - 1, 1);
            s_id = (i < n && !cancel_requested(a.cancel)) ? defer[1 + i] : -1;
        }
        __syncthreads();
        const int id = s_id;
        if (id < 0) break;
        pixelwise_block<PwFat>(a, a.bx0 + id % a.nbx, a.by0 + id / a.nbx, smem_raw);
        __syncthreads();
    }
}

// Per-sample kernel: one thread per output pixel (pixelwise_regen_pixels); no shared memory, no
// barriers.  CTA b covers pixels [256 (b % row_ctas), +256) of row b / row_ctas.
__global__ void __launch_bounds__(kPwRegenThreads) pixelwise_regen_kernel(const __grid_constant__ PixelwiseArgs a,
                                                                          int row_ctas) {
    if (a.cancel) {  // once per warp: the warp's lanes work in step, so the whole warp stops
        int stop = 0;
        if ((threadIdx.x & 31) == 0) stop = cancel_requested(a.cancel) ? 1 : 0;
        if (__shfl_sync(0xffffffffu, stop, 0)) return;
    }
    pixelwise_regen_pixels(a, (int)(blockIdx.x % (unsigned)row_ctas) * kPwRegenThreads,
                           (int)(blockIdx.x / (unsigned)row_ctas));
}

bool pixelwise_prefers_regen(const PixelwiseArgs &a) {
    if (!(a.rm > 0.0f)) return true;  // nothing can cover a sample: the per-sample loop exits at once
    // a sample's range must fit the 64-bit cell mask of pixelwise_pixel
    const double axis = std::floor(2.0 * (double)a.rm / (double)a.delta) + 2.0;
    if (!(axis * axis <= 64.0)) return false;
    // cell indices of every sample must stay far inside int (the flattened loop's range arithmetic)
    const double reach = (double)std::max(a.out_w, a.out_h) / a.zoom +
                         std::max({std::fabs(a.offx_min), std::fabs(a.offx_max), std::fabs(a.offy_min),
                                   std::fabs(a.offy_max)}) + a.rm + 2.0;
    if (reach / a.delta > 1.0e9) return false;
    // an interior root block: its samples' reach in cells against its staged window
    const double samples = (double)a.bsize * a.bsize * a.zoom * a.zoom * a.n;
    const double edge = std::floor((a.bsize + 2.0 * a.rm) / a.delta) + 1.0;
    return samples * a.regen_cells < kPwRegenKernel * edge * edge;
}

cudaError_t launch_pixelwise_regen(const PixelwiseArgs &a, cudaStream_t s) {
    const long long row_ctas = (a.out_w + kPwRegenThreads - 1) / kPwRegenThreads;
    const long long grid = row_ctas * a.out_h;
    if (grid <= 0) return cudaSuccess;
    pixelwise_regen_kernel<<<(unsigned)grid, kPwRegenThreads, 0, s>>>(a, (int)row_ctas);
    return cudaGetLastError();
}

template <class K>
static cudaError_t set_smem(K k, size_t smem) {
    return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
}

cudaError_t launch_pixelwise(const PixelwiseArgs &a, int nby, int *defer, unsigned int *cellmask, cudaStream_t s) {
    if (pixelwise_prefers_regen(a)) return launch_pixelwise_regen(a, s);
    const size_t lean_smem = sizeof(PwShared<PwLean>), fat_smem = sizeof(PwShared<PwFat>);
    cudaError_t e = set_smem(pixelwise_kernel<PwLean>, lean_smem);
    if (e == cudaSuccess) e = set_smem(pixelwise_kernel<PwFat>, fat_smem);
    if (e == cudaSuccess) e = set_smem(pixelwise_deferred_kernel, fat_smem);
    if (e != cudaSuccess) return e;
    const long long nblocks = (long long)a.nbx * nby;
    if (nblocks <= 0) return cudaSuccess;
    if (!defer) {
        pixelwise_kernel<PwFat><<<(unsigned)nblocks, PwFat::kThreads, fat_smem, s>>>(a, nullptr);
        return cudaGetLastError();
    }
    e = cudaMemsetAsync(defer, 0, 2 * sizeof(int), s);  // [0] the fat pass's counter, [1] the list's count
    if (e != cudaSuccess) return e;
    int dev = 0, sms = 0;
    e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    PwSparseGrid g;
    const bool sparse = cellmask && plan_sparse(a, nby, sms, &g);
    if (sparse) {
        g.cellmask = cellmask;
        const long long words = (long long)g.gw * g.ghw;
        cell_mask_kernel<<<(unsigned)((words + 255) / 256), 256, 0, s>>>(a, g, cellmask);
        PixelwiseArgs as = a;  // the sparse pass reads the offsets sorted by x
        char *scratch = reinterpret_cast<char *>(cellmask);
        as.offs = reinterpret_cast<const float2 *>(scratch + sparse_mask_bytes(g));
        float4 *gm_ent = nullptr;
        int *gm_idx = nullptr;
        if (plan_grain_major(a, &g)) {
            gm_ent = reinterpret_cast<float4 *>(scratch + sparse_gm_ent_at(g, a.n));
            gm_idx = reinterpret_cast<int *>(scratch + sparse_gm_idx_at(g, a.n));
            g.gm_ent = gm_ent;
            g.gm_idx = gm_idx;
        }
        sort_offsets_kernel<<<1, kPwKChunk, 0, s>>>(a.offs, a.n, a.zoom, const_cast<float2 *>(as.offs), gm_ent, gm_idx);
        const size_t sparse_smem = sizeof(PwSparseShared);
        e = set_smem(pixelwise_sparse_kernel, sparse_smem);
        if (e != cudaSuccess) return e;
        pixelwise_sparse_kernel<<<(unsigned)((long long)g.nsbx * g.nsby), PwSparse::kThreads, sparse_smem, s>>>(
            as, g, nby, defer + 1);
    } else {
        pixelwise_kernel<PwLean><<<(unsigned)nblocks, PwLean::kThreads, lean_smem, s>>>(a, defer + 1);
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const long long grid = std::min<long long>(nblocks, (long long)std::max(1, sms) * PwFat::kCtasPerSm);
    PixelwiseArgs ad = a;  // after the sparse pass, the fat pass reads cell emptiness from its bitmask
    if (sparse) {
        ad.cellmask = cellmask;
        ad.cm_gi0 = g.gi0;
        ad.cm_gj0 = g.gj0;
        ad.cm_gw = g.gw;
        ad.cm_ghw = g.ghw;
    }
    pixelwise_deferred_kernel<<<(unsigned)grid, PwFat::kThreads, fat_smem, s>>>(ad, defer + 1);
    return cudaGetLastError();
}

// ------------------------------------------------------------------ epilogue: counts -> values (+ colour)
__global__ void epilogue_kernel(const EpilogueArgs a) {
    long long n = (long long)a.out_w * a.out_h;
    long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float v = FG_FMUL(a.plane[i], a.inv_samples);  // sum * inv_samples (src/pixelwise.rs:38)
    a.plane[i] = v;
    if (!a.out_rgb8) return;
    unsigned char *o = a.out_rgb8 + 3 * i;
    if (a.mode == 1) {
        int x = (int)(i % a.out_w), y = (int)(i / a.out_w);
        float cbv, crv;
        if (a.in_w == a.out_w && a.in_h == a.out_h) {
            cbv = a.cb[i]; crv = a.cr[i];
        } else {
            float sxs = FG_FDIV((float)a.in_w, (float)a.out_w), sys = FG_FDIV((float)a.in_h, (float)a.out_h);
            long long src = (long long)nearest_src(y, sys, a.in_h) * a.in_w + nearest_src(x, sxs, a.in_w);
            cbv = a.cb[src]; crv = a.cr[src];
        }
        luma_rgb8(v, cbv, crv, o);
    } else if (a.mode == 2) {
        o[0] = to_u8(a.p0[i]); o[1] = to_u8(a.p1[i]); o[2] = to_u8(v);
    }
}

cudaError_t launch_epilogue(const EpilogueArgs &a, cudaStream_t s) {
    long long n = (long long)a.out_w * a.out_h;
    if (n <= 0) return cudaSuccess;
    epilogue_kernel<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(a);
    return cudaGetLastError();
}

__global__ void rgb_pack_kernel(const float *p0, const float *p1, const float *p2, int n, unsigned char *out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[3 * i] = to_u8(p0[i]); out[3 * i + 1] = to_u8(p1[i]); out[3 * i + 2] = to_u8(p2[i]);
}
cudaError_t launch_rgb_pack(const float *p0, const float *p1, const float *p2, int n, unsigned char *out,
                            cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    rgb_pack_kernel<<<(n + 255) / 256, 256, 0, s>>>(p0, p1, p2, n, out);
    return cudaGetLastError();
}

}  // namespace fg
