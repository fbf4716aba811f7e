// fg_batch.cu -- many images, of uneven sizes and parameters, in one persistent launch behind a CUDA graph.
//
// A batch mixes pixel-wise and grain-wise images (each with its own Params/Derived, exactly as the
// per-image entry points render them).  Creating a batch plans every image (launch plans as in
// fg_capi.cu, under the batch's tuning), cuts the work into items -- pixel-wise root blocks and
// grain-wise input tiles -- and sorts them by estimated cost, largest first; it then captures one
// CUDA graph of five kernels:
//   1. a segmented kernel that zeroes the accumulators (pixel-wise output planes, grain-wise sample
//      masks, the work counter) and builds the pixel-wise images' cell tables;
//   2. the per-sample kernel over the pixel-wise images whose planes take that path per image
//      (pixelwise_prefers_regen), one thread per output pixel;
//   3. a lean persistent kernel (256 threads, 4 CTAs per SM) over the other pixel-wise images' root
//      blocks, which leaves blocks too dense for its shared-memory buffers to the next kernel (as the
//      per-image lean pass does);
//   4. the persistent kernel: 2 CTAs per SM pull the deferred pixel-wise blocks, then the grain-wise
//      tiles, from an atomic counter and run the same tile code as the per-image kernels
//      (fg_pixelwise.cuh / fg_grainwise.cuh), so results are identical;
//   5. a segmented epilogue kernel: pixel-wise count * (1/N), grain-wise popcount * (1/N).
// fg_batch_run replays the graph.  fg_batch_autotune times candidate tunings (grain-wise tile mask
// budget, pixel-wise block edge, CTAs per SM) on the batch itself and returns the fastest.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/film_grain_gb300.h"
#include "fg_grainwise.cuh"
#include "fg_host.h"
#include "fg_internal.h"
#include "fg_kernels.cuh"
#include "fg_pixelwise.cuh"

namespace fg {

struct BatchImage {
    int algo;   // FG_ALGO_PIXEL or FG_ALGO_GRAIN
    int small;  // grain-wise: coordinates within +-2^22 (directed-rounding floor/ceil)
    PixelwiseArgs pa;
    GrainwiseArgs ga;
};

struct BatchItem {
    int image, x, y;
    int pad;  // grain-wise: part | parts << 16
};

// One contiguous range of a segmented elementwise pass.
struct Segment {
    int op;             // 0 zero u32 words, 1 cell params, 2 pixel-wise scale, 3 grain-wise popcount
    int words;          // op 3: mask words per pixel
    long long n;        // elements
    void *a;            // op 0: u32 words; 1: lambda; 2: plane; 3: masks
    void *b;            // op 1: cell table; 3: output plane
    float f;            // op 1: delta; 2, 3: 1/N
};
struct Chunk {
    int seg;
    int pad;
    long long begin, end;
};

constexpr long long kChunk = 1 << 16;

__global__ void batch_segments_kernel(const Segment *__restrict__ segs, const Chunk *__restrict__ chunks) {
    const Chunk c = chunks[blockIdx.x];
    const Segment sg = segs[c.seg];
    for (long long i = c.begin + threadIdx.x; i < c.end; i += blockDim.x) {
        if (sg.op == 0) {
            static_cast<unsigned int *>(sg.a)[i] = 0u;
        } else if (sg.op == 1) {
            const float l = static_cast<const float *>(sg.a)[i];
            CellParam cp;
            cp.thresh = 0x7FFFFFFFFFFFFFFFll;
            cp.exp_lambda = 0.0;
            if (l > 0.0f) {
                const float expected = FG_FMUL(FG_FMUL(l, sg.f), sg.f);
                if (expected > 0.0f) {
                    const double e = (double)expected;
                    if (e < 12.0) {
                        const double el = exp(-e);
                        cp.exp_lambda = el;
                        cp.thresh = (long long)FG_DMUL(el, 9007199254740992.0);
                    } else {
                        cp.thresh = -1;
                        cp.exp_lambda = -e;
                    }
                }
            }
            static_cast<CellParam *>(sg.b)[i] = cp;
        } else if (sg.op == 2) {
            float *p = static_cast<float *>(sg.a);
            p[i] = FG_FMUL(p[i], sg.f);
        } else {
            const unsigned int *m = static_cast<const unsigned int *>(sg.a) + i * sg.words;
            unsigned cnt = 0;
            for (int w = 0; w < sg.words; w++) cnt += __popc(m[w]);
            static_cast<float *>(sg.b)[i] = FG_FMUL((float)cnt, sg.f);
        }
    }
}

// counters: [0] the lean kernel's next item, [1] the persistent kernel's next item, [2] deferred items.

// One image of the per-sample kernel: its CTAs are [first, first + row_ctas * out_h).
struct RegenRange {
    int image, row_ctas;
    long long first;
};

// Pixel-wise images on the per-sample path (pixelwise_prefers_regen): CTA b finds its image by a
// binary search over the ranges (ascending first) and covers 256 pixels of one of its rows.
__global__ void __launch_bounds__(kPwRegenThreads)
    batch_regen_kernel(const BatchImage *__restrict__ images, const RegenRange *__restrict__ ranges, int n_ranges) {
    __shared__ int s_r;
    __shared__ __align__(16) PixelwiseArgs s_pa;
    const long long b = blockIdx.x;
    if (threadIdx.x == 0) {
        int lo = 0, hi = n_ranges - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (ranges[mid].first <= b) lo = mid;
            else hi = mid - 1;
        }
        s_r = lo;
    }
    __syncthreads();
    const RegenRange R = ranges[s_r];
    {
        const int *src = reinterpret_cast<const int *>(&images[R.image].pa);
        int *dst = reinterpret_cast<int *>(&s_pa);
        for (int k = threadIdx.x; k < (int)(sizeof(PixelwiseArgs) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
    }
    __syncthreads();
    const long long local = b - R.first;
    pixelwise_regen_pixels(s_pa, (int)(local % R.row_ctas) * kPwRegenThreads, (int)(local / R.row_ctas));
}

// Pixel-wise items in lean CTAs (256 threads, 4 per SM); the root blocks they leave to fat CTAs are
// appended to `deferred` for the persistent kernel.
__global__ void __launch_bounds__(PwLean::kThreads, PwLean::kCtasPerSm)
    batch_lean_kernel(const BatchImage *__restrict__ images, const BatchItem *__restrict__ items, int n_items,
                      int *counters, BatchItem *__restrict__ deferred) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    __shared__ int s_image;
    __shared__ __align__(16) PixelwiseArgs s_pa;
    if (threadIdx.x == 0) s_image = -1;
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(&counters[0], 1);
        __syncthreads();
        const int it = s_item;
        if (it >= n_items) break;
        const BatchItem w = items[it];
        if (w.image != s_image) {
            const int *src = reinterpret_cast<const int *>(&images[w.image].pa);
            int *dst = reinterpret_cast<int *>(&s_pa);
            for (int k = threadIdx.x; k < (int)(sizeof(PixelwiseArgs) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) s_image = w.image;
        const bool left = pixelwise_block<PwLean>(s_pa, w.x, w.y, smem_raw, true);
        if (left && threadIdx.x == 0) deferred[atomicAdd(&counters[2], 1)] = w;
        __syncthreads();
    }
}

// The deferred pixel-wise blocks first (the densest), then the grain-wise tiles.
__global__ void __launch_bounds__(512, 2) batch_persistent_kernel(const BatchImage *__restrict__ images,
                                                                  const BatchItem *__restrict__ items, int n_items,
                                                                  int *counters, const BatchItem *__restrict__ deferred) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ int s_item;
    __shared__ int s_image;
    __shared__ __align__(16) BatchImage s_img;
    if (threadIdx.x == 0) s_image = -1;
    const int nd = counters[2];
    while (true) {
        if (threadIdx.x == 0) s_item = atomicAdd(&counters[1], 1);
        __syncthreads();
        const int it = s_item;
        if (it >= nd + n_items) break;
        const BatchItem w = it < nd ? deferred[it] : items[it - nd];
        if (w.image != s_image) {  // load the image's descriptor into shared memory
            const int *src = reinterpret_cast<const int *>(&images[w.image]);
            int *dst = reinterpret_cast<int *>(&s_img);
            for (int k = threadIdx.x; k < (int)(sizeof(BatchImage) / sizeof(int)); k += blockDim.x) dst[k] = src[k];
        }
        __syncthreads();
        if (threadIdx.x == 0) s_image = w.image;
        if (s_img.algo == FG_ALGO_PIXEL) pixelwise_block<PwFat>(s_img.pa, w.x, w.y, smem_raw);
        else if (s_img.small) grainwise_tile<true>(s_img.ga, w.x, w.y, smem_raw, w.pad & 0xFFFF, w.pad >> 16);
        else grainwise_tile<false>(s_img.ga, w.x, w.y, smem_raw, w.pad & 0xFFFF, w.pad >> 16);
        __syncthreads();
    }
}

}  // namespace fg

using namespace fg;

struct fg_batch {
    int n_images = 0;
    fg_batch_tuning tuning{};
    std::vector<void *> owned;  // device allocations (freed on destroy)
    BatchImage *d_images = nullptr;
    BatchItem *d_items = nullptr;     // grain-wise tiles, heaviest first
    int n_items = 0;
    BatchItem *d_px_items = nullptr;  // pixel-wise root blocks, heaviest first (the lean kernel's list)
    int n_px_items = 0;
    BatchItem *d_deferred = nullptr;  // pixel-wise blocks the lean kernel leaves to fat CTAs
    RegenRange *d_regen = nullptr;    // pixel-wise images on the per-sample kernel
    int n_regen = 0;
    long long regen_ctas = 0;
    int *d_counter = nullptr;         // [0] lean next, [1] persistent next, [2] deferred count
    int lean_grid = 0;
    size_t lean_smem = 0;
    Segment *d_segs = nullptr;
    Chunk *d_pre_chunks = nullptr, *d_post_chunks = nullptr;
    int n_pre_chunks = 0, n_post_chunks = 0;
    size_t smem = 0;
    int grid = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

namespace fg {

static void free_batch(fg_batch *b) {
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    for (void *p : b->owned) cudaFree(p);
    delete b;
}

template <class T>
static cudaError_t dev_copy(fg_batch *b, const std::vector<T> &v, T **out) {
    void *p = nullptr;
    cudaError_t e = cudaMalloc(&p, std::max<size_t>(sizeof(T), v.size() * sizeof(T)));
    if (e != cudaSuccess) return e;
    b->owned.push_back(p);
    if (!v.empty()) e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    *out = static_cast<T *>(p);
    return e;
}

static cudaError_t dev_alloc(fg_batch *b, size_t bytes, void **out) {
    cudaError_t e = cudaMalloc(out, std::max<size_t>(bytes, 16));
    if (e == cudaSuccess) b->owned.push_back(*out);
    return e;
}

static void add_chunks(std::vector<Chunk> &chunks, int seg, long long n) {
    for (long long s = 0; s < n; s += kChunk) chunks.push_back(Chunk{seg, 0, s, std::min(n, s + kChunk)});
}

fg_batch_tuning default_tuning() {
    fg_batch_tuning t;
    t.grain_mask_words = 8192;
    t.pixel_max_block_log2 = 4;
    t.ctas_per_sm = 2;
    return t;
}

static fg_status batch_build(const fg_batch_image *imgs, int n, const fg_batch_tuning &tun, cudaStream_t s,
                             fg_batch **out) {
    fg_batch *b = new fg_batch();
    b->n_images = n;
    b->tuning = tun;
    std::vector<BatchImage> images(n);
    struct CostItem {
        double cost;
        BatchItem it;
    };
    std::vector<CostItem> work, px_work;
    struct GrainTile {
        double cost;
        BatchItem it;
        int batches;  // the most CTAs the tile can be split over (its 32-pixel batches)
    };
    std::vector<GrainTile> grain_tiles;
    std::vector<RegenRange> regen;
    long long regen_ctas = 0;
    std::vector<Segment> segs;
    std::vector<Chunk> pre, post;
    size_t smem = pixelwise_smem_bytes();
    auto fail = [&](fg_status st) {
        free_batch(b);
        return st;
    };
#define FG_BCUDA(call, what)                                       \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return fail(cuda_error(e_, what));  \
    } while (0)
    segs.push_back(Segment{0, 0, 4, nullptr, nullptr, 0.0f});  // the work counters, filled below
    for (int i = 0; i < n; i++) {
        const fg_batch_image &im = imgs[i];
        if (!im.params || !im.derived || !im.d_lambda || !im.d_out || !im.offsets)
            return fail(set_error(FG_ERR_INVALID, "batch image " + std::to_string(i) + ": null pointer"));
        fg_status st = check_render_args(im.params, im.derived);
        if (st != FG_OK) return fail(st);
        const fg_params &p = *im.params;
        const fg_derived &d = *im.derived;
        const int algo = im.algo == FG_ALGO_PIXEL ? FG_ALGO_PIXEL : FG_ALGO_GRAIN;
        const long long n_in = d.input_width * d.input_height, n_out = d.output_width * d.output_height;
        BatchImage &B = images[i];
        std::memset(&B, 0, sizeof B);
        B.algo = algo;
        if (algo == FG_ALGO_PIXEL) {
            void *d_offs, *d_cells, *d_diag;
            FG_BCUDA(dev_alloc(b, sizeof(float) * 2 * p.n_samples, &d_offs), "batch alloc");
            FG_BCUDA(cudaMemcpy(d_offs, im.offsets, sizeof(float) * 2 * p.n_samples, cudaMemcpyHostToDevice), "H2D");
            FG_BCUDA(dev_alloc(b, sizeof(CellParam) * n_in, &d_cells), "batch alloc");
            FG_BCUDA(dev_alloc(b, sizeof(unsigned long long) * kPwDiagWords, &d_diag), "batch alloc");
            const PwPlan pl = plan_pixelwise(p, d, im.offsets, tun.pixel_max_block_log2);
            PixelwiseArgs &a = B.pa;
            a = pixelwise_args(p, d, pl, im.d_lambda, (const CellParam *)d_cells, (const float *)d_offs, im.d_out,
                               (unsigned long long *)d_diag);
            segs.push_back(Segment{0, 0, n_out, im.d_out, nullptr, 0.0f});
            add_chunks(pre, (int)segs.size() - 1, n_out);
            segs.push_back(Segment{0, 0, kPwDiagWords * 2, d_diag, nullptr, 0.0f});
            add_chunks(pre, (int)segs.size() - 1, kPwDiagWords * 2);
            segs.push_back(Segment{1, 0, n_in, (void *)im.d_lambda, d_cells, d.delta});
            add_chunks(pre, (int)segs.size() - 1, n_in);
            segs.push_back(Segment{2, 0, n_out, im.d_out, nullptr, 1.0f / (float)p.n_samples});
            add_chunks(post, (int)segs.size() - 1, n_out);
            if (pixelwise_prefers_regen(a)) {  // the per-sample kernel takes the whole image
                const int row_ctas = (int)((d.output_width + kPwRegenThreads - 1) / kPwRegenThreads);
                regen.push_back(RegenRange{i, row_ctas, regen_ctas});
                regen_ctas += (long long)row_ctas * d.output_height;
                continue;
            }
            // cost: the cells each block hashes (its window, or its samples' reach when that is smaller
            // and the block regenerates) plus its samples
            const double cell_area = (double)(pl.bsize + 2.0 * d.rm) / d.delta + 4.0;
            const double block_samples = (double)pl.bsize * pl.bsize * p.zoom * p.zoom * p.n_samples;
            const double per_block =
                std::min(cell_area * cell_area, block_samples * a.regen_cells) + 1.5 * block_samples;
            for (int by = 0; by < pl.nby; by++)
                for (int bx = 0; bx < pl.nbx; bx++)
                    px_work.push_back(CostItem{per_block, BatchItem{i, pl.bx0 + bx, pl.by0 + by, 0}});
        } else {
            const size_t tab_bytes = grain_table_bytes(p.n_samples);
            std::vector<unsigned char> tab(tab_bytes);
            grain_table(im.offsets, p.n_samples, tab.data());
            void *d_tab, *d_mask;
            FG_BCUDA(dev_alloc(b, tab_bytes, &d_tab), "batch alloc");
            FG_BCUDA(cudaMemcpy(d_tab, tab.data(), tab_bytes, cudaMemcpyHostToDevice), "H2D");
            const size_t mask_bytes = grainwise_mask_bytes(p, d);
            FG_BCUDA(dev_alloc(b, mask_bytes, &d_mask), "batch alloc");
            GrainwiseArgs &a = B.ga;
            a = grainwise_args(p, d, im.offsets, im.d_lambda, d_tab, (unsigned int *)d_mask, tun.grain_mask_words);
            B.small = grainwise_small_coords(a) ? 1 : 0;
            smem = std::max(smem, grainwise_smem_bytes(a));
            segs.push_back(Segment{0, 0, (long long)(mask_bytes / 4), d_mask, nullptr, 0.0f});
            add_chunks(pre, (int)segs.size() - 1, (long long)(mask_bytes / 4));
            segs.push_back(Segment{3, a.words, n_out, d_mask, im.d_out, 1.0f / (float)p.n_samples});
            add_chunks(post, (int)segs.size() - 1, n_out);
            const int ntx = (a.in_w + a.tin_w - 1) / a.tin_w, nty = (a.in_h + a.tin_h - 1) / a.tin_h;
            // cost: expected grains of the tile (sum of lambda, from the host copy when given)
            for (int ty = 0; ty < nty; ty++) {
                for (int tx = 0; tx < ntx; tx++) {
                    double lam_sum = 0.0;
                    const int x0 = tx * a.tin_w, y0 = ty * a.tin_h;
                    const int x1 = std::min(a.in_w, x0 + a.tin_w), y1 = std::min(a.in_h, y0 + a.tin_h);
                    if (im.h_lambda) {
                        for (int y = y0; y < y1; y++)
                            for (int x = x0; x < x1; x++) lam_sum += im.h_lambda[(long long)y * a.in_w + x];
                    } else {
                        lam_sum = 50.0 * (x1 - x0) * (y1 - y0);
                    }
                    const double cost = lam_sum * (60.0 + 0.3 * p.n_samples) + 20.0 * (x1 - x0) * (y1 - y0);
                    const int batches = grainwise_variant(a.n) == 0 ? 1 : ((x1 - x0) * (y1 - y0) + 31) / 32;
                    grain_tiles.push_back(GrainTile{cost, BatchItem{i, tx, ty, 0}, batches});
                }
            }
        }
    }
    if (smem > 200 * 1024) return fail(set_error(FG_ERR_UNSUPPORTED, "batch tile needs too much shared memory"));
    // Heavy grain-wise tiles are split over CTAs (part | parts << 16 in the item's last word) so that no
    // item is far above the average share of an SM slot: a tile of cost c gets ceil(c / target) parts,
    // at most one per kGwWarps of its 32-pixel batches.
    {
        double total_cost = 0.0;
        for (const GrainTile &g : grain_tiles) total_cost += g.cost;
        for (const CostItem &c : px_work) total_cost += c.cost;
        int dev = 0, sms = 0;
        FG_BCUDA(cudaGetDevice(&dev), "device");
        FG_BCUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
        const double target = total_cost / (8.0 * std::max(1, sms) * std::max(1, tun.ctas_per_sm)) + 1.0;
        for (const GrainTile &g : grain_tiles) {
            const int most = std::max(1, std::min(g.batches / kGwWarps, 0xFFFF));  // a batch per warp at least
            const int parts = (int)std::max(1.0, std::min((double)most, std::ceil(g.cost / target)));
            for (int q = 0; q < parts; q++) {
                BatchItem it = g.it;
                it.pad = q | (parts << 16);
                work.push_back(CostItem{g.cost / parts, it});
            }
        }
    }
    auto by_cost = [](const CostItem &x, const CostItem &y) { return x.cost > y.cost; };
    std::stable_sort(work.begin(), work.end(), by_cost);
    std::stable_sort(px_work.begin(), px_work.end(), by_cost);
    std::vector<BatchItem> items(work.size()), px_items(px_work.size());
    for (size_t k = 0; k < work.size(); k++) items[k] = work[k].it;
    for (size_t k = 0; k < px_work.size(); k++) px_items[k] = px_work[k].it;
    b->n_items = (int)items.size();
    b->n_px_items = (int)px_items.size();
    if (regen_ctas > 0x7FFFFFFFll) return fail(set_error(FG_ERR_UNSUPPORTED, "batch: too many per-sample pixels"));
    b->n_regen = (int)regen.size();
    b->regen_ctas = regen_ctas;
    FG_BCUDA(dev_copy(b, regen, &b->d_regen), "batch upload");
    FG_BCUDA(dev_copy(b, px_items, &b->d_px_items), "batch upload");
    FG_BCUDA(dev_alloc(b, sizeof(BatchItem) * std::max<size_t>(1, px_items.size()), (void **)&b->d_deferred),
             "batch alloc");
    FG_BCUDA(dev_alloc(b, sizeof(int) * 4, (void **)&b->d_counter), "batch alloc");
    segs[0].a = b->d_counter;
    add_chunks(pre, 0, 4);
    FG_BCUDA(dev_copy(b, images, &b->d_images), "batch upload");
    FG_BCUDA(dev_copy(b, items, &b->d_items), "batch upload");
    FG_BCUDA(dev_copy(b, segs, &b->d_segs), "batch upload");
    FG_BCUDA(dev_copy(b, pre, &b->d_pre_chunks), "batch upload");
    FG_BCUDA(dev_copy(b, post, &b->d_post_chunks), "batch upload");
    b->n_pre_chunks = (int)pre.size();
    b->n_post_chunks = (int)post.size();
    b->smem = smem;
    int dev = 0, sms = 0;
    FG_BCUDA(cudaGetDevice(&dev), "device");
    FG_BCUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    b->grid = std::max(1, std::min(b->n_items + b->n_px_items, sms * std::max(1, tun.ctas_per_sm)));
    b->lean_smem = sizeof(PwShared<PwLean>);
    b->lean_grid = std::max(1, std::min(b->n_px_items, sms * PwLean::kCtasPerSm));
    FG_BCUDA(cudaFuncSetAttribute(batch_persistent_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
             "smem attribute");
    FG_BCUDA(cudaFuncSetAttribute(batch_lean_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->lean_smem),
             "smem attribute");
    // capture the launches
    cudaStream_t cs;
    FG_BCUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking), "stream");
    cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        batch_segments_kernel<<<b->n_pre_chunks, 256, 0, cs>>>(b->d_segs, b->d_pre_chunks);
        if (b->n_regen > 0)
            batch_regen_kernel<<<(unsigned)b->regen_ctas, kPwRegenThreads, 0, cs>>>(b->d_images, b->d_regen,
                                                                                  b->n_regen);
        if (b->n_px_items > 0)
            batch_lean_kernel<<<b->lean_grid, PwLean::kThreads, b->lean_smem, cs>>>(b->d_images, b->d_px_items,
                                                                                 b->n_px_items, b->d_counter,
                                                                                 b->d_deferred);
        batch_persistent_kernel<<<b->grid, 512, smem, cs>>>(b->d_images, b->d_items, b->n_items, b->d_counter,
                                                            b->d_deferred);
        batch_segments_kernel<<<b->n_post_chunks, 256, 0, cs>>>(b->d_segs, b->d_post_chunks);
        e = cudaStreamEndCapture(cs, &b->graph);
    }
    cudaStreamDestroy(cs);
    if (e != cudaSuccess) return fail(cuda_error(e, "graph capture"));
    FG_BCUDA(cudaGraphInstantiate(&b->exec, b->graph, 0), "graph instantiate");
    (void)s;
#undef FG_BCUDA
    *out = b;
    return FG_OK;
}

}  // namespace fg

extern "C" {

FG_API fg_status fg_batch_create(const fg_batch_image *images, int32_t n_images, const fg_batch_tuning *tuning,
                                 fg_batch **out) {
    if (!images || n_images <= 0 || !out) return set_error(FG_ERR_INVALID, "empty batch");
    const fg_batch_tuning t = tuning ? *tuning : default_tuning();
    if (t.grain_mask_words < 1024 || t.pixel_max_block_log2 < -4 || t.pixel_max_block_log2 > 6 || t.ctas_per_sm < 1)
        return set_error(FG_ERR_INVALID, "invalid batch tuning");
    fg_status st = batch_build(images, n_images, t, nullptr, out);
    if (st == FG_OK) clear_error();
    return st;
}

FG_API fg_status fg_batch_run(fg_batch *batch, void *stream) {
    if (!batch || !batch->exec) return set_error(FG_ERR_INVALID, "null batch");
    cudaError_t e = cudaGraphLaunch(batch->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_error(e, "graph launch");
    return FG_OK;
}

FG_API fg_status fg_batch_destroy(fg_batch *batch) {
    free_batch(batch);
    return FG_OK;
}

FG_API fg_status fg_batch_get_tuning(const fg_batch *batch, fg_batch_tuning *out) {
    if (!batch || !out) return set_error(FG_ERR_INVALID, "null batch");
    *out = batch->tuning;
    return FG_OK;
}

FG_API fg_status fg_batch_kernel_count(const fg_batch *batch, int32_t *out) {
    if (!batch || !batch->graph || !out) return set_error(FG_ERR_INVALID, "null batch");
    size_t n = 0;
    cudaError_t e = cudaGraphGetNodes(batch->graph, nullptr, &n);
    if (e != cudaSuccess) return cuda_error(e, "graph nodes");
    *out = (int32_t)n;
    return FG_OK;
}

FG_API fg_status fg_batch_autotune(const fg_batch_image *images, int32_t n_images, void *stream, fg_batch_tuning *best,
                                   float *best_ms) {
    if (!images || n_images <= 0 || !best) return set_error(FG_ERR_INVALID, "empty batch");
    cudaStream_t s = (cudaStream_t)stream;
    const int masks[] = {16384, 8192};
    const int blocks[] = {4, 2};
    const int ctas[] = {2};
    float best_t = 1e30f;
    fg_batch_tuning best_cfg = default_tuning();
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int m : masks) {
        for (int bl : blocks) {
            for (int c : ctas) {
                fg_batch_tuning t;
                t.grain_mask_words = m;
                t.pixel_max_block_log2 = bl;
                t.ctas_per_sm = c;
                fg_batch *b = nullptr;
                if (batch_build(images, n_images, t, s, &b) != FG_OK) continue;
                float ms = 1e30f;
                bool ok = cudaGraphLaunch(b->exec, s) == cudaSuccess;  // warm-up
                for (int r = 0; ok && r < 2; r++) {
                    cudaEventRecord(e0, s);
                    ok = cudaGraphLaunch(b->exec, s) == cudaSuccess;
                    cudaEventRecord(e1, s);
                    ok = ok && cudaEventSynchronize(e1) == cudaSuccess;
                    float t_ms = 0.0f;
                    cudaEventElapsedTime(&t_ms, e0, e1);
                    ms = std::min(ms, t_ms);
                }
                cudaStreamSynchronize(s);
                free_batch(b);
                if (ok && ms < best_t) {
                    best_t = ms;
                    best_cfg = t;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best_t >= 1e30f) return set_error(FG_ERR_CUDA, "no tuning candidate ran");
    *best = best_cfg;
    if (best_ms) *best_ms = best_t;
    clear_error();
    return FG_OK;
}

}  // extern "C"
