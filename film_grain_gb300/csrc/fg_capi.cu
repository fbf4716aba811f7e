// fg_capi.cu -- the render entry points of the C-ABI: buffer staging, launch planning and the
// whole-image orchestration of render_from_workspace_impl (src/lib.rs:134-173).
#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/film_grain_gb300.h"
#include "fg_host.h"
#include "fg_kernels.cuh"
#include "fg_internal.h"

namespace fg {

static thread_local unsigned long long g_pw_diag[kPwDiagWords] = {0, 0, 0, 0, 0, 0};

fg_status cuda_error(cudaError_t e, const char *what) {
    return set_error(e == cudaErrorMemoryAllocation ? FG_ERR_NOMEM : FG_ERR_CUDA,
                     std::string("gpu error: ") + what + ": " + cudaGetErrorString(e));
}

#define FG_CUDA(call, what)                                  \
    do {                                                     \
        cudaError_t e_ = (call);                             \
        if (e_ != cudaSuccess) return cuda_error(e_, what);  \
    } while (0)

bool is_device_ptr(const void *p) {
    if (!p) return false;
    cudaPointerAttributes attr;
    cudaError_t e = cudaPointerGetAttributes(&attr, p);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

static bool cancelled(const volatile int32_t *cancel) { return cancel && *cancel != 0; }

// ------------------------------------------------------------------ in-launch cancellation
// The caller's cancel flag is ordinary host memory that the GPU cannot be assumed to reach, so while a
// synchronous render runs a watcher thread polls it (every 200 us) and mirrors a non-zero value into
// a word of mapped pinned memory that the kernels read (cancel_requested).  The words come from one
// pinned block kept for the life of the process, one 64-byte line per render in flight.
class CancelSlots {
  public:
    static CancelSlots &get() {
        static CancelSlots s;
        return s;
    }
    int *acquire() {
        std::lock_guard<std::mutex> lock(mu_);
        if (!base_) {
            void *p = nullptr;
            if (cudaHostAlloc(&p, kSlots * kLine, cudaHostAllocMapped | cudaHostAllocPortable) != cudaSuccess) {
                cudaGetLastError();
                return nullptr;  // no in-launch polling; the flag is still read between launches
            }
            base_ = static_cast<int *>(p);
            for (int i = kSlots - 1; i >= 0; i--) free_.push_back(i);
        }
        if (free_.empty()) return nullptr;
        int *w = base_ + free_.back() * (kLine / sizeof(int));
        free_.pop_back();
        ((volatile int *)w)[0] = 0;
        ((volatile int *)w)[1] = 0;
        return w;
    }
    void release(int *w) {
        std::lock_guard<std::mutex> lock(mu_);
        free_.push_back((int)((w - base_) / (kLine / sizeof(int))));
    }

  private:
    static constexpr int kSlots = 256;
    static constexpr size_t kLine = 64;
    std::mutex mu_;
    int *base_ = nullptr;
    std::vector<int> free_;
};

class CancelWatch {
  public:
    explicit CancelWatch(const volatile int32_t *cancel) : cancel_(cancel) {
        if (!cancel) return;
        host_ = CancelSlots::get().acquire();
        if (!host_) return;
        void *d = nullptr;
        if (cudaHostGetDevicePointer(&d, host_, 0) != cudaSuccess) {
            cudaGetLastError();
            CancelSlots::get().release(host_);
            host_ = nullptr;
            return;
        }
        dev_ = static_cast<int *>(d);
        thread_ = std::thread([this] {
            while (!done_.load(std::memory_order_acquire)) {
                if (*cancel_ != 0) {
                    ((volatile int *)host_)[0] = 1;
                    return;
                }
                std::this_thread::sleep_for(std::chrono::microseconds(200));
            }
        });
    }
    // Called once the render's work on the GPU has finished (or failed).
    ~CancelWatch() {
        if (thread_.joinable()) {
            done_.store(true, std::memory_order_release);
            thread_.join();
        }
        if (host_) CancelSlots::get().release(host_);
    }
    CancelWatch(const CancelWatch &) = delete;
    CancelWatch &operator=(const CancelWatch &) = delete;
    int *dev() const { return dev_; }
    // whether a CTA stopped on the flag
    bool stopped() const { return host_ && ((volatile int *)host_)[1] != 0; }

  private:
    const volatile int32_t *cancel_;
    int *host_ = nullptr;
    int *dev_ = nullptr;
    std::atomic<bool> done_{false};
    std::thread thread_;
};

static fg_status cancelled_error(const CancelWatch &w) {
    return set_error(FG_ERR_CANCELLED, w.stopped() ? "cancelled (stopped inside a kernel)" : "cancelled");
}

void offset_extents(const float *offs, uint32_t n, float ext[4]) {
    ext[0] = ext[1] = ext[2] = ext[3] = 0.0f;
    for (uint32_t k = 0; k < n; k++) {
        ext[0] = std::fmin(ext[0], offs[2 * k]);
        ext[1] = std::fmax(ext[1], offs[2 * k]);
        ext[2] = std::fmin(ext[2], offs[2 * k + 1]);
        ext[3] = std::fmax(ext[3], offs[2 * k + 1]);
    }
}

fg_status check_render_args(const fg_params *p, const fg_derived *d) {
    if (!p || !d) return set_error(FG_ERR_INVALID, "null params or derived");
    if (d->input_width <= 0 || d->input_height <= 0 || d->output_width <= 0 || d->output_height <= 0)
        return set_error(FG_ERR_INVALID, "plane dimensions must be positive");
    if (d->input_width > (1 << 24) || d->input_height > (1 << 24) || d->output_width > (1 << 24) ||
        d->output_height > (1 << 24) || d->input_width * d->input_height >= (1ll << 31) ||
        d->output_width * d->output_height >= (1ll << 31))
        return set_error(FG_ERR_UNSUPPORTED, "plane larger than 2^31 pixels or 2^24 per side");
    if (p->n_samples == 0 || p->n_samples > 65536) return set_error(FG_ERR_UNSUPPORTED, "n_samples must be in 1..65536");
    if (!(p->zoom > 0.0f) || !(d->delta > 0.0f)) return set_error(FG_ERR_INVALID, "zoom and delta must be positive");
    if (p->radius_dist == FG_RADIUS_LOGNORM && !p->has_log_params)
        return set_error(FG_ERR_INVALID, "missing log-normal parameters");
    return FG_OK;
}

// Pixel-wise launch plan: the largest power-of-two block edge whose staged window fits.
PwPlan plan_pixelwise(const fg_params &p, const fg_derived &d, const float *h_offs_in, int max_block_log2) {
    PwPlan pl;
    offset_extents(h_offs_in, p.n_samples, pl.ext);
    const float rm = d.rm, delta = d.delta;
    int b;
    for (b = max_block_log2; b > -8; b--) {
        float B = std::ldexp(1.0f, b);
        double wc = std::floor((B + 2.0 * rm) / delta) + 4.0;
        if (wc <= kPwEdgeMax && wc * wc <= kPwCellMax) break;
    }
    pl.bsize = std::ldexp(1.0f, b);
    const float inv_zoom = 1.0f / p.zoom;
    float xmin = 0.5f * inv_zoom - pl.ext[1], ymin = 0.5f * inv_zoom - pl.ext[3];
    float xmax = ((float)(d.output_width - 1) + 0.5f) * inv_zoom - pl.ext[0];
    float ymax = ((float)(d.output_height - 1) + 0.5f) * inv_zoom - pl.ext[2];
    pl.bx0 = (int)std::floor(xmin / pl.bsize) - 1;
    pl.by0 = (int)std::floor(ymin / pl.bsize) - 1;
    pl.nbx = (int)std::floor(xmax / pl.bsize) + 1 - pl.bx0 + 1;
    pl.nby = (int)std::floor(ymax / pl.bsize) + 1 - pl.by0 + 1;
    return pl;
}

PixelwiseArgs pixelwise_args(const fg_params &p, const fg_derived &d, const PwPlan &pl, const float *d_lam,
                             const CellParam *d_cells, const float *d_offs_in, float *d_out, unsigned long long *d_diag) {
    PixelwiseArgs a;
    std::memset(&a, 0, sizeof a);
    a.lam = d_lam;
    a.cells = d_cells;
    a.offs = reinterpret_cast<const float2 *>(d_offs_in);
    a.out = d_out;
    a.diag = d_diag;
    a.in_w = (int)d.input_width; a.in_h = (int)d.input_height;
    a.out_w = (int)d.output_width; a.out_h = (int)d.output_height;
    a.n = (int)p.n_samples;
    a.rm = d.rm;
    a.delta = d.delta;
    {
        const double t = d.rm > 0.0f ? 2.0 * (double)d.rm / (double)d.delta + 1.0 : 0.0;
        a.regen_cells = (float)(t * t);
    }
    a.inv_zoom = 1.0f / p.zoom;
    a.zoom = p.zoom;
    a.bsize = pl.bsize;
    a.inv_bsize = 1.0f / pl.bsize;
    a.bx0 = pl.bx0; a.by0 = pl.by0; a.nbx = pl.nbx;
    a.offx_min = pl.ext[0]; a.offx_max = pl.ext[1]; a.offy_min = pl.ext[2]; a.offy_max = pl.ext[3];
    a.seed = p.seed;
    a.lognorm = p.radius_dist == FG_RADIUS_LOGNORM;
    a.radius_mean = p.radius_mean;
    a.log_mu = (double)p.radius_log_mu;
    a.log_sigma = (double)p.radius_log_sigma;
    return a;
}

// Stream-ordered device buffer that frees itself.
struct DevBuf {
    void *p = nullptr;
    cudaStream_t s = nullptr;
    cudaError_t alloc(size_t bytes, cudaStream_t st) {
        s = st;
        return cudaMallocAsync(&p, bytes ? bytes : 16, st);
    }
    ~DevBuf() {
        if (p) cudaFreeAsync(p, s);
    }
};

fg_status enqueue_pixelwise(const float *d_lam, const fg_params &p, const fg_derived &d, const float *h_offs_in,
                            const float *d_offs_in, float *d_out, CellParam *d_cells, unsigned long long *d_diag,
                            const EpilogueArgs *colour, cudaStream_t s, bool may_allocate, int *d_cancel) {
    const int in_w = (int)d.input_width, in_h = (int)d.input_height;
    const int out_w = (int)d.output_width, out_h = (int)d.output_height;
    const PwPlan pl = plan_pixelwise(p, d, h_offs_in, 4);
    FG_CUDA(launch_cell_params(d_lam, in_w, in_h, d.delta, d_cells, s), "cell params");
    FG_CUDA(cudaMemsetAsync(d_out, 0, sizeof(float) * (size_t)out_w * out_h, s), "memset");
    PixelwiseArgs a = pixelwise_args(p, d, pl, d_lam, d_cells, d_offs_in, d_out, d_diag);
    a.cancel = d_cancel;
    DevBuf defer;  // the first pass's list of deferred root blocks (none without allocation: fat CTAs only)
    DevBuf cellmask;  // the sparse pass's emptiness bitmask of the plane's cells
    if (may_allocate) {
        FG_CUDA(defer.alloc((2 + (size_t)pl.nbx * pl.nby) * sizeof(int), s), "alloc defer list");
        const size_t mask_bytes = pixelwise_cellmask_bytes(a, pl.nby);
        if (mask_bytes && cellmask.alloc(mask_bytes, s) != cudaSuccess) {
            cudaGetLastError();  // no room for the bitmask: the plane takes the lean pass
            cellmask.p = nullptr;
        }
    }
    FG_CUDA(launch_pixelwise(a, pl.nby, static_cast<int *>(defer.p), static_cast<unsigned int *>(cellmask.p), s),
            "pixelwise kernel");
    EpilogueArgs e;
    if (colour) e = *colour;
    else std::memset(&e, 0, sizeof e);
    e.plane = d_out;
    e.out_w = out_w; e.out_h = out_h; e.in_w = in_w; e.in_h = in_h;
    e.inv_samples = 1.0f / (float)p.n_samples;
    FG_CUDA(launch_epilogue(e, s), "pixelwise epilogue");
    return FG_OK;
}

size_t grain_table_bytes(uint32_t n) { return (size_t)n * sizeof(float4) + (kGwBucketCount + 1) * sizeof(int); }

void grain_table(const float *h_offs, uint32_t n, void *blob) {
    struct Entry {
        float fx;
        float4 e;
    };
    std::vector<Entry> t(n);
    for (uint32_t k = 0; k < n; k++) {
        const float ox = h_offs[2 * k], oy = h_offs[2 * k + 1];
        float fx = ox - std::floor(ox), fy = oy - std::floor(oy);
        if (!(fx < 1.0f)) fx = 0.0f;  // a tiny negative offset can round up to 1; cyclically that is 0
        if (!(fy < 1.0f)) fy = 0.0f;
        int kb = (int)k;
        float kf;
        std::memcpy(&kf, &kb, 4);
        t[k] = Entry{fx, make_float4(fy, ox, oy, kf)};
    }
    std::stable_sort(t.begin(), t.end(), [](const Entry &a, const Entry &b) { return a.fx < b.fx; });
    float4 *entries = reinterpret_cast<float4 *>(blob);
    int *bstart = reinterpret_cast<int *>(entries + n);
    for (uint32_t k = 0; k < n; k++) entries[k] = t[k].e;
    uint32_t j = 0;
    for (int b = 0; b <= kGwBucketCount; b++) {
        const float v = (float)b / (float)kGwBucketCount;
        while (j < n && t[j].fx < v) j++;
        bstart[b] = b == kGwBucketCount ? (int)n : (int)j;
    }
}

// Shared-memory sample-mask words per grain-wise tile (sets the tile edge).  Measured on GB300 with
// N = 128 at zoom 2 (1024^2 plane): 6144 words 29.6 ms, 8192 26.3 ms, 12288 28.7 ms, 16384 31.7 ms.
constexpr int kGrainMaskWords = 8192;

GrainwiseArgs grainwise_args(const fg_params &p, const fg_derived &d, const float *h_offs, const float *d_lam,
                             const void *d_table, unsigned int *d_gmask, int mask_words) {
    GrainwiseArgs a;
    std::memset(&a, 0, sizeof a);
    float ext[4];
    offset_extents(h_offs, p.n_samples, ext);
    a.lam = d_lam;
    a.sorted_offs = reinterpret_cast<const float4 *>(d_table);
    a.bucket_start = reinterpret_cast<const int *>(reinterpret_cast<const float4 *>(d_table) + p.n_samples);
    a.gmask = d_gmask;
    a.in_w = (int)d.input_width; a.in_h = (int)d.input_height;
    a.out_w = (int)d.output_width; a.out_h = (int)d.output_height;
    a.n = (int)p.n_samples;
    a.words = (a.n + 31) / 32;
    // Input tile: its zoomed rectangle should fill about `mask_words` words of shared memory.
    // floor(x0*zoom + tin*zoom) - floor(x0*zoom) <= ceil(tin*zoom), so that bounds the rectangle.
    const int side = std::max(1, (int)std::floor(std::sqrt((double)mask_words / a.words)));
    const int tin = std::max(1, (int)std::floor(side / p.zoom));
    a.tin_w = std::min(tin, a.in_w);
    a.tin_h = std::min(tin, a.in_h);
    a.rmax_w = std::max(1, std::min(a.out_w, (int)std::ceil(a.tin_w * (double)p.zoom)));
    a.rmax_h = std::max(1, std::min(a.out_h, (int)std::ceil(a.tin_h * (double)p.zoom)));
    a.rm = d.rm;
    a.zoom = p.zoom;
    a.parts = 1;
    a.offx_min = ext[0]; a.offx_max = ext[1]; a.offy_min = ext[2]; a.offy_max = ext[3];
    // Rounding margin of the candidate intervals: each of the three f32 roundings between
    // czx + offx and the bounds() comparison moves a value by at most half an ulp of the largest
    // coordinate M; the fraction arithmetic adds a few 2^-24.
    const double M = (double)std::max(d.output_width, d.output_height) + 8.0 +
                     std::max(std::max(-ext[0], ext[1]), std::max(-ext[2], ext[3])) + d.rm * p.zoom;
    const double U = std::ldexp(1.0, (int)std::floor(std::log2(M)) - 23);
    a.frac_eps = (float)(4.0 * U + std::ldexp(1.0, -20));
    a.seed = p.seed;
    a.lognorm = p.radius_dist == FG_RADIUS_LOGNORM;
    a.radius_mean = p.radius_mean;
    a.log_mu = (double)p.radius_log_mu;
    a.log_sigma = (double)p.radius_log_sigma;
    return a;
}

size_t grainwise_mask_bytes(const fg_params &p, const fg_derived &d) {
    return (size_t)d.output_width * d.output_height * ((p.n_samples + 31) / 32) * sizeof(unsigned int);
}

fg_status enqueue_grainwise(const GrainwiseArgs &a, cudaStream_t s) {
    if (grainwise_smem_bytes(a) > 200 * 1024)
        return set_error(FG_ERR_UNSUPPORTED, "n_samples too large for the grain-wise tile");
    FG_CUDA(cudaMemsetAsync(a.gmask, 0, (size_t)a.out_w * a.out_h * a.words * sizeof(unsigned int), s), "memset mask");
    GrainwiseArgs b = a;
    DevBuf work;  // the tile scheduler's area, freed in stream order after the launch
    FG_CUDA(work.alloc(grainwise_work_ints(a) * sizeof(int), s), "alloc tile scheduler");
    b.work = static_cast<int *>(work.p);
    int dev = 0, sms = 0;
    FG_CUDA(cudaGetDevice(&dev), "device");
    FG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev), "device attribute");
    b.parts = grainwise_parts(a, sms);
    FG_CUDA(launch_grainwise(b, s), "grainwise kernel");
    return FG_OK;
}

fg_status enqueue_grainwise_epilogue(const GrainwiseArgs &a, float *d_out, int mode, unsigned char *d_rgb8,
                                     const float *d_cb, const float *d_cr, cudaStream_t s) {
    GrainwiseEpilogueArgs e;
    std::memset(&e, 0, sizeof e);
    e.gmask = a.gmask;
    e.out = d_out;
    e.out_rgb8 = d_rgb8;
    e.cb = d_cb;
    e.cr = d_cr;
    e.out_w = a.out_w; e.out_h = a.out_h; e.in_w = a.in_w; e.in_h = a.in_h;
    e.n = a.n;
    e.words = a.words;
    e.mode = mode;
    FG_CUDA(launch_grainwise_epilogue(e, s), "grainwise epilogue");
    return FG_OK;
}

// The stream-ordered pool of the current device keeps its memory between renders (raised release
// threshold), set once per device; safe to call from several threads.
static void keep_pool_memory() {
    static std::atomic<bool> done[128];
    static std::mutex mu;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) {
        cudaGetLastError();
        return;
    }
    if (done[dev].load(std::memory_order_acquire)) return;
    std::lock_guard<std::mutex> lock(mu);
    if (done[dev].load(std::memory_order_relaxed)) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        uint64_t thr = UINT64_MAX;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    cudaGetLastError();
    done[dev].store(true, std::memory_order_release);
}

// Shared body of the synchronous integrator entry points.
static fg_status render_plane_sync(int algo, const float *lambda, const fg_params *params, const fg_derived *derived,
                                   const float *offsets, float *out, const volatile int32_t *cancel, void *stream) {
    fg_status st = check_render_args(params, derived);
    if (st != FG_OK) return st;
    if (!lambda || !offsets || !out) return set_error(FG_ERR_INVALID, "null buffer");
    if (cancelled(cancel)) return set_error(FG_ERR_CANCELLED, "cancelled");
    keep_pool_memory();
    cudaStream_t s = (cudaStream_t)stream;
    const fg_params &p = *params;
    const fg_derived &d = *derived;
    CancelWatch watch(cancel);
    const size_t n_in = (size_t)d.input_width * d.input_height, n_out = (size_t)d.output_width * d.output_height;
    const size_t off_bytes = sizeof(float) * 2 * p.n_samples;

    std::vector<float> h_offs(2 * (size_t)p.n_samples);
    const bool offs_dev = is_device_ptr(offsets);
    if (offs_dev) FG_CUDA(cudaMemcpy(h_offs.data(), offsets, off_bytes, cudaMemcpyDeviceToHost), "offsets D2H");
    else std::memcpy(h_offs.data(), offsets, off_bytes);

    DevBuf b_lam, b_out, b_offs, b_cells, b_diag;
    const float *d_lam = lambda;
    float *d_out = out;
    const float *d_offs = offsets;
    if (!is_device_ptr(lambda)) {
        FG_CUDA(b_lam.alloc(sizeof(float) * n_in, s), "alloc lambda");
        FG_CUDA(cudaMemcpyAsync(b_lam.p, lambda, sizeof(float) * n_in, cudaMemcpyHostToDevice, s), "lambda H2D");
        d_lam = (const float *)b_lam.p;
    }
    const bool out_dev = is_device_ptr(out);
    if (!out_dev) {
        FG_CUDA(b_out.alloc(sizeof(float) * n_out, s), "alloc out");
        d_out = (float *)b_out.p;
    }
    if (algo == FG_ALGO_GRAIN) {
        std::vector<unsigned char> tab(grain_table_bytes(p.n_samples));
        grain_table(h_offs.data(), p.n_samples, tab.data());
        FG_CUDA(b_offs.alloc(tab.size(), s), "alloc offsets");
        FG_CUDA(cudaMemcpyAsync(b_offs.p, tab.data(), tab.size(), cudaMemcpyHostToDevice, s), "offsets H2D");
        d_offs = (const float *)b_offs.p;
    } else if (!offs_dev) {
        FG_CUDA(b_offs.alloc(off_bytes, s), "alloc offsets");
        FG_CUDA(cudaMemcpyAsync(b_offs.p, h_offs.data(), off_bytes, cudaMemcpyHostToDevice, s), "offsets H2D");
        d_offs = (const float *)b_offs.p;
    }
    if (algo == FG_ALGO_PIXEL) {
        FG_CUDA(b_cells.alloc(sizeof(CellParam) * n_in, s), "alloc cell table");
        FG_CUDA(b_diag.alloc(sizeof(unsigned long long) * kPwDiagWords, s), "alloc diag");
        FG_CUDA(cudaMemsetAsync(b_diag.p, 0, sizeof(unsigned long long) * kPwDiagWords, s), "memset diag");
        st = enqueue_pixelwise(d_lam, p, d, h_offs.data(), d_offs, d_out, (CellParam *)b_cells.p,
                               (unsigned long long *)b_diag.p, nullptr, s, true, watch.dev());
    } else {
        FG_CUDA(b_cells.alloc(grainwise_mask_bytes(p, d), s), "alloc sample masks");
        GrainwiseArgs a = grainwise_args(p, d, h_offs.data(), d_lam, d_offs, (unsigned int *)b_cells.p, kGrainMaskWords);
        a.cancel = watch.dev();
        st = enqueue_grainwise(a, s);
        if (st == FG_OK) st = enqueue_grainwise_epilogue(a, d_out, 0, nullptr, nullptr, nullptr, s);
    }
    if (st != FG_OK) {
        cudaStreamSynchronize(s);
        return st;
    }
    if (!out_dev) FG_CUDA(cudaMemcpyAsync(out, d_out, sizeof(float) * n_out, cudaMemcpyDeviceToHost, s), "out D2H");
    if (algo == FG_ALGO_PIXEL)
        FG_CUDA(cudaMemcpyAsync(g_pw_diag, b_diag.p, sizeof g_pw_diag, cudaMemcpyDeviceToHost, s), "diag D2H");
    FG_CUDA(cudaStreamSynchronize(s), "render");
    if (cancelled(cancel)) return cancelled_error(watch);
    clear_error();
    return FG_OK;
}

}  // namespace fg

using namespace fg;

extern "C" {

FG_API fg_status fg_render_pixelwise(const float *lambda, const fg_params *params, const fg_derived *derived,
                                     const float *offsets_input, float *out, const volatile int32_t *cancel,
                                     void *stream) {
    return render_plane_sync(FG_ALGO_PIXEL, lambda, params, derived, offsets_input, out, cancel, stream);
}

FG_API fg_status fg_render_grainwise(const float *lambda, const fg_params *params, const fg_derived *derived,
                                     const float *offsets, float *out, const volatile int32_t *cancel, void *stream) {
    return render_plane_sync(FG_ALGO_GRAIN, lambda, params, derived, offsets, out, cancel, stream);
}

FG_API fg_status fg_render_pixelwise_async(const float *d_lambda, const fg_params *params, const fg_derived *derived,
                                           const float *offsets_input, float *d_out, void *stream) {
    fg_status st = check_render_args(params, derived);
    if (st != FG_OK) return st;
    if (!d_lambda || !offsets_input || !d_out) return set_error(FG_ERR_INVALID, "null buffer");
    if (is_device_ptr(offsets_input)) return set_error(FG_ERR_INVALID, "offsets_input must be host memory");
    keep_pool_memory();
    cudaStream_t s = (cudaStream_t)stream;
    const size_t n_in = (size_t)derived->input_width * derived->input_height;
    const size_t off_bytes = sizeof(float) * 2 * params->n_samples;
    DevBuf b_offs, b_cells, b_diag;
    FG_CUDA(b_offs.alloc(off_bytes, s), "alloc offsets");
    FG_CUDA(cudaMemcpyAsync(b_offs.p, offsets_input, off_bytes, cudaMemcpyHostToDevice, s), "offsets H2D");
    FG_CUDA(b_cells.alloc(sizeof(CellParam) * n_in, s), "alloc cell table");
    FG_CUDA(b_diag.alloc(sizeof(unsigned long long) * kPwDiagWords, s), "alloc diag");
    FG_CUDA(cudaMemsetAsync(b_diag.p, 0, sizeof(unsigned long long) * kPwDiagWords, s), "memset diag");
    return enqueue_pixelwise(d_lambda, *params, *derived, offsets_input, (const float *)b_offs.p, d_out,
                             (CellParam *)b_cells.p, (unsigned long long *)b_diag.p, nullptr, s);
}

FG_API fg_status fg_render_grainwise_async(const float *d_lambda, const fg_params *params, const fg_derived *derived,
                                           const float *offsets, float *d_out, void *stream) {
    fg_status st = check_render_args(params, derived);
    if (st != FG_OK) return st;
    if (!d_lambda || !offsets || !d_out) return set_error(FG_ERR_INVALID, "null buffer");
    if (is_device_ptr(offsets)) return set_error(FG_ERR_INVALID, "offsets must be host memory");
    keep_pool_memory();
    cudaStream_t s = (cudaStream_t)stream;
    std::vector<unsigned char> tab(grain_table_bytes(params->n_samples));
    grain_table(offsets, params->n_samples, tab.data());
    DevBuf b_offs, b_mask;
    FG_CUDA(b_offs.alloc(tab.size(), s), "alloc offsets");
    FG_CUDA(cudaMemcpyAsync(b_offs.p, tab.data(), tab.size(), cudaMemcpyHostToDevice, s), "offsets H2D");
    FG_CUDA(b_mask.alloc(grainwise_mask_bytes(*params, *derived), s), "alloc sample masks");
    GrainwiseArgs a = grainwise_args(*params, *derived, offsets, d_lambda, b_offs.p, (unsigned int *)b_mask.p, kGrainMaskWords);
    st = enqueue_grainwise(a, s);
    if (st == FG_OK) st = enqueue_grainwise_epilogue(a, d_out, 0, nullptr, nullptr, nullptr, s);
    return st;
}

FG_API fg_status fg_render_image(const float *rgb, int64_t width, int64_t height, const fg_params *params,
                                 uint8_t *out_rgb8, fg_render_stats *stats, const volatile int32_t *cancel,
                                 void *stream) {
    if (!rgb || !params || !out_rgb8) return set_error(FG_ERR_INVALID, "null pointer");
    if (width <= 0 || height <= 0) return set_error(FG_ERR_INVALID, "input image is empty");
    if (cancelled(cancel)) return set_error(FG_ERR_CANCELLED, "cancelled");
    const fg_params &p = *params;
    int64_t x0 = 0, y0 = 0, cw = width, ch = height;
    if (p.has_roi) {
        if ((int64_t)p.roi_x1 > width || (int64_t)p.roi_y1 > height)
            return set_error(FG_ERR_INVALID, "ROI exceeds image bounds");
        x0 = p.roi_x0; y0 = p.roi_y0;
        cw = (int64_t)p.roi_x1 - p.roi_x0; ch = (int64_t)p.roi_y1 - p.roi_y0;
        if (cw <= 0 || ch <= 0) return set_error(FG_ERR_INVALID, "ROI width and height must be positive");
    }
    fg_derived d;
    std::vector<float> offs(2 * (size_t)p.n_samples), offs_in(2 * (size_t)p.n_samples);
    fg_status st = derive(p, cw, ch, &d, offs.data(), offs_in.data());
    if (st != FG_OK) return st;
    st = check_render_args(params, &d);
    if (st != FG_OK) return st;
    const int32_t algo = choose_algorithm(p, d);
    const bool luma = p.color_mode == FG_COLOR_LUMA;
    const int nplanes = luma ? 1 : 3;
    const size_t n_in = (size_t)cw * ch, n_out = (size_t)d.output_width * d.output_height;

    keep_pool_memory();
    cudaStream_t s = (cudaStream_t)stream;
    CancelWatch watch(cancel);
    DevBuf b_lam, b_out, b_rgb8, b_rgb, b_planes, b_max, b_offs, b_cells, b_diag;
    // the cropped interleaved RGB to the device, then the colour split, the plane maxima and lambda
    // there (fg_lambda.cu): no host pass over the image
    FG_CUDA(b_rgb.alloc(sizeof(float) * 3 * n_in, s), "alloc rgb");
    FG_CUDA(cudaMemcpy2DAsync(b_rgb.p, sizeof(float) * 3 * (size_t)cw, rgb + 3 * ((size_t)y0 * width + x0),
                              sizeof(float) * 3 * (size_t)width, sizeof(float) * 3 * (size_t)cw, (size_t)ch,
                              cudaMemcpyHostToDevice, s),
            "rgb H2D");
    FG_CUDA(b_planes.alloc(sizeof(float) * 3 * n_in, s), "alloc planes");
    FG_CUDA(b_max.alloc(sizeof(unsigned int) * 3, s), "alloc plane maxima");
    FG_CUDA(b_lam.alloc(sizeof(float) * n_in * nplanes, s), "alloc lambda");
    FG_CUDA(b_out.alloc(sizeof(float) * n_out * nplanes, s), "alloc planes");
    FG_CUDA(b_rgb8.alloc(3 * n_out, s), "alloc rgb8");
    std::vector<unsigned char> tab;
    if (algo == FG_ALGO_PIXEL) {
        FG_CUDA(b_offs.alloc(sizeof(float) * 2 * p.n_samples, s), "alloc offsets");
        FG_CUDA(cudaMemcpyAsync(b_offs.p, offs_in.data(), sizeof(float) * 2 * p.n_samples, cudaMemcpyHostToDevice, s),
                "offsets H2D");
    } else {
        tab.resize(grain_table_bytes(p.n_samples));
        grain_table(offs.data(), p.n_samples, tab.data());
        FG_CUDA(b_offs.alloc(tab.size(), s), "alloc offsets");
        FG_CUDA(cudaMemcpyAsync(b_offs.p, tab.data(), tab.size(), cudaMemcpyHostToDevice, s), "offsets H2D");
    }
    float *d_lam = (float *)b_lam.p, *d_out = (float *)b_out.p;
    st = enqueue_split_lambda((const float *)b_rgb.p, (long long)n_in, luma ? 1 : 0, (float *)b_planes.p,
                              (unsigned int *)b_max.p, d.inv_e_pi_r2, d_lam, s);
    if (st != FG_OK) {
        cudaStreamSynchronize(s);
        return st;
    }
    float *d_cb = nullptr, *d_cr = nullptr;
    if (luma) {
        d_cb = (float *)b_planes.p + n_in;
        d_cr = d_cb + n_in;
    }
    const size_t mask_bytes = algo == FG_ALGO_GRAIN ? grainwise_mask_bytes(p, d) : 0;
    if (algo == FG_ALGO_PIXEL) {
        FG_CUDA(b_cells.alloc(sizeof(CellParam) * n_in, s), "alloc cell table");
        FG_CUDA(b_diag.alloc(sizeof(unsigned long long) * kPwDiagWords, s), "alloc diag");
        FG_CUDA(cudaMemsetAsync(b_diag.p, 0, sizeof(unsigned long long) * kPwDiagWords, s), "memset diag");
    } else {
        FG_CUDA(b_cells.alloc(mask_bytes * nplanes, s), "alloc sample masks");
    }
    for (int c = 0; c < nplanes; c++) {
        if (cancelled(cancel)) {
            cudaStreamSynchronize(s);
            return cancelled_error(watch);
        }
        float *d_plane = d_out + (size_t)c * n_out;
        if (algo == FG_ALGO_PIXEL) {
            EpilogueArgs e;
            std::memset(&e, 0, sizeof e);
            if (luma) {
                e.mode = 1; e.out_rgb8 = (unsigned char *)b_rgb8.p; e.cb = d_cb; e.cr = d_cr;
            } else if (c == 2) {
                e.mode = 2; e.out_rgb8 = (unsigned char *)b_rgb8.p; e.p0 = d_out; e.p1 = d_out + n_out;
            }
            st = enqueue_pixelwise(d_lam + (size_t)c * n_in, p, d, offs_in.data(), (const float *)b_offs.p, d_plane,
                                   (CellParam *)b_cells.p, (unsigned long long *)b_diag.p, &e, s, true, watch.dev());
        } else {
            unsigned int *plane_mask = (unsigned int *)((unsigned char *)b_cells.p + mask_bytes * c);
            GrainwiseArgs a = grainwise_args(p, d, offs.data(), d_lam + (size_t)c * n_in, b_offs.p, plane_mask, kGrainMaskWords);
            a.cancel = watch.dev();
            st = enqueue_grainwise(a, s);
            if (st == FG_OK && c == nplanes - 1) {
                a.gmask = (unsigned int *)b_cells.p;  // all planes' masks, consecutive
                st = enqueue_grainwise_epilogue(a, nullptr, luma ? 1 : 2, (unsigned char *)b_rgb8.p, d_cb, d_cr, s);
            }
        }
        if (st != FG_OK) {
            cudaStreamSynchronize(s);
            return st;
        }
    }
    FG_CUDA(cudaMemcpyAsync(out_rgb8, b_rgb8.p, 3 * n_out, cudaMemcpyDeviceToHost, s), "rgb8 D2H");
    FG_CUDA(cudaStreamSynchronize(s), "render");
    if (cancelled(cancel)) return cancelled_error(watch);
    if (stats) fill_stats(p, d, algo, stats);
    clear_error();
    return FG_OK;
}

// Counters of the calling thread's last synchronous pixel-wise render: samples evaluated on the
// per-sample regeneration path, blocks without a staged window, block subdivisions, blocks run.
FG_API void fg_pixelwise_diagnostics(unsigned long long out[4]) {
    for (int i = 0; i < 4; i++) out[i] = g_pw_diag[i];
}

// The sparse pass's blocks of that render by the form of their sample step: sample-major, grain-major.
FG_API void fg_pixelwise_sparse_forms(unsigned long long out[2]) {
    out[0] = g_pw_diag[4];
    out[1] = g_pw_diag[5];
}

FG_API fg_status fg_pixelwise_kernel_count(const fg_params *params, const fg_derived *derived,
                                           const float *offsets_input, int32_t *out) {
    if (!params || !derived || !offsets_input || !out) return set_error(FG_ERR_INVALID, "null argument");
    fg_status st = check_render_args(params, derived);
    if (st != FG_OK) return st;
    const PwPlan pl = plan_pixelwise(*params, *derived, offsets_input, 4);
    const PixelwiseArgs a = pixelwise_args(*params, *derived, pl, nullptr, nullptr, nullptr, nullptr, nullptr);
    *out = pixelwise_prefers_regen(a) ? 3 : (pixelwise_cellmask_bytes(a, pl.nby) ? 6 : 4);
    clear_error();
    return FG_OK;
}

}  // extern "C"
