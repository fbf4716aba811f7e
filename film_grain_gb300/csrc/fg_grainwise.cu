// fg_grainwise.cu -- the grain-wise integrator (src/grainwise.rs:12-142) for sm_103a.
//
// The reference walks input pixels, draws Poisson(lambda) grains from each pixel's stream, and for
// every grain and offset k ORs bit k into the 64-bit sample masks of the output pixels whose centres
// fall in the offset disk (AtomicU64::fetch_or), then popcounts the masks.  Here one CTA owns an
// output tile: its N-bit masks live in shared memory as ceil(N/32) 32-bit words per pixel; the CTA
// regenerates the grains of every input pixel whose offset disks can reach the tile (the pixel
// streams are deterministic, so tiles never need each other's grains), rasterises them with the
// reference's exact bounds() and centre test, and finishes with the popcount * (1/N) epilogue --
// optionally fused with the luma colour recombination and u8 packing.  Bits are set with
// shared-memory atomicOr; OR is idempotent and commutative, so the result is independent of order.
#include "fg_kernels.cuh"
#include "fg_rng.cuh"
#include "fg_color.cuh"

namespace fg {

constexpr int kGwThreads = 256;

__device__ __forceinline__ int gw_f2i(float v) { return __float2int_rz(v); }

__global__ void __launch_bounds__(kGwThreads) grainwise_kernel(const GrainwiseArgs a) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    float2 *offs = reinterpret_cast<float2 *>(smem_raw);
    unsigned int *mask = reinterpret_cast<unsigned int *>(offs + a.n);
    const int tid = threadIdx.x;
    const int tx0 = blockIdx.x * a.tile_w, ty0 = blockIdx.y * a.tile_h;
    const int tx1 = min(tx0 + a.tile_w, a.out_w), ty1 = min(ty0 + a.tile_h, a.out_h);
    const int words = a.words;
    const int tile_words = a.tile_w * a.tile_h * words;

    for (int k = tid; k < a.n; k += kGwThreads) offs[k] = a.offs[k];
    for (int t = tid; t < tile_words; t += kGwThreads) mask[t] = 0u;
    __syncthreads();

    // Input pixels whose grains can reach the tile (conservative: one extra pixel of margin).
    const float reach = FG_FMUL(a.rm, a.zoom) + 2.0f;
    const int ix0 = max(0, (int)floorf(((float)tx0 - reach - a.offx_max) / a.zoom) - 1);
    const int ix1 = min(a.in_w, (int)ceilf(((float)tx1 + reach - a.offx_min) / a.zoom) + 1);
    const int iy0 = max(0, (int)floorf(((float)ty0 - reach - a.offy_max) / a.zoom) - 1);
    const int iy1 = min(a.in_h, (int)ceilf(((float)ty1 + reach - a.offy_min) / a.zoom) + 1);
    const int fw = ix1 - ix0, fh = iy1 - iy0;
    const UniformF32 U = uniform_f32_new(0.0f, 1.0f);
    const float zoom = a.zoom;
    const int last_x = a.out_w - 1, last_y = a.out_h - 1;

    if (fw > 0 && fh > 0) {
        for (int p = tid; p < fw * fh; p += kGwThreads) {
            const int x = ix0 + p % fw, y = iy0 + p / fw;
            const float lv = a.lam[(long long)y * a.in_w + x];
            if (!(lv > 0.0f)) continue;
            Xoshiro rng = pixel_rng(a.seed, x, y);
            const PoissonParams P = poisson_new((double)lv);
            const uint32_t q = poisson_sample(P, rng);
            for (uint32_t g = 0; g < q; g++) {
                const float cx = FG_FADD((float)x, uniform_f32_from(U, rng.next()));
                const float cy = FG_FADD((float)y, uniform_f32_from(U, rng.next()));
                float r = a.lognorm ? (float)exp(normal_sample(a.log_mu, a.log_sigma, rng)) : a.radius_mean;
                if (r > a.rm) r = a.rm;
                if (r <= 0.0f) continue;
                const float ro = FG_FMUL(r, zoom);
                if (ro <= 0.0f) continue;
                const float rsq = FG_FMUL(ro, ro);
                const float czx = FG_FMUL(cx, zoom), czy = FG_FMUL(cy, zoom);
                for (int k = 0; k < a.n; k++) {
                    const float2 o = offs[k];
                    const float tx = FG_FADD(czx, o.x);
                    const float ty = FG_FADD(czy, o.y);
                    // bounds(tx, radius_out, output_width) (src/grainwise.rs:126-142)
                    int xlo = gw_f2i(ceilf(FG_FSUB(FG_FSUB(tx, ro), 0.5f)));
                    int xhi = gw_f2i(floorf(FG_FSUB(FG_FADD(tx, ro), 0.5f)));
                    if (xhi < xlo || xlo > last_x || xhi < 0) continue;
                    int ylo = gw_f2i(ceilf(FG_FSUB(FG_FSUB(ty, ro), 0.5f)));
                    int yhi = gw_f2i(floorf(FG_FSUB(FG_FADD(ty, ro), 0.5f)));
                    if (yhi < ylo || ylo > last_y || yhi < 0) continue;
                    // clamp to the image, then keep the tile's part
                    xlo = max(max(xlo, 0), tx0); xhi = min(min(xhi, last_x), tx1 - 1);
                    ylo = max(max(ylo, 0), ty0); yhi = min(min(yhi, last_y), ty1 - 1);
                    if (xlo > xhi || ylo > yhi) continue;
                    const unsigned bit = 1u << (k & 31);
                    const int word = k >> 5;
                    for (int oy = ylo; oy <= yhi; oy++) {
                        const float dy = FG_FSUB(FG_FADD((float)oy, 0.5f), ty);
                        const float dysq = FG_FMUL(dy, dy);
                        if (dysq > rsq) continue;
                        for (int ox = xlo; ox <= xhi; ox++) {
                            const float dx = FG_FSUB(FG_FADD((float)ox, 0.5f), tx);
                            if (FG_FADD(FG_FMUL(dx, dx), dysq) <= rsq)
                                atomicOr(&mask[((oy - ty0) * a.tile_w + (ox - tx0)) * words + word], bit);
                        }
                    }
                }
            }
        }
    }
    __syncthreads();

    // popcount * (1/N) (src/grainwise.rs:114-122), optionally fused with the luma recombination.
    const float inv_samples = FG_FDIV(1.0f, (float)(a.n > 0 ? a.n : 1));
    const int tw = tx1 - tx0, th = ty1 - ty0;
    for (int t = tid; t < tw * th; t += kGwThreads) {
        const int lx = t % tw, ly = t / tw;
        const unsigned int *m = mask + (ly * a.tile_w + lx) * words;
        unsigned c = 0;
        for (int w = 0; w < words; w++) c += __popc(m[w]);
        const float v = FG_FMUL((float)c, inv_samples);
        const int ox = tx0 + lx, oy = ty0 + ly;
        const long long idx = (long long)oy * a.out_w + ox;
        if (a.out) a.out[idx] = v;
        if (a.out_rgb8) {
            float cbv, crv;
            if (a.in_w == a.out_w && a.in_h == a.out_h) {
                cbv = a.cb[idx]; crv = a.cr[idx];
            } else {
                const float sxs = FG_FDIV((float)a.in_w, (float)a.out_w), sys = FG_FDIV((float)a.in_h, (float)a.out_h);
                const long long src = (long long)nearest_src(oy, sys, a.in_h) * a.in_w + nearest_src(ox, sxs, a.in_w);
                cbv = a.cb[src]; crv = a.cr[src];
            }
            luma_rgb8(v, cbv, crv, a.out_rgb8 + 3 * idx);
        }
    }
}

size_t grainwise_smem_bytes(const GrainwiseArgs &a) {
    return (size_t)a.n * sizeof(float2) + (size_t)a.tile_w * a.tile_h * a.words * sizeof(unsigned int);
}

cudaError_t launch_grainwise(const GrainwiseArgs &a, cudaStream_t s) {
    size_t smem = grainwise_smem_bytes(a);
    cudaError_t e = cudaFuncSetAttribute(grainwise_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    dim3 grid((a.out_w + a.tile_w - 1) / a.tile_w, (a.out_h + a.tile_h - 1) / a.tile_h);
    if (grid.x == 0 || grid.y == 0) return cudaSuccess;
    grainwise_kernel<<<grid, kGwThreads, smem, s>>>(a);
    return cudaGetLastError();
}

}  // namespace fg
