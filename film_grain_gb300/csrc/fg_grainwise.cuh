// fg_grainwise.cuh -- device code of the grain-wise integrator (src/grainwise.rs:12-142), shared by
// the standalone kernel (fg_grainwise.cu) and the batched persistent kernel (fg_batch.cu).
#pragma once
#include "fg_kernels.cuh"
#include "fg_rng.cuh"
#include "fg_color.cuh"

namespace fg {

constexpr int kGwThreads = 512;
constexpr int kGwWarps = kGwThreads / 32;
constexpr int kGwQueue = 64;     // grains per warp queue (a full batch of 32 plus a partial step)
constexpr int kGwList = 256;     // surviving (grain, offset) pairs per warp list
constexpr int kGwBuckets = kGwBucketCount;

// The CTA's shared-memory mask covers the output rectangle [rx0, rx0 + rw) x [ry0, ry0 + rh); bits of
// other output pixels go straight to the global mask.
struct GwTile {
    int rx0, ry0, rw, rh, words, out_w;
    float flast_x, flast_y;          // last output column / row as floats
    unsigned int *gmask;             // out_w x out_h x words
};

// floor / ceil of an f32.  With kSmall (every coordinate within +-2^22) they are one directed-rounding
// add and one exact subtract of 1.5 * 2^23, which stay on the FP32 pipes.
template <bool kSmall>
__device__ __forceinline__ float gw_floor(float v) {
    if (kSmall) return __fsub_rn(__fadd_rd(v, 12582912.0f), 12582912.0f);
    return floorf(v);
}
template <bool kSmall>
__device__ __forceinline__ float gw_ceil(float v) {
    if (kSmall) return __fsub_rn(__fadd_ru(v, 12582912.0f), 12582912.0f);
    return ceilf(v);
}

// bounds(center, radius, limit) (src/grainwise.rs:126-142) as [max(lo, lo_t), min(hi, hi_t)] with
// lo = ceil((c - r) - 0.5), hi = floor((c + r) - 0.5) and [lo_t, hi_t] = [0, limit-1]: the reference
// yields Some iff lo <= hi, lo <= limit-1 and hi >= 0, and then clamps to [0, limit-1], which is
// exactly this interval when it is non-empty.  Coordinates stay below 2^24, so comparing integral
// floats is the reference's i32 comparison.
template <bool kSmall>
__device__ __forceinline__ bool gw_range(float c, float r, float lo_t, float hi_t, float &a, float &b) {
    a = fmaxf(gw_ceil<kSmall>(FG_FSUB(FG_FSUB(c, r), 0.5f)), lo_t);
    b = fminf(gw_floor<kSmall>(FG_FSUB(FG_FADD(c, r), 0.5f)), hi_t);
    return a <= b;
}

// Stage B: the reference's exact bounds() on both axes, then its centre tests and bit sets
// (src/grainwise.rs:69-101) for one (grain, offset) pair.  G = (czx, czy, radius_out, -),
// e = (frac(offy), offx, offy, k).
template <bool kSmall>
__device__ __forceinline__ void gw_splat(const GwTile &T, unsigned int *mask, const float4 G, const float4 e) {
    const float ro = G.z;
    const float ty = FG_FADD(G.y, e.z);
    float y0, y1, x0, x1;
    if (!gw_range<kSmall>(ty, ro, 0.0f, T.flast_y, y0, y1)) return;
    const float tx = FG_FADD(G.x, e.y);
    if (!gw_range<kSmall>(tx, ro, 0.0f, T.flast_x, x0, x1)) return;
    const float rsq = FG_FMUL(ro, ro);
    const int k = __float_as_int(e.w);
    const unsigned bit = 1u << (k & 31);
    const int word = k >> 5;
    int oy = (int)y0;
    for (float fyv = y0; fyv <= y1; fyv = FG_FADD(fyv, 1.0f), oy++) {
        const float dy = FG_FSUB(FG_FADD(fyv, 0.5f), ty);
        const float dysq = FG_FMUL(dy, dy);
        if (dysq > rsq) continue;
        int ox = (int)x0;
        for (float fxv = x0; fxv <= x1; fxv = FG_FADD(fxv, 1.0f), ox++) {
            const float dx = FG_FSUB(FG_FADD(fxv, 0.5f), tx);
            if (FG_FADD(FG_FMUL(dx, dx), dysq) <= rsq) {
                const int lx = ox - T.rx0, ly = oy - T.ry0;
                if ((unsigned)lx < (unsigned)T.rw && (unsigned)ly < (unsigned)T.rh)
                    atomicOr(mask + (ly * T.rw + lx) * T.words + word, bit);
                else
                    atomicOr(T.gmask + ((long long)oy * T.out_w + ox) * T.words + word, bit);
            }
        }
    }
}

// Candidate ranges of one grain in the sorted offset table: the entries whose frac(offx) lies in the
// cyclic interval [c - h, c + h], c = frac(1/2 - czx), h = radius_out + margin, rounded out to whole
// buckets of the index `bstart` (bstart[b] = first entry with frac >= b / kGwBuckets).  Entries the
// rounding adds are harmless: every entry still goes through the exact reference test.  Packed as
// (first | end << 16) for the two pieces of the cyclic interval.
__device__ __forceinline__ uint2 gw_candidates(const int *bstart, int n, float czx, float ro, float eps) {
    const float h = FG_FADD(ro, eps);
    if (h >= 0.5f) return make_uint2((unsigned)n << 16, 0u);
    const float fz = FG_FSUB(czx, floorf(czx));     // exact
    float c = FG_FSUB(0.5f, fz);
    if (c < 0.0f) c = FG_FADD(c, 1.0f);
    const float lo = FG_FSUB(c, h), hi = FG_FADD(c, h);
    const float nb = (float)kGwBuckets;
    int s0, e0, s1 = 0, e1 = 0;
    if (lo < 0.0f) {  // [0, hi] and [lo + 1, 1)
        s0 = 0;
        e0 = bstart[min(kGwBuckets - 1, (int)(hi * nb)) + 1];
        s1 = bstart[min(kGwBuckets - 1, max(0, (int)(FG_FADD(lo, 1.0f) * nb)))];
        e1 = n;
    } else if (hi >= 1.0f) {  // [lo, 1) and [0, hi - 1]
        s0 = bstart[min(kGwBuckets - 1, (int)(lo * nb))];
        e0 = n;
        e1 = bstart[min(kGwBuckets - 1, max(0, (int)(FG_FSUB(hi, 1.0f) * nb))) + 1];
    } else {
        s0 = bstart[min(kGwBuckets - 1, (int)(lo * nb))];
        e0 = bstart[min(kGwBuckets - 1, (int)(hi * nb)) + 1];
    }
    return make_uint2((unsigned)s0 | ((unsigned)e0 << 16), (unsigned)s1 | ((unsigned)e1 << 16));
}

// Stage B over the warp's survivor list: one (grain, offset) pair per lane.
template <bool kSmall>
__device__ __forceinline__ void gw_drain(const GwTile &T, unsigned int *mask, const float4 *tab, const float4 *q,
                                         const unsigned *list, int &ln, int lane) {
    for (int b = 0; b < ln; b += 32) {
        if (b + lane < ln) {
            const unsigned v = list[b + lane];
            gw_splat<kSmall>(T, mask, q[v >> 16], tab[v & 0xFFFFu]);
        }
    }
    ln = 0;
    __syncwarp();
}

// Stage A over one batch of `count` queued grains: the (grain, candidate offset) pairs are flattened
// across the lanes (every lane busy).  A pair can set a bit only if some pixel row lies within
// radius_out of ty = czy + offy, i.e. only if frac(offy) lies within h = radius_out + margin of
// cy = frac(1/2 - czy) on the unit circle; that test filters the pairs, and the survivors -- (grain,
// table index) -- are compacted into the warp's list for the exact stage B.
template <bool kSmall>
__device__ __forceinline__ void gw_raster_batch(const GwTile &T, unsigned int *mask, const float4 *tab,
                                                const float *fy, const float4 *q, const uint2 *qr, int count,
                                                int *cpre, unsigned *list, int &ln, float eps, int lane) {
    int c = 0;
    if (lane < count) {
        const uint2 r = qr[lane];
        c = (int)(r.x >> 16) - (int)(r.x & 0xFFFFu) + (int)(r.y >> 16) - (int)(r.y & 0xFFFFu);
    }
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, c, o);
        if (lane >= o) c += y;
    }
    const int total = __shfl_sync(0xffffffffu, c, 31);
    cpre[lane + 1] = c;
    if (lane == 0) cpre[0] = 0;
    __syncwarp();
    int g = 0;
    for (int base = 0; base < total; base += 32) {
        const int t = base + lane;
        bool surv = false;
        unsigned item = 0;
        if (t < total) {
            while (cpre[g + 1] <= t) g++;
            const uint2 r = qr[g];
            const int o = t - cpre[g];
            const int n0 = (int)(r.x >> 16) - (int)(r.x & 0xFFFFu);
            const int i = o < n0 ? (int)(r.x & 0xFFFFu) + o : (int)(r.y & 0xFFFFu) + (o - n0);
            const float2 gy = *reinterpret_cast<const float2 *>(&q[g].z);  // (radius_out, cy)
            const float h = FG_FADD(gy.x, eps);
            const float d = fabsf(FG_FSUB(fy[i], gy.y));
            surv = d <= h || d >= FG_FSUB(1.0f, h);
            item = ((unsigned)g << 16) | (unsigned)i;
        }
        const unsigned sb = __ballot_sync(0xffffffffu, surv);
        if (surv) list[ln + __popc(sb & ((1u << lane) - 1u))] = item;
        ln += __popc(sb);
        __syncwarp();
        if (ln > kGwList - 32) gw_drain<kSmall>(T, mask, tab, q, list, ln, lane);
    }
    gw_drain<kSmall>(T, mask, tab, q, list, ln, lane);
}

// ------------------------------------------------------------------ bitmask candidate filter (N <= 256)
// For N <= 256 the candidate offsets of a grain are found as a bitmask over the sample index k: the
// unit interval of frac(offset) is cut into 128 buckets, and for each axis a sparse table holds, for
// every bucket b and level L, the OR of the sample masks of buckets b .. b + 2^L - 1 (cyclic).  The
// cyclic interval [c - h, c + h] of an axis test, rounded out to whole buckets, is the OR of two table
// entries; the AND of the x and y masks is a superset of the pairs that pass both of the tests the
// flattened stage A applies (so of every pair that can set a bit), and those pairs go to stage B.
constexpr int kGbBuckets = 128;
constexpr int kGbLevels = 7;     // spans 1 .. 64 buckets; 128 or more is the full mask
constexpr int kGbMaxWords = 8;   // N <= 256

__host__ __device__ inline bool grainwise_uses_bits(int n) { return n <= 32 * kGbMaxWords; }

// Words between consecutive table entries: W rounded up to odd, so that the lanes of a warp reading
// word w of the entries of different buckets b hit different banks ((b * S + w) mod 32 is one-to-one
// in b mod 32 for odd S); with the stride W = 8 they met on 4 banks.
__host__ __device__ inline int gb_entry_stride(int W) { return W | 1; }

// The samples whose frac(offset) lies in the cyclic interval [c - h, c + h] (c in [0, 1)), rounded out
// to whole buckets, written to m (kAnd = false) or ANDed into it (kAnd = true).
template <int MW, bool kAnd>
__device__ __forceinline__ void gb_axis_mask(const unsigned *tab, int W, int S, float c, float h, int n,
                                             unsigned (&m)[MW]) {
    const int blo = __float2int_rd(FG_FMUL(FG_FSUB(c, h), (float)kGbBuckets));
    const int bhi = __float2int_rd(FG_FMUL(FG_FADD(c, h), (float)kGbBuckets));
    const int len = bhi - blo + 1;
    if (h >= 0.5f || len >= kGbBuckets) {
        if (!kAnd) {
#pragma unroll
            for (int w = 0; w < MW; w++) {
                const int rem = n - 32 * w;
                m[w] = rem >= 32 ? 0xFFFFFFFFu : (rem > 0 ? (1u << rem) - 1u : 0u);
            }
        }
        return;
    }
    const int b0 = blo & (kGbBuckets - 1);
    const int L = 31 - __clz(len);
    const unsigned *e0 = tab + (L * kGbBuckets + b0) * S;
    const unsigned *e1 = tab + (L * kGbBuckets + ((b0 + len - (1 << L)) & (kGbBuckets - 1))) * S;
#pragma unroll
    for (int w = 0; w < MW; w++) {
        const unsigned v = w < W ? (e0[w] | e1[w]) : 0u;
        m[w] = kAnd ? (m[w] & v) : v;
    }
}

// Part `part` of `parts` of a tile: a contiguous range of its 32-pixel batches (a heavy tile is split
// over several CTAs, each with its own copy of the tile's masks; OR makes the result the same).
template <bool kSmall, int MW>
__device__ __forceinline__ void grainwise_tile_bits(const GrainwiseArgs &a, int tile_x, int tile_y,
                                                    unsigned char *smem_raw, int part, int parts) {
    const int W = (a.n + 31) >> 5;
    float2 *offk = reinterpret_cast<float2 *>(smem_raw);                         // [n] (offx, offy) by k
    const int S = gb_entry_stride(W);
    unsigned *tabx = reinterpret_cast<unsigned *>(offk + ((a.n + 1) & ~1));     // [levels][buckets][S]
    unsigned *taby = tabx + kGbLevels * kGbBuckets * S;
    unsigned short *bk = reinterpret_cast<unsigned short *>(taby + kGbLevels * kGbBuckets * S);  // [n] buckets
    int *next_px = reinterpret_cast<int *>(bk + ((a.n + 7) & ~7));             // [4]: batch counter
    unsigned int *mask = reinterpret_cast<unsigned int *>(next_px + 4);
    const int tid = threadIdx.x, lane = tid & 31;

    const int ix0 = tile_x * a.tin_w, iy0 = tile_y * a.tin_h;
    const int ix1 = min(ix0 + a.tin_w, a.in_w), iy1 = min(iy0 + a.tin_h, a.in_h);
    GwTile T;
    T.rx0 = min(a.out_w, (int)floorf((float)ix0 * a.zoom));
    T.ry0 = min(a.out_h, (int)floorf((float)iy0 * a.zoom));
    T.rw = min(a.rmax_w, min(a.out_w, (int)floorf((float)ix1 * a.zoom)) - T.rx0);
    T.rh = min(a.rmax_h, min(a.out_h, (int)floorf((float)iy1 * a.zoom)) - T.ry0);
    T.rw = max(T.rw, 0);
    T.rh = max(T.rh, 0);
    T.words = a.words;
    T.out_w = a.out_w;
    T.flast_x = (float)(a.out_w - 1);
    T.flast_y = (float)(a.out_h - 1);
    T.gmask = a.gmask;
    const int region_words = T.rw * T.rh * a.words;

    // offsets by sample index, and each sample's x / y bucket
    for (int i = tid; i < a.n; i += kGwThreads) {
        const float4 e = a.sorted_offs[i];  // (frac(offy), offx, offy, k)
        const int k = __float_as_int(e.w);
        offk[k] = make_float2(e.y, e.z);
        float fx = FG_FSUB(e.y, floorf(e.y));
        if (!(fx < 1.0f)) fx = 0.0f;  // a tiny negative offset rounds up to 1; cyclically that is 0
        bk[k] =(unsigned short)((int)FG_FMUL(fx, (float)kGbBuckets) | ((int)FG_FMUL(e.x, (float)kGbBuckets) << 8));
    }
    for (int t = tid; t < region_words; t += kGwThreads) mask[t] = 0u;
    const int fw = ix1 - ix0, total = fw * (iy1 - iy0);
    const int nbatch = (total + 31) >> 5;
    const int px_begin = 32 * (int)(((long long)nbatch * part) / parts);
    const int px_end = min(total, 32 * (int)(((long long)nbatch * (part + 1)) / parts));
    if (tid == 0) *next_px = px_begin;
    __syncthreads();
    for (int t = tid; t < 2 * kGbBuckets * W; t += kGwThreads) {  // level 0: one bucket each
        const int axis = t / (kGbBuckets * W), r = t - axis * kGbBuckets * W;
        const int b = r / W, w = r - b * W;
        unsigned bits = 0u;
        for (int j = 0; j < 32; j++) {
            const int k = w * 32 + j;
            if (k < a.n && ((bk[k] >> (8 * axis)) & 0xFF) == b) bits |= 1u << j;
        }
        (axis ? taby : tabx)[b * S + w] = bits;
    }
    __syncthreads();
    for (int L = 1; L < kGbLevels; L++) {
        for (int t = tid; t < 2 * kGbBuckets * W; t += kGwThreads) {
            const int axis = t / (kGbBuckets * W), r = t - axis * kGbBuckets * W;
            const int b = r / W, w = r - b * W;
            unsigned *tb = axis ? taby : tabx;
            const int b2 = (b + (1 << (L - 1))) & (kGbBuckets - 1);
            tb[(L * kGbBuckets + b) * S + w] = tb[((L - 1) * kGbBuckets + b) * S + w] |
                                               tb[((L - 1) * kGbBuckets + b2) * S + w];
        }
        __syncthreads();
    }

    const UniformF32 U = uniform_f32_new(0.0f, 1.0f);
    const float zoom = a.zoom;
    for (;;) {
        // the next 32 footprint pixels of this part (a shared counter balances the warps), one per
        // lane, Poisson set-up in step across the warp
        int base = 0;
        if (lane == 0) base = atomicAdd(next_px, 32);
        base = __shfl_sync(0xffffffffu, base, 0);
        if (base >= px_end) break;
        const int pi = base + lane;
        uint32_t left = 0;
        int px = 0, py = 0;
        Xoshiro rng = {0, 0, 0, 0};
        if (pi < px_end) {
            px = ix0 + pi % fw;
            py = iy0 + pi / fw;
            const float lv = a.lam[(long long)py * a.in_w + px];
            if (lv > 0.0f) {
                rng = pixel_rng(a.seed, px, py);
                const PoissonParams P = poisson_new((double)lv);
                left = poisson_sample(P, rng);
            }
        }
        while (__any_sync(0xffffffffu, left > 0)) {
            // one grain per lane; its candidate samples as a bitmask
            unsigned m[MW];
#pragma unroll
            for (int w = 0; w < MW; w++) m[w] = 0u;
            int cnt = 0;
            float gx = 0.0f, gy = 0.0f, gr = 0.0f;  // this lane's grain: zoomed centre, zoomed radius
            if (left > 0) {
                left--;
                const float cx = FG_FADD((float)px, uniform_f32_from(U, rng.next()));
                const float cy = FG_FADD((float)py, uniform_f32_from(U, rng.next()));
                float r = a.lognorm ? lognormal_radius_f32(a.log_mu, a.log_sigma, rng) : a.radius_mean;
                if (r > a.rm) r = a.rm;
                if (r > 0.0f) {
                    const float ro = FG_FMUL(r, zoom);
                    if (ro > 0.0f) {
                        const float czx = FG_FMUL(cx, zoom), czy = FG_FMUL(cy, zoom);
                        float cyf = FG_FSUB(0.5f, FG_FSUB(czy, floorf(czy)));  // frac(1/2 - czy)
                        if (cyf < 0.0f) cyf = FG_FADD(cyf, 1.0f);
                        float cxf = FG_FSUB(0.5f, FG_FSUB(czx, floorf(czx)));  // frac(1/2 - czx)
                        if (cxf < 0.0f) cxf = FG_FADD(cxf, 1.0f);
                        gx = czx;
                        gy = czy;
                        gr = ro;
                        const float h = FG_FADD(ro, a.frac_eps);
                        gb_axis_mask<MW, false>(tabx, W, S, cxf, h, a.n, m);
                        gb_axis_mask<MW, true>(taby, W, S, cyf, h, a.n, m);
#pragma unroll
                        for (int w = 0; w < MW; w++) cnt += __popc(m[w]);
                    }
                }
            }
            // this step's (grain, sample) pairs, 32 at a time: pair p belongs to the first lane whose
            // inclusive candidate count exceeds p (a binary search over shuffled prefixes), and is the
            // (p - exclusive count)-th set bit of that lane's mask.  Every lane stays converged and the
            // grains never leave the registers of the lanes that drew them.
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            const int tot = __shfl_sync(0xffffffffu, incl, 31);
            for (int b = 0; b < tot; b += 32) {
                const int p = b + lane;
                int src = 0;
#pragma unroll
                for (int step = 16; step > 0; step >>= 1) {
                    const int v = __shfl_sync(0xffffffffu, incl, src + step - 1);
                    if (v <= p) src += step;
                }
                int j = p - (__shfl_sync(0xffffffffu, incl, src) - __shfl_sync(0xffffffffu, cnt, src));
                unsigned word = 0u;
                int wsel = 0;
#pragma unroll
                for (int w = 0; w < MW; w++) {
                    const unsigned mw = __shfl_sync(0xffffffffu, m[w], src);
                    const int c = __popc(mw);
                    if (wsel == w) {
                        if (j < c) word = mw;
                        else { j -= c; wsel = w + 1; }
                    }
                }
                int bit = 0;  // the j-th set bit of `word`
#pragma unroll
                for (int half = 16; half > 0; half >>= 1) {
                    const int c = __popc(word & ((1u << half) - 1u));
                    if (j >= c) {
                        j -= c;
                        bit += half;
                        word >>= half;
                    }
                }
                const float sx = __shfl_sync(0xffffffffu, gx, src);
                const float sy = __shfl_sync(0xffffffffu, gy, src);
                const float sr = __shfl_sync(0xffffffffu, gr, src);
                if (p < tot) {
                    const int k = wsel * 32 + bit;
                    const float2 o = offk[k];
                    gw_splat<kSmall>(T, mask, make_float4(sx, sy, sr, 0.0f), make_float4(0.0f, o.x, o.y, __int_as_float(k)));
                }
            }
        }
    }
    __syncthreads();

    // OR the rectangle's words into the global mask (other CTAs' spills land there too).
    for (int t = tid; t < region_words; t += kGwThreads) {
        const unsigned v = mask[t];
        if (v) {
            const int w = t % a.words, px = t / a.words;
            const int lx = px % T.rw, ly = px / T.rw;
            atomicOr(a.gmask + ((long long)(T.ry0 + ly) * a.out_w + (T.rx0 + lx)) * a.words + w, v);
        }
    }
}

inline size_t grainwise_bits_smem_bytes(const GrainwiseArgs &a) {
    const size_t W = (size_t)(a.n + 31) / 32;
    return (size_t)((a.n + 1) & ~1) * sizeof(float2) +
           2 * (size_t)kGbLevels * kGbBuckets * gb_entry_stride((int)W) * sizeof(unsigned) +
           (size_t)((a.n + 7) & ~7) * sizeof(unsigned short) + 4 * sizeof(int) +
           (size_t)a.rmax_w * a.rmax_h * a.words * sizeof(unsigned int);
}

// The tile variant for n samples: 4 or 8 = the bitmask filter with that many mask words, 0 = the
// flattened stage A (n > 256).
__host__ __device__ inline int grainwise_variant(int n) { return n <= 128 ? 4 : (grainwise_uses_bits(n) ? 8 : 0); }

template <bool kSmall>
__device__ __forceinline__ void grainwise_tile_flat(const GrainwiseArgs &a, int tile_x, int tile_y,
                                                    unsigned char *smem_raw);

// One input tile of the grain-wise kernel (all threads of the CTA; `smem_raw` holds its shared memory).
// kVariant: grainwise_variant(a.n), or -1 to dispatch at run time (the batched kernel).
// parts > 1 splits the tile's pixels over CTAs (bitmask variants only; the flat variant takes whole tiles).
template <bool kSmall, int kVariant = -1>
__device__ __forceinline__ void grainwise_tile(const GrainwiseArgs &a, int tile_x, int tile_y,
                                               unsigned char *smem_raw, int part = 0, int parts = 1) {
    const int v = kVariant >= 0 ? kVariant : grainwise_variant(a.n);
    if (v == 4) grainwise_tile_bits<kSmall, 4>(a, tile_x, tile_y, smem_raw, part, parts);
    else if (v == 8) grainwise_tile_bits<kSmall, kGbMaxWords>(a, tile_x, tile_y, smem_raw, part, parts);
    else grainwise_tile_flat<kSmall>(a, tile_x, tile_y, smem_raw);
}

template <bool kSmall>
__device__ __forceinline__ void grainwise_tile_flat(const GrainwiseArgs &a, int tile_x, int tile_y,
                                                    unsigned char *smem_raw) {
    float4 *tab = reinterpret_cast<float4 *>(smem_raw);                   // [n] offsets, by frac(offx)
    float4 *queue = tab + a.n;                                            // [warps][kGwQueue] grains
    uint2 *qrange = reinterpret_cast<uint2 *>(queue + kGwWarps * kGwQueue); // [warps][kGwQueue]
    unsigned *lists = reinterpret_cast<unsigned *>(qrange + kGwWarps * kGwQueue);  // [warps][kGwList]
    float *fy = reinterpret_cast<float *>(lists + kGwWarps * kGwList);    // [n] frac(offy), table order
    int *cpre = reinterpret_cast<int *>(fy + a.n);                        // [warps][33]
    int *bstart = cpre + kGwWarps * 33;                                   // [kGwBuckets + 1]
    unsigned int *mask = reinterpret_cast<unsigned int *>(bstart + kGwBuckets + 3);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;

    // This CTA's input tile and the output rectangle its mask covers (the zoomed tile).
    const int ix0 = tile_x * a.tin_w, iy0 = tile_y * a.tin_h;
    const int ix1 = min(ix0 + a.tin_w, a.in_w), iy1 = min(iy0 + a.tin_h, a.in_h);
    GwTile T;
    T.rx0 = min(a.out_w, (int)floorf((float)ix0 * a.zoom));
    T.ry0 = min(a.out_h, (int)floorf((float)iy0 * a.zoom));
    T.rw = min(a.rmax_w, min(a.out_w, (int)floorf((float)ix1 * a.zoom)) - T.rx0);
    T.rh = min(a.rmax_h, min(a.out_h, (int)floorf((float)iy1 * a.zoom)) - T.ry0);
    T.rw = max(T.rw, 0);
    T.rh = max(T.rh, 0);
    T.words = a.words;
    T.out_w = a.out_w;
    T.flast_x = (float)(a.out_w - 1);
    T.flast_y = (float)(a.out_h - 1);
    T.gmask = a.gmask;
    const int region_words = T.rw * T.rh * a.words;

    for (int k = tid; k < a.n; k += kGwThreads) {
        const float4 e = a.sorted_offs[k];
        tab[k] = e;
        fy[k] = e.x;
    }
    for (int t = tid; t < region_words; t += kGwThreads) mask[t] = 0u;
    for (int b = tid; b <= kGwBuckets; b += kGwThreads) bstart[b] = a.bucket_start[b];
    __syncthreads();

    const int fw = ix1 - ix0, total = fw * (iy1 - iy0);
    const UniformF32 U = uniform_f32_new(0.0f, 1.0f);
    const float zoom = a.zoom;
    float4 *q = queue + warp * kGwQueue;
    uint2 *qr = qrange + warp * kGwQueue;
    unsigned *list = lists + warp * kGwList;
    int *wc = cpre + warp * 33;

    int qn = 0;  // warp-uniform grain-queue fill
    int ln = 0;  // warp-uniform survivor-list fill
    for (int base = warp * 32; base < total; base += kGwThreads) {
        // one footprint pixel per lane, Poisson set-up in step across the warp
        const int pi = base + lane;
        uint32_t left = 0;
        int px = 0, py = 0;
        Xoshiro rng = {0, 0, 0, 0};
        if (pi < total) {
            px = ix0 + pi % fw;
            py = iy0 + pi / fw;
            const float lv = a.lam[(long long)py * a.in_w + px];
            if (lv > 0.0f) {
                rng = pixel_rng(a.seed, px, py);
                const PoissonParams P = poisson_new((double)lv);
                left = poisson_sample(P, rng);
            }
        }
        while (__any_sync(0xffffffffu, left > 0)) {
            bool valid = false;
            float4 G;
            uint2 R;
            if (left > 0) {
                left--;
                const float cx = FG_FADD((float)px, uniform_f32_from(U, rng.next()));
                const float cy = FG_FADD((float)py, uniform_f32_from(U, rng.next()));
                float r = a.lognorm ? lognormal_radius_f32(a.log_mu, a.log_sigma, rng) : a.radius_mean;
                if (r > a.rm) r = a.rm;
                if (r > 0.0f) {
                    const float ro = FG_FMUL(r, zoom);
                    if (ro > 0.0f) {
                        valid = true;
                        const float czy = FG_FMUL(cy, zoom);
                        float cyf = FG_FSUB(0.5f, FG_FSUB(czy, floorf(czy)));  // frac(1/2 - czy)
                        if (cyf < 0.0f) cyf = FG_FADD(cyf, 1.0f);
                        G = make_float4(FG_FMUL(cx, zoom), czy, ro, cyf);
                        R = gw_candidates(bstart, a.n, G.x, ro, a.frac_eps);
                    }
                }
            }
            const unsigned vb = __ballot_sync(0xffffffffu, valid);
            if (valid) {
                const int slot = qn + __popc(vb & ((1u << lane) - 1u));
                q[slot] = G;
                qr[slot] = R;
            }
            qn += __popc(vb);
            __syncwarp();
            if (qn >= 32) {
                gw_raster_batch<kSmall>(T, mask, tab, fy, q, qr, 32, wc, list, ln, a.frac_eps, lane);
                __syncwarp();
                if (lane + 32 < qn) {
                    q[lane] = q[lane + 32];
                    qr[lane] = qr[lane + 32];
                }
                qn -= 32;
                __syncwarp();
            }
        }
    }
    if (qn > 0) gw_raster_batch<kSmall>(T, mask, tab, fy, q, qr, qn, wc, list, ln, a.frac_eps, lane);
    __syncthreads();

    // OR the rectangle's words into the global mask (other CTAs' spills land there too).
    for (int t = tid; t < region_words; t += kGwThreads) {
        const unsigned v = mask[t];
        if (v) {
            const int w = t % a.words, px = t / a.words;
            const int lx = px % T.rw, ly = px / T.rw;
            atomicOr(a.gmask + ((long long)(T.ry0 + ly) * a.out_w + (T.rx0 + lx)) * a.words + w, v);
        }
    }
}


// Shared-memory bytes of one grain-wise tile.
inline size_t grainwise_tile_smem_bytes(const GrainwiseArgs &a) {
    if (grainwise_uses_bits(a.n)) return grainwise_bits_smem_bytes(a);
    return (size_t)a.n * sizeof(float4) + (size_t)kGwWarps * kGwQueue * sizeof(float4) +
           (size_t)kGwWarps * kGwQueue * sizeof(uint2) + (size_t)kGwWarps * kGwList * sizeof(unsigned) +
           (size_t)a.n * sizeof(float) + ((size_t)kGwWarps * 33 + kGwBuckets + 3) * sizeof(int) +
           (size_t)a.rmax_w * a.rmax_h * a.words * sizeof(unsigned int);
}

}  // namespace fg
