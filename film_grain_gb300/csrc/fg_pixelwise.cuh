// fg_pixelwise.cuh -- device code of the pixel-wise coverage estimator (src/pixelwise.rs:11-106),
// shared by the standalone kernel (fg_pixelwise.cu) and the batched persistent kernel (fg_batch.cu).
#pragma once
#include "fg_kernels.cuh"
#include "fg_rng.cuh"

namespace fg {

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ int f2i_floor(float v) { return __float2int_rz(floorf(v)); }  // Rust `floor() as i32`

__device__ __forceinline__ float xg_of(int x, float inv_zoom, float off) {
    return FG_FSUB(FG_FMUL(FG_FADD((float)x, 0.5f), inv_zoom), off);
}

// First x in [0, n] with xg_of(x) >= X (n when none); xg_of is monotone in x.
static __device__ int first_at_least(float X, int n, float inv_zoom, float zoom, float off) {
    float approx = FG_FSUB(FG_FMUL(FG_FADD(X, off), zoom), 0.5f);
    int guess;
    if (!(approx > -8.0f)) guess = 0;
    else if (!(approx < (float)n + 8.0f)) guess = n;
    else guess = (int)floorf(approx);
    int lo = max(0, guess - 3), hi = min(n, guess + 4);
    if (lo > hi) { lo = 0; hi = n; }
    if (lo > 0 && !(xg_of(lo - 1, inv_zoom, off) < X)) lo = 0;
    if (hi < n && !(xg_of(hi, inv_zoom, off) >= X)) hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (xg_of(mid, inv_zoom, off) >= X) hi = mid;
        else lo = mid + 1;
    }
    return lo;
}

// mix3 (src/rng.rs:40-44) split into its column stage, shared by all cells of column i, and its
// row stage: mix3(seed, CELL, i, j) = cell_row_hash(cell_col_hash(seed, i), j).
__device__ __forceinline__ uint64_t cell_col_hash(unsigned long long seed, int i) {
    return splitmix64(rotl64((seed ^ kCellStream) + (uint64_t)(int64_t)i, 17));
}
__device__ __forceinline__ uint64_t cell_row_hash(uint64_t col, int j) {
    return splitmix64(rotl64(col + (uint64_t)(int64_t)j, 41));
}

// Grain count of the cell with hash h; when q > 0 the stream is left positioned after the Poisson
// draws.  q == 0 is decided from the first draw alone: only state words s0 and s3 (seed words 1, 2, 7
// and 8) enter it.
__device__ __forceinline__ uint32_t cell_count_h(uint64_t h, long long thresh, double exp_lambda, Xoshiro &rng) {
    const long long v = (long long)(small_first_u64(h) >> 11);
    if (v <= thresh) return 0u;
    rng = small_seed(h);
    if (thresh >= 0) {
        (void)rng.next();  // the first draw, already evaluated
        return poisson_knuth_tail(u53_unit((uint64_t)v), exp_lambda, rng);
    }
    PoissonParams P = poisson_new(-exp_lambda);
    return poisson_rejection(P, rng);
}

// Grain count of cell (i, j); when q > 0 the stream is left positioned after the Poisson draws.
__device__ __forceinline__ uint32_t cell_count(unsigned long long seed, int i, int j, const CellParam &cp,
                                               Xoshiro &rng) {
    return cell_count_h(cell_row_hash(cell_col_hash(seed, i), j), cp.thresh, cp.exp_lambda, rng);
}

__device__ __forceinline__ float radius_draw(const PixelwiseArgs &a, Xoshiro &rng) {
    if (!a.lognorm) return a.radius_mean;
    return lognormal_radius_f32(a.log_mu, a.log_sigma, rng);
}

// Index of the lambda pixel of cell (i, j): the cell origin's pixel, clamped to the plane
// (src/pixelwise.rs:69-72).
__device__ __forceinline__ long long cell_pixel(const PixelwiseArgs &a, int i, int j) {
    float sx = FG_FMUL((float)i, a.delta), sy = FG_FMUL((float)j, a.delta);
    long long ix = (long long)floorf(sx), iy = (long long)floorf(sy);
    ix = ix < 0 ? 0 : (ix > a.in_w - 1 ? a.in_w - 1 : ix);
    iy = iy < 0 ? 0 : (iy > a.in_h - 1 ? a.in_h - 1 : iy);
    return iy * (long long)a.in_w + ix;
}

// One cell of the reference's per-sample loop: does a grain of cell (i, j), whose lambda pixel has
// Poisson set-up cp and whose column hash is colh, cover (xg, yg)?  (src/pixelwise.rs:67-103)
__device__ __forceinline__ bool regen_cell(const PixelwiseArgs &a, const UniformF32 &U, float xg, float yg, int i,
                                           int j, uint64_t colh, const CellParam &cp) {
    Xoshiro rng;
    const uint32_t q = cell_count_h(cell_row_hash(colh, j), cp.thresh, cp.exp_lambda, rng);
    if (q == 0) return false;
    const float sx = FG_FMUL((float)i, a.delta), sy = FG_FMUL((float)j, a.delta);
    for (uint32_t g = 0; g < q; g++) {
        float cx = FG_FADD(sx, uniform_f32_from(U, rng.next()));
        float cy = FG_FADD(sy, uniform_f32_from(U, rng.next()));
        float r = radius_draw(a, rng);
        if (r > a.rm) r = a.rm;
        if (r <= 0.0f) continue;
        float dx = FG_FSUB(xg, cx), dy = FG_FSUB(yg, cy);
        if (FG_FADD(FG_FMUL(dx, dx), FG_FMUL(dy, dy)) <= FG_FMUL(r, r)) return true;
    }
    return false;
}

// The reference's per-sample loop (evaluate_indicator, src/pixelwise.rs:47-106), regenerating the
// cells of [i0, i1] x [j0, j1].  The indicator is an OR over the cells, so the visiting order does not
// change it: the middle cell (the sample's own when the range is 3 wide) goes first, as it is the
// likeliest to hold a covering grain, then the others column by column.
static __device__ bool eval_regen(const PixelwiseArgs &a, const UniformF32 &U, float xg, float yg, int i0, int i1,
                                  int j0, int j1) {
    const int ic = i0 + ((i1 - i0) >> 1), jc = j0 + ((j1 - j0) >> 1);
    if (regen_cell(a, U, xg, yg, ic, jc, cell_col_hash(a.seed, ic), a.cells[cell_pixel(a, ic, jc)])) return true;
    for (int i = i0; i <= i1; i++) {
        const uint64_t colh = cell_col_hash(a.seed, i);
        for (int j = j0; j <= j1; j++)
            if ((i != ic || j != jc) && regen_cell(a, U, xg, yg, i, j, colh, a.cells[cell_pixel(a, i, j)]))
                return true;
    }
    return false;
}

// Hit count of output pixel (x, y) over its N samples by the reference's per-sample loop
// (src/pixelwise.rs:30-38 around evaluate_indicator, src/pixelwise.rs:47-106), for sparse and
// moderately dense grains.  Called by all 32 lanes of a warp (neighbouring pixels; `valid` false for
// lanes past the row's end, which take part without samples); the lanes take the samples in step, and
// each sample runs in two phases:
//   1. every cell of its range gets the emptiness test alone (the first uniform against the Poisson
//      threshold, cell_count_h): the same short work on every lane, one column hash per column; the
//      non-empty cells go to a 64-bit mask, cell (i0 + di, j0 + dj) at bit di * 8 + dj with the middle
//      cell swapped into bit 0;
//   2. the (lane, non-empty cell) pairs of the whole warp are dealt out 32 at a time, each lane
//      regenerating one cell's grains against its owner's sample and ORing a hit back to the owner.
//      Lane-major order (kRankMajor false; sparse grains, few pairs): pair p goes to lane p % 32, which
//      finds its owner by a shuffle binary search over the inclusive counts and the cell by a
//      rank-select in the owner's mask (pairs of owners already covered are skipped).  Rank-major
//      order (moderately dense grains): each round deals every uncovered lane's lowest pending cell,
//      then their second cells, and so on, so that a sample covered by its middle cell drops out
//      before the rest of its cells are dealt.
// Coverage is an OR over the cells, so neither the order nor the dealing changes it.  A range wider
// than 8 cells on an axis (outside the plane-level choice of this path) runs the plain loop instead.
template <bool kRankMajor>
__device__ __forceinline__ uint32_t pixelwise_pixel_split(const PixelwiseArgs &a, const UniformF32 &U, int x, int y,
                                                          bool valid) {
    if (!(a.rm > 0.0f)) return 0u;
    const int lane = threadIdx.x & 31;
    uint32_t hits = 0;
    for (int k = 0; k < a.n; k++) {
        float xg = 0.0f, yg = 0.0f;
        int i0 = 0, j0 = 0, mid = 0;
        unsigned long long m = 0ull;
        bool hit = false;
        if (valid) {
            const float2 o = a.offs[k];
            xg = xg_of(x, a.inv_zoom, o.x);
            yg = xg_of(y, a.inv_zoom, o.y);
            i0 = f2i_floor(FG_FDIV(FG_FSUB(xg, a.rm), a.delta));
            const int i1 = f2i_floor(FG_FDIV(FG_FADD(xg, a.rm), a.delta));
            j0 = f2i_floor(FG_FDIV(FG_FSUB(yg, a.rm), a.delta));
            const int j1 = f2i_floor(FG_FDIV(FG_FADD(yg, a.rm), a.delta));
            if (i0 <= i1 && j0 <= j1) {  // else no cell (src/pixelwise.rs:60-62)
                const int ni = i1 - i0 + 1, nj = j1 - j0 + 1;
                if (ni > 8 || nj > 8) {
                    hit = eval_regen(a, U, xg, yg, i0, i1, j0, j1);
                } else {
                    // phase 1
                    mid = ((ni - 1) >> 1) * 8 + ((nj - 1) >> 1);
                    // (the screen may pass a cell whose seed words are all zero: phase 2 counts it exactly)
                    long long pix = -1;
                    uint64_t bound = 0;
                    for (int di = 0; di < ni; di++) {
                        const int i = i0 + di;
                        const uint64_t colh = cell_col_hash(a.seed, i);
                        for (int dj = 0; dj < nj; dj++) {
                            const int j = j0 + dj;
                            const long long p = cell_pixel(a, i, j);
                            if (p != pix) {
                                pix = p;
                                bound = screen_bound(a.cells[p].thresh);
                            }
                            const int idx = di * 8 + dj;
                            const int pos = idx == mid ? 0 : (idx == 0 ? mid : idx);
                            if (first_draw_screen(cell_row_hash(colh, j), bound)) m |= 1ull << pos;
                        }
                    }
                }
            }
        }
        if (kRankMajor) {
            // phase 2: the warp's pairs, 32 per round in rank-major order: first every uncovered lane's
            // lowest pending cell (the middle one when it holds grains), then their second cells, and so
            // on, so that a covered sample drops out before its further cells are dealt.
            for (;;) {
                const bool live = m != 0ull && !hit;
                const int mine = live ? __popcll((long long)m) : 0;
                int owner = -1, rank = 0, before = 0, assigned = 0;
                for (int r = 0; before < 32; r++) {
                    const unsigned mask_r = __ballot_sync(0xffffffffu, mine > r);
                    const int c = __popc(mask_r);
                    if (c == 0) break;
                    if (mine > r && before + __popc(mask_r & ((1u << lane) - 1u)) < 32) assigned++;
                    if (owner < 0 && lane < before + c) {
                        // the (lane - before)-th set bit of mask_r
                        int q = lane - before, bit = 0;
                        unsigned w = mask_r;
#pragma unroll
                        for (int half = 16; half > 0; half >>= 1) {
                            const int cl = __popc(w & ((1u << half) - 1u));
                            if (q >= cl) {
                                q -= cl;
                                bit += half;
                                w >>= half;
                            }
                        }
                        owner = bit;
                        rank = r;
                    }
                    before += c;
                }
                if (before == 0) break;  // no lane has a pending cell
                const int src = owner < 0 ? 0 : owner;
                const unsigned mlo = __shfl_sync(0xffffffffu, (unsigned)m, src);
                const unsigned mhi = __shfl_sync(0xffffffffu, (unsigned)(m >> 32), src);
                const float sx = __shfl_sync(0xffffffffu, xg, src), sy = __shfl_sync(0xffffffffu, yg, src);
                const int si0 = __shfl_sync(0xffffffffu, i0, src), sj0 = __shfl_sync(0xffffffffu, j0, src);
                const int smid = __shfl_sync(0xffffffffu, mid, src);
                bool h = false;
                if (owner >= 0) {
                    // the rank-th set bit of the owner's pending mask
                    int r = rank;
                    unsigned word = mlo;
                    int base = 0;
                    const int c = __popc(mlo);
                    if (r >= c) {
                        r -= c;
                        word = mhi;
                        base = 32;
                    }
                    int bit = 0;
#pragma unroll
                    for (int half = 16; half > 0; half >>= 1) {
                        const int cl = __popc(word & ((1u << half) - 1u));
                        if (r >= cl) {
                            r -= cl;
                            bit += half;
                            word >>= half;
                        }
                    }
                    const int pos = base + bit;
                    const int idx = pos == 0 ? smid : (pos == smid ? 0 : pos);
                    const int i = si0 + (idx >> 3), j = sj0 + (idx & 7);
                    h = regen_cell(a, U, sx, sy, i, j, cell_col_hash(a.seed, i), a.cells[cell_pixel(a, i, j)]);
                }
                const unsigned hm = __reduce_or_sync(0xffffffffu, h ? (1u << src) : 0u);
                hit = hit || ((hm >> lane) & 1u) != 0u;
                for (int t = 0; t < assigned; t++) m &= m - 1ull;  // this round dealt the lowest `assigned` cells
            }
        } else {
            // phase 2: the warp's pairs, 32 at a time in lane-major order
            const int cnt = __popcll((long long)m);
            int incl = cnt;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
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
                src = min(src, 31);
                int r = p - (__shfl_sync(0xffffffffu, incl, src) - __shfl_sync(0xffffffffu, cnt, src));
                const unsigned mlo = __shfl_sync(0xffffffffu, (unsigned)m, src);
                const unsigned mhi = __shfl_sync(0xffffffffu, (unsigned)(m >> 32), src);
                const bool done = __shfl_sync(0xffffffffu, hit ? 1 : 0, src) != 0;
                const float sx = __shfl_sync(0xffffffffu, xg, src), sy = __shfl_sync(0xffffffffu, yg, src);
                const int si0 = __shfl_sync(0xffffffffu, i0, src), sj0 = __shfl_sync(0xffffffffu, j0, src);
                const int smid = __shfl_sync(0xffffffffu, mid, src);
                bool h = false;
                if (p < tot && !done) {
                    // the r-th set bit of the owner's mask
                    unsigned word = mlo;
                    int base = 0;
                    const int c = __popc(mlo);
                    if (r >= c) {
                        r -= c;
                        word = mhi;
                        base = 32;
                    }
                    int bit = 0;
#pragma unroll
                    for (int half = 16; half > 0; half >>= 1) {
                        const int cl = __popc(word & ((1u << half) - 1u));
                        if (r >= cl) {
                            r -= cl;
                            bit += half;
                            word >>= half;
                        }
                    }
                    const int pos = base + bit;
                    const int idx = pos == 0 ? smid : (pos == smid ? 0 : pos);
                    const int i = si0 + (idx >> 3), j = sj0 + (idx & 7);
                    h = regen_cell(a, U, sx, sy, i, j, cell_col_hash(a.seed, i), a.cells[cell_pixel(a, i, j)]);
                }
                const unsigned hm = __reduce_or_sync(0xffffffffu, h ? (1u << src) : 0u);
                hit = hit || ((hm >> lane) & 1u) != 0u;
            }
        }
        hits += hit ? 1u : 0u;
    }
    return hits;
}

// The same hit count for dense grains, where most samples are covered by the first cells they
// visit: the loop is flattened so that each iteration visits ONE cell of the current sample and a
// lane moves on to its next sample as soon as the current one is decided.  Each sample visits its
// middle cell first, then the rest of its range column by column.
__device__ __forceinline__ uint32_t pixelwise_pixel_flat(const PixelwiseArgs &a, const UniformF32 &U, int x,
                                                         int y) {
    if (!(a.rm > 0.0f)) return 0u;
    uint32_t hits = 0;
    int k = 0;
    float xg = 0.0f, yg = 0.0f;
    int i0 = 0, j0 = 0, ni = 0, nj = 0, ic = 0, jc = 0, ri = 0, rj = 0;
    bool active = false, first = false;
    int col_i = 0;
    bool have_col = false;
    uint64_t colh = 0;
    long long pix = -1;
    CellParam cp;
    cp.thresh = 0; cp.exp_lambda = 0.0;
    while (true) {
        if (!active) {
            if (k >= a.n) break;
            const float2 o = a.offs[k];
            xg = xg_of(x, a.inv_zoom, o.x);
            yg = xg_of(y, a.inv_zoom, o.y);
            i0 = f2i_floor(FG_FDIV(FG_FSUB(xg, a.rm), a.delta));
            const int i1 = f2i_floor(FG_FDIV(FG_FADD(xg, a.rm), a.delta));
            j0 = f2i_floor(FG_FDIV(FG_FSUB(yg, a.rm), a.delta));
            const int j1 = f2i_floor(FG_FDIV(FG_FADD(yg, a.rm), a.delta));
            if (i0 > i1 || j0 > j1) {  // src/pixelwise.rs:60-62
                k++;
                continue;
            }
            ni = i1 - i0 + 1;
            nj = j1 - j0 + 1;
            ic = (ni - 1) >> 1;
            jc = (nj - 1) >> 1;
            ri = 0; rj = 0;
            first = true;
            active = true;
        }
        const int i = i0 + (first ? ic : ri), j = j0 + (first ? jc : rj);
        if (!have_col || i != col_i) {
            col_i = i;
            have_col = true;
            colh = cell_col_hash(a.seed, i);
        }
        const long long p = cell_pixel(a, i, j);
        if (p != pix) {
            pix = p;
            cp = a.cells[p];
        }
        const bool hit = regen_cell(a, U, xg, yg, i, j, colh, cp);
        if (first) {
            first = false;
        } else if (++rj == nj) {
            rj = 0;
            ++ri;
        }
        if (ri == ic && rj == jc && ++rj == nj) {  // the middle cell went first: skip it
            rj = 0;
            ++ri;
        }
        if (hit || ri >= ni) {
            hits += hit ? 1u : 0u;
            k++;
            active = false;
        }
    }
    return hits;
}

// The per-sample path for the kPwRegenThreads pixels [x0, x0 + kPwRegenThreads) of row y (one per
// thread of the CTA): each warp (32 neighbouring pixels) votes on its pixels' expected grains per cell
// λδ² and takes the flattened form when most exceed kPwRegenFlatLd, the rank-major two-phase form when
// most exceed kPwRegenRankLd, else the lane-major two-phase form, and writes the hit counts.  Thread 0 adds the CTA's samples and the CTA to the diagnostics
// (regenerated samples, unstaged blocks, blocks).
__device__ __forceinline__ void pixelwise_regen_pixels(const PixelwiseArgs &a, int x0, int y) {
    const int x = x0 + (int)threadIdx.x;
    if (threadIdx.x == 0) {
        const int px = min(kPwRegenThreads, a.out_w - x0);
        atomicAdd(&a.diag[0], (unsigned long long)px * (unsigned long long)a.n);
        atomicAdd(&a.diag[1], 1ull);
        atomicAdd(&a.diag[3], 1ull);
    }
    float ld = 0.0f;  // expected grains per cell at this pixel
    if (x < a.out_w) {
        const int xi = min(a.in_w - 1, max(0, (int)floorf(((float)x + 0.5f) * a.inv_zoom)));
        const int yi = min(a.in_h - 1, max(0, (int)floorf(((float)y + 0.5f) * a.inv_zoom)));
        ld = a.lam[(long long)yi * a.in_w + xi] * a.delta * a.delta;
    }
    const bool flat = __popc(__ballot_sync(0xffffffffu, ld > kPwRegenFlatLd)) >= 16;
    const bool rank_major = __popc(__ballot_sync(0xffffffffu, ld > kPwRegenRankLd)) >= 16;
    const bool valid = x < a.out_w;
    const UniformF32 U = uniform_f32_new(0.0f, a.delta);
    if (flat) {
        if (!valid) return;
        a.out[(long long)y * a.out_w + x] = (float)pixelwise_pixel_flat(a, U, x, y);
    } else {
        const uint32_t hits = rank_major ? pixelwise_pixel_split<true>(a, U, x, y, valid)    // all 32 lanes
                                         : pixelwise_pixel_split<false>(a, U, x, y, valid);
        if (valid) a.out[(long long)y * a.out_w + x] = (float)hits;
    }
}

// Block-wide exclusive scan of one int per thread (any blockDim.x that is a multiple of 32, <= 1024).
__device__ __forceinline__ int block_excl_scan(int v, int *wsum, int *total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = (lane < nwarps) ? wsum[lane] : 0;
        int t = w;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < nwarps) wsum[lane] = t - w;
        if (lane == nwarps - 1) wsum[32] = t;
    }
    __syncthreads();
    int r = wsum[warp] + x - v;
    *total = wsum[32];
    __syncthreads();
    return r;
}

// ------------------------------------------------------------------ shared-memory layout
template <class C>
struct PwShared {
    float4 grains[C::kGrainMax];
    unsigned short pre[kPwCellMax + 8];   // counts, then exclusive prefix (row-major window cells)
    unsigned short list[C::kListMax];     // non-empty cells
    int colix[kPwEdgeMax], rowiy[kPwEdgeMax];
    int4 rect[kPwKChunk];                 // owned pixel rectangle per offset: xa, xe, ya, ye
    int spre[kPwKChunk + 1];
    unsigned int cnt[kPwFootMax];
    int wsum[40];
    int stack[32][3];                     // (level, ix, iy)
    int sp;
    int nlist;
    int total;
    int flags;                            // bit0: overflow, bit1: leaf slow path
    int fx0, fx1, fy0, fy1;               // owned-pixel footprint
    int nsamples;
    float est_grains, est_cells;          // lean pass: expected grains / non-empty cells of the window
    int stop;                             // cancellation seen: the block stops
};



// One root block of the pixel-wise tile kernel (all threads of the CTA; `smem_raw` holds PwShared<C>).
// With C::kDefers and may_defer, a root block whose window is expected to overflow the lean buffers
// (or does overflow them) is left to a fat CTA: the call produces no output and returns true.
template <class C>
__device__ __forceinline__ bool pixelwise_block(const PixelwiseArgs &a, int root_x, int root_y,
                                                unsigned char *smem_raw, bool may_defer = false) {
    PwShared<C> &S = *reinterpret_cast<PwShared<C> *>(smem_raw);
    const int tid = threadIdx.x, nthreads = blockDim.x;
    const bool lean = C::kDefers && may_defer;
    bool deferred = false;
    const UniformF32 U = uniform_f32_new(0.0f, a.delta);
    // the cancellation word, read now and tested after the ownership pass (its latency overlaps it)
    int cancel_seen = 0;
    if (tid == 0 && a.cancel) cancel_seen = *(volatile int *)a.cancel;

    if (tid == 0) {
        S.sp = 1;
        S.stack[0][0] = 0; S.stack[0][1] = root_x; S.stack[0][2] = root_y;
    }
    __syncthreads();

    while (true) {
        __syncthreads();
        if (S.sp == 0) break;
        const int level = S.stack[S.sp - 1][0];
        const int sbx = S.stack[S.sp - 1][1];
        const int sby = S.stack[S.sp - 1][2];
        __syncthreads();
        if (tid == 0) S.sp--;
        const float bs = ldexpf(a.bsize, -level);
        const float X0 = FG_FMUL((float)sbx, bs), X1 = FG_FMUL((float)(sbx + 1), bs);
        const float Y0 = FG_FMUL((float)sby, bs), Y1 = FG_FMUL((float)(sby + 1), bs);

        // ---- staged window of cells
        // Every owned sample has xg in [X0, X1) and computes its cell range with these same rounded
        // operations, which are monotone, so its range lies inside [wi0, wi1] x [wj0, wj1].
        const int wi0 = f2i_floor(FG_FDIV(FG_FSUB(X0, a.rm), a.delta));
        const int wi1 = f2i_floor(FG_FDIV(FG_FADD(X1, a.rm), a.delta));
        const int wj0 = f2i_floor(FG_FDIV(FG_FSUB(Y0, a.rm), a.delta));
        const int wj1 = f2i_floor(FG_FDIV(FG_FADD(Y1, a.rm), a.delta));
        const long long Wc = (long long)wi1 - wi0 + 1, Hc = (long long)wj1 - wj0 + 1;
        const bool window_fits = Wc > 0 && Hc > 0 && Wc <= kPwEdgeMax && Hc <= kPwEdgeMax && Wc * Hc <= kPwCellMax;
        const int nc = window_fits ? (int)(Wc * Hc) : 0;

        bool regen_dense = false;
        if (lean && level == 0) {
            // expected grains and non-empty cells of the window: lambda integrated over its rectangle
            // (a cell takes the lambda of the pixel containing its origin; edge pixels extend outwards)
            const float wx0 = FG_FMUL((float)wi0, a.delta), wx1 = FG_FMUL((float)(wi1 + 1), a.delta);
            const float wy0 = FG_FMUL((float)wj0, a.delta), wy1 = FG_FMUL((float)(wj1 + 1), a.delta);
            const int px0 = (int)floorf(wx0), px1 = (int)floorf(wx1), py0 = (int)floorf(wy0), py1 = (int)floorf(wy1);
            const int nx = px1 - px0 + 1, npx = nx * (py1 - py0 + 1);
            if (tid == 0) { S.est_grains = 0.0f; S.est_cells = 0.0f; }
            __syncthreads();
            float g = 0.0f, c = 0.0f;
            const float inv_cell = 1.0f / (a.delta * a.delta);
            for (int t = tid; t < npx; t += nthreads) {
                const int px = px0 + t % nx, py = py0 + t / nx;
                const float ox = fminf((float)(px + 1), wx1) - fmaxf((float)px, wx0);
                const float oy = fminf((float)(py + 1), wy1) - fmaxf((float)py, wy0);
                if (ox > 0.0f && oy > 0.0f) {
                    const int cx = min(max(px, 0), a.in_w - 1), cy = min(max(py, 0), a.in_h - 1);
                    const float lam = a.lam[(long long)cy * a.in_w + cx];
                    g += lam * ox * oy;
                    c += (1.0f - __expf(-lam * a.delta * a.delta)) * ox * oy * inv_cell;
                }
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                g += __shfl_xor_sync(0xffffffffu, g, o);
                c += __shfl_xor_sync(0xffffffffu, c, o);
            }
            if ((tid & 31) == 0 && (g > 0.0f || c > 0.0f)) {
                atomicAdd(&S.est_grains, g);
                atomicAdd(&S.est_cells, c);
            }
            __syncthreads();
            if (S.est_grains > 0.75f * (float)C::kGrainMax || S.est_cells > 0.75f * (float)C::kListMax) {
                // an interior block's samples (border blocks own fewer)
                const float reach_est = FG_FMUL(FG_FMUL(bs, bs), a.zoom * a.zoom) * (float)a.n * a.regen_cells;
                if (reach_est < kPwRegenOverflow * (float)nc && S.est_cells > kPwRegenDense * (float)nc) {
                    regen_dense = true;
                } else {
                    deferred = true;
                    continue;  // loop head syncs; the stack is empty
                }
            }
        }


        // ---- ownership: rectangles per offset, sample total and pixel footprint
        if (tid == 0) { S.fx0 = 0x7fffffff; S.fx1 = -1; S.fy0 = 0x7fffffff; S.fy1 = -1; S.nsamples = 0; }
        __syncthreads();
        // With N <= kPwKChunk these rectangles are kept for pass C (one chunk).
        const bool one_chunk = a.n <= kPwKChunk;
        {
            int lx0 = 0x7fffffff, lx1 = -1, ly0 = 0x7fffffff, ly1 = -1, ns = 0;
            for (int k = tid; k < a.n; k += nthreads) {
                float2 o = a.offs[k];
                int xa = first_at_least(X0, a.out_w, a.inv_zoom, a.zoom, o.x);
                int xe = first_at_least(X1, a.out_w, a.inv_zoom, a.zoom, o.x);
                int ya = first_at_least(Y0, a.out_h, a.inv_zoom, a.zoom, o.y);
                int ye = first_at_least(Y1, a.out_h, a.inv_zoom, a.zoom, o.y);
                if (one_chunk) S.rect[k] = make_int4(xa, xe, ya, ye);
                if (xe > xa && ye > ya) {
                    ns += (xe - xa) * (ye - ya);
                    lx0 = min(lx0, xa); lx1 = max(lx1, xe);
                    ly0 = min(ly0, ya); ly1 = max(ly1, ye);
                }
            }
            // one shared atomic per warp instead of one per thread
            ns = __reduce_add_sync(0xffffffffu, ns);
            lx0 = __reduce_min_sync(0xffffffffu, lx0);
            lx1 = __reduce_max_sync(0xffffffffu, lx1);
            ly0 = __reduce_min_sync(0xffffffffu, ly0);
            ly1 = __reduce_max_sync(0xffffffffu, ly1);
            if ((tid & 31) == 0 && ns > 0) {
                atomicAdd(&S.nsamples, ns);
                atomicMin(&S.fx0, lx0); atomicMax(&S.fx1, lx1);
                atomicMin(&S.fy0, ly0); atomicMax(&S.fy1, ly1);
            }
        }
        if (tid == 0) {
            S.stop = cancel_seen;
            if (cancel_seen) {
                S.sp = 0;  // drop the block's remaining quadrants too
                *(volatile int *)(a.cancel + 1) = 1;
            }
        }
        __syncthreads();
        if (S.nsamples == 0 || S.stop) continue;
        const int fx0 = S.fx0, fy0 = S.fy0, fw = S.fx1 - S.fx0, fh = S.fy1 - S.fy0;
        const bool use_cnt = (long long)fw * fh <= kPwFootMax;

        // ---- staging or regeneration.  Staging visits every window cell once; regeneration (the
        // reference's own per-sample loop) visits each owned sample's reach of ~regen_cells cells, with
        // an early exit on the first covering grain.  Blocks whose samples reach fewer cells than the
        // window holds (border blocks, which own few samples) regenerate, and so do dense windows that
        // overflow shared memory: they would stage again at every subdivision level, while most of
        // their samples are covered by the first cells they visit.
        const float reach = (float)S.nsamples * a.regen_cells;
        const bool regen = regen_dense || (window_fits && reach < kPwRegenSparse * (float)nc);

        if (use_cnt)
            for (int t = tid; t < fw * fh; t += nthreads) S.cnt[t] = 0u;
        if (tid == 0) { S.nlist = 0; S.flags = 0; }
        if (window_fits && !regen) {
            for (int t = tid; t < Wc; t += nthreads) {
                long long ix = (long long)floorf(FG_FMUL((float)(wi0 + t), a.delta));
                S.colix[t] = (int)(ix < 0 ? 0 : (ix > a.in_w - 1 ? a.in_w - 1 : ix));
            }
            for (int t = tid; t < Hc; t += nthreads) {
                long long iy = (long long)floorf(FG_FMUL((float)(wj0 + t), a.delta));
                S.rowiy[t] = (int)(iy < 0 ? 0 : (iy > a.in_h - 1 ? a.in_h - 1 : iy));
            }
        }
        __syncthreads();

        bool staged = false;
        if (window_fits && !regen) {
            // ---- pass A1: which window cells hold grains.  The first uniform alone decides q == 0
            // (cell_count_h), so every cell costs the same; each thread walks a contiguous run of cells
            // in column-major order, reusing the column stage of the cell hash and the lambda pixel's
            // Poisson set-up along the run -- or, when the plane's emptiness bitmask covers the window
            // (blocks the sparse pass left to this one), reading the cells' bits from it.  Empty cells
            // get count 0; the others join the list (one shared atomic per warp step) and get their
            // count in A2.
            {
                const int per = (nc + nthreads - 1) / nthreads;
                const int c0 = tid * per, c1 = min(nc, c0 + per);
                const int lane = tid & 31;
                int ci = c0 / (int)Hc, cj = c0 % (int)Hc;
                int col = -1, pix = -1;
                uint64_t colh = 0, bound = 0;
                const bool from_mask = a.cellmask != nullptr && wi0 >= a.cm_gi0 &&
                                       wi0 + (int)Wc <= a.cm_gi0 + a.cm_gw && wj0 >= a.cm_gj0 &&
                                       wj0 + (int)Hc <= a.cm_gj0 + 32 * a.cm_ghw;
                long long mword_at = -1;
                unsigned mword = 0u;
                for (int step = 0; step < per; step++) {
                    const int c = c0 + step;
                    bool nonempty = false;
                    int rc = 0;
                    if (c < c1) {
                        rc = cj * (int)Wc + ci;
                        if (from_mask) {
                            const int gr = wj0 + cj - a.cm_gj0;
                            const long long at = (long long)(gr >> 5) * a.cm_gw + (wi0 + ci - a.cm_gi0);
                            if (at != mword_at) {
                                mword_at = at;
                                mword = __ldg(a.cellmask + at);
                            }
                            nonempty = ((mword >> (gr & 31)) & 1u) != 0u;
                        } else {
                            if (ci != col) {
                                col = ci;
                                colh = cell_col_hash(a.seed, wi0 + ci);
                            }
                            const int p = S.rowiy[cj] * a.in_w + S.colix[ci];
                            if (p != pix) {
                                pix = p;
                                bound = screen_bound(a.cells[p].thresh);
                            }
                            nonempty = first_draw_screen(cell_row_hash(colh, wj0 + cj), bound);
                        }
                        // (a cell whose seed words are all zero may pass: A2 counts it exactly)
                        if (!nonempty) S.pre[rc] = 0;
                        if (++cj == (int)Hc) {
                            cj = 0;
                            ci++;
                        }
                    }
                    const unsigned nb = __ballot_sync(0xffffffffu, nonempty);
                    if (nb) {
                        int slot0 = 0;
                        if (lane == __ffs(nb) - 1) slot0 = atomicAdd(&S.nlist, __popc(nb));
                        slot0 = __shfl_sync(0xffffffffu, slot0, __ffs(nb) - 1);
                        const int idx = slot0 + __popc(nb & ((1u << lane) - 1u));
                        if (nonempty && idx < C::kListMax) S.list[idx] = (unsigned short)rc;
                    }
                }
            }
            __syncthreads();
            const bool list_overflow = S.nlist > C::kListMax;  // handled like a grain overflow below
            // ---- pass A2: the grain counts of the non-empty cells, one cell per thread
            if (!list_overflow) {
                const int nl = S.nlist;
                for (int t = tid; t < nl; t += nthreads) {
                    const int rc = S.list[t];
                    const int ci = rc % (int)Wc, cj = rc / (int)Wc;
                    const CellParam cp = a.cells[(long long)S.rowiy[cj] * a.in_w + S.colix[ci]];
                    Xoshiro rng;
                    const uint32_t q = cell_count_h(cell_row_hash(cell_col_hash(a.seed, wi0 + ci), wj0 + cj), cp.thresh,
                                                    cp.exp_lambda, rng);
                    S.pre[rc] = (unsigned short)(q > 65535u ? 65535u : q);
                }
            }
            __syncthreads();
            // ---- exclusive prefix over the counts (each thread owns a contiguous run)
            if (list_overflow) {
                if (tid == 0) S.flags |= 1;
            } else {
                const int per = (nc + nthreads - 1) / nthreads;
                const int b = tid * per, e = min(nc, b + per);
                int local = 0;
                for (int c = b; c < e; c++) local += S.pre[c];
                int total;
                int run = block_excl_scan(local, S.wsum, &total);
                if (total <= C::kGrainMax) {
                    for (int c = b; c < e; c++) {
                        int q = S.pre[c];
                        S.pre[c] = (unsigned short)run;
                        run += q;
                    }
                }
                if (tid == 0) {
                    S.pre[nc] = (unsigned short)(total <= C::kGrainMax ? total : 0);
                    S.total = total;
                    if (total > C::kGrainMax) S.flags |= 1;
                }
            }
            __syncthreads();
            if (S.flags & 1) {
                if (reach < kPwRegenOverflow * (float)nc && (float)S.nlist > kPwRegenDense * (float)nc) {
                    // regenerated in pass C (staged stays false)
                } else if (lean && level == 0) {  // a fat CTA takes this block whole
                    deferred = true;
                    continue;  // loop head syncs; the stack is empty
                } else if (level < kPwMaxLevel) {
                    if (tid == 0) {
                        atomicAdd(&a.diag[2], 1ull);
                        for (int q = 0; q < 4; q++) {
                            int s = S.sp++;
                            S.stack[s][0] = level + 1;
                            S.stack[s][1] = 2 * sbx + (q & 1);
                            S.stack[s][2] = 2 * sby + (q >> 1);
                        }
                    }
                    continue;  // loop head syncs
                }
            } else {
                staged = true;
            }
        }
        if (!staged && tid == 0) atomicAdd(&a.diag[1], 1ull);

        if (staged) {
            // ---- pass B: regenerate the non-empty cells' grains into their CSR slots
            const int nl = S.nlist;
            for (int t = tid; t < nl; t += nthreads) {
                const int c = S.list[t];
                const int ci = c % (int)Wc, cj = c / (int)Wc;
                const int i = wi0 + ci, j = wj0 + cj;
                const CellParam cp = a.cells[(long long)S.rowiy[cj] * a.in_w + S.colix[ci]];
                const int base = S.pre[c], end = S.pre[c + 1];  // pass A's slot range for this cell
                uint32_t q = (uint32_t)(end - base);
                Xoshiro rng;
                if (cp.thresh >= 0) {
                    // Knuth regime: the Poisson draw consumed exactly q + 1 uniforms; skip them.
                    rng = small_seed(cell_row_hash(cell_col_hash(a.seed, i), j));
                    for (uint32_t u = 0; u <= q; u++) (void)rng.next();
                } else {
                    q = min(q, cell_count(a.seed, i, j, cp, rng));
                }
                const float sx = FG_FMUL((float)i, a.delta), sy = FG_FMUL((float)j, a.delta);
                for (uint32_t g = 0; g < q; g++) {
                    float cx = FG_FADD(sx, uniform_f32_from(U, rng.next()));
                    float cy = FG_FADD(sy, uniform_f32_from(U, rng.next()));
                    float r = radius_draw(a, rng);
                    if (r > a.rm) r = a.rm;
                    float rr = (r <= 0.0f) ? -1.0f : FG_FMUL(r, r);  // -1 never passes the disk test
                    S.grains[base + g] = make_float4(cx, cy, rr, 0.0f);
                }
            }
            __syncthreads();
        }

        // ---- pass C: evaluate the owned samples, offsets in chunks
        unsigned long long slow = 0;
        for (int k0 = 0; k0 < a.n; k0 += kPwKChunk) {
            const int kn = min(kPwKChunk, a.n - k0);
            int cntk = 0;
            if (tid < kn) {
                int4 R;
                if (one_chunk) {
                    R = S.rect[tid];
                } else {
                    float2 o = a.offs[k0 + tid];
                    R.x = first_at_least(X0, a.out_w, a.inv_zoom, a.zoom, o.x);
                    R.y = first_at_least(X1, a.out_w, a.inv_zoom, a.zoom, o.x);
                    R.z = first_at_least(Y0, a.out_h, a.inv_zoom, a.zoom, o.y);
                    R.w = first_at_least(Y1, a.out_h, a.inv_zoom, a.zoom, o.y);
                    S.rect[tid] = R;
                }
                if (R.y > R.x && R.w > R.z) cntk = (R.y - R.x) * (R.w - R.z);
            }
            int tot;
            int off = block_excl_scan(tid < kPwKChunk ? cntk : 0, S.wsum, &tot);
            if (tid < kPwKChunk) S.spre[tid] = off;
            if (tid == 0) S.spre[kPwKChunk] = tot;
            __syncthreads();
            for (int s = tid; s < tot; s += nthreads) {
                int lo = 0, hi = kn - 1;  // last kk with spre[kk] <= s
                while (lo < hi) {
                    int mid = (lo + hi + 1) >> 1;
                    if (S.spre[mid] <= s) lo = mid;
                    else hi = mid - 1;
                }
                const int kk = lo;
                const int4 R = S.rect[kk];
                const int w = R.y - R.x;
                const int l = s - S.spre[kk];
                const int x = R.x + l % w, y = R.z + l / w;
                const float2 o = a.offs[k0 + kk];
                const float xg = xg_of(x, a.inv_zoom, o.x);
                const float yg = xg_of(y, a.inv_zoom, o.y);
                bool hit = false;
                if (a.rm > 0.0f) {
                    const int i0 = f2i_floor(FG_FDIV(FG_FSUB(xg, a.rm), a.delta));
                    const int i1 = f2i_floor(FG_FDIV(FG_FADD(xg, a.rm), a.delta));
                    const int j0 = f2i_floor(FG_FDIV(FG_FSUB(yg, a.rm), a.delta));
                    const int j1 = f2i_floor(FG_FDIV(FG_FADD(yg, a.rm), a.delta));
                    if (i0 <= i1 && j0 <= j1) {
                        if (staged && i0 >= wi0 && i1 <= wi1 && j0 >= wj0 && j1 <= wj1) {
                            const int ci0 = i0 - wi0, ci1 = i1 - wi0;
                            for (int j = j0; j <= j1 && !hit; j++) {
                                const int row = (j - wj0) * (int)Wc;
                                const int gs = S.pre[row + ci0], ge = S.pre[row + ci1 + 1];
                                for (int g = gs; g < ge; g++) {
                                    const float4 G = S.grains[g];
                                    const float dx = FG_FSUB(xg, G.x), dy = FG_FSUB(yg, G.y);
                                    if (FG_FADD(FG_FMUL(dx, dx), FG_FMUL(dy, dy)) <= G.z) { hit = true; break; }
                                }
                            }
                        } else {
                            slow++;
                            hit = eval_regen(a, U, xg, yg, i0, i1, j0, j1);
                        }
                    }
                }
                if (hit) {
                    const bool in_foot = use_cnt && x >= fx0 && x - fx0 < fw && y >= fy0 && y - fy0 < fh;
                    if (in_foot) atomicAdd(&S.cnt[(y - fy0) * fw + (x - fx0)], 1u);
                    else atomicAdd(&a.out[(long long)y * a.out_w + x], 1.0f);
                }
            }
            __syncthreads();
        }
        if (slow) atomicAdd(&a.diag[0], slow);

        // ---- flush per-pixel counts
        if (use_cnt) {
            for (int t = tid; t < fw * fh; t += nthreads) {
                unsigned c = S.cnt[t];
                if (c) atomicAdd(&a.out[(long long)(fy0 + t / fw) * a.out_w + (fx0 + t % fw)], (float)c);
            }
        }
        if (tid == 0) atomicAdd(&a.diag[3], 1ull);
    }
    return deferred;
}


}  // namespace fg
