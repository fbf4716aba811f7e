// fg_pixelwise_sparse.cuh -- the sparse block pass of the pixel-wise coverage estimator
// (src/pixelwise.rs:11-106): the first pass over every block of a plane whose grains are sparse
// enough to stage a large window in shared memory.  Blocks that turn out denser are left to the fat
// block pass (pixelwise_block<PwFat>), as the fat-grid blocks they cover.
//
// A CTA owns a square block of input space [X0, X1) x [Y0, Y1) (edge a power of two, `ratio` fat-grid
// blocks per side) and evaluates every sample (pixel, offset) whose point xg = ((x + 0.5) * inv_zoom) -
// offsets_input[k] lands in it:
//   0. (cell_mask_kernel, before the pass) the emptiness of every cell of the plane's cell grid is one
//      bit of a column-major bitmask in global memory: a thread owns one column and 32 rows (the column
//      stage of the cell hash computed once) and stores one word; a cell is empty when its first
//      uniform does not exceed its Knuth threshold (cell_count_h).  Every cell is hashed once per plane;
//   1. the CTA copies the bits of its window -- the cells its owned samples can reach -- into shared
//      memory (column-major: word k of window column c holds rows 32k .. 32k + 31);
//   2. the set bits, ranked in column-major order, list the non-empty cells; their grain counts (the
//      Poisson draws of src/pixelwise.rs:77-82) are prefix-summed into a CSR over the list and their
//      grains (centre, radius^2) regenerated into shared memory;
//   3. sample-major: each thread takes the owned pixels of one offset (or a share of them) and runs the
//      reference's per-sample test: for each cell column i0..i1 of the sample's range
//      (src/pixelwise.rs:55-58), the bits of rows j0..j1 are cut from the mask, and when any is set
//      their grains -- contiguous in the CSR, since cells of one column follow each other in the list
//      -- get the disk test dx*dx + dy*dy <= r*r (src/pixelwise.rs:96-99);
//      or grain-major (sparse_grain_pass), when a grain's reach is below half an output pixel and the
//      cost model favours it: a warp takes 32 staged grains, lists the candidate samples within their
//      radii through a table of the offsets binned by their phase, gives the candidates the same disk
//      test 32 at a time, and sets a bit per covered sample whose range holds the grain's cell;
//   4. hit counts go to per-pixel shared counters, then to the output plane (integers, exact in f32).
// The indicator is an OR over the grains of the sample's cells, so the result equals the reference's
// early-exit loop bit for bit.
#pragma once
#include "fg_pixelwise.cuh"

namespace fg {

struct PwSparse {
    static constexpr int kThreads = 256, kCtasPerSm = 3;
    static constexpr int kGrainMax = 2048;   // staged grains
    static constexpr int kListMax = 2048;    // non-empty cells of the window
    static constexpr int kMaskWords = 1280;  // window bitmask, columns an odd number of words apart
    static constexpr int kRowsMax = 256;     // window rows
    static constexpr int kRangeSlots = 4;    // tabulated cell ranges per offset and axis
    static constexpr int kGmBins = 16;       // phase bins per axis of the grain-major form's offset table
    static constexpr int kGmBitsWords = 1024;  // owned-sample bits of the grain-major form
    static constexpr int kGmHitMax = 2560;     // disk tests passed, listed for the hits' pass
    static constexpr int kGmPairs = 256;       // a warp's queue of (grain, entry) candidates
};

// Mask words per window column in shared memory: the column's words rounded up to an odd count, so
// that lanes reading the same word row of columns a multiple of 8 apart meet on different banks.
__host__ __device__ __forceinline__ int sparse_col_stride(int hw) { return hw | 1; }

// A sample's cell range on one axis, relative to the window [w0, w1] (at most kMaskWords cells): low
// 11 bits the first cell - w0, high 5 bits the last cell - the first; kRangeSlow when the range leaves
// the window or spans more than 32 cells (the per-sample loop decides such samples).
constexpr unsigned kRangeSlow = 0xFFFFu;
__device__ __forceinline__ unsigned sparse_range_code(float g, float rm, float delta, int w0, int w1) {
    const int c0 = f2i_floor(FG_FDIV(FG_FSUB(g, rm), delta));  // src/pixelwise.rs:55-58
    const int c1 = f2i_floor(FG_FDIV(FG_FADD(g, rm), delta));
    if (c0 < w0 || c1 > w1 || c1 < c0 || c1 - c0 > 31) return kRangeSlow;
    return (unsigned)(c0 - w0) | ((unsigned)(c1 - c0) << 11);
}

// The window's cells (steps 1 and 2, and step 3 in the sample-major form).
struct PwSparseWindow {
    uint2 mask2[PwSparse::kMaskWords];           // (word w, the next word of the same column or 0)
    unsigned short wrank[PwSparse::kMaskWords];  // non-empty cells before each mask word (column-major)
    unsigned short list[PwSparse::kListMax];     // non-empty cells: window index i * Hc + j, column-major
    unsigned int gsc[PwSparse::kListMax];        // per listed cell: first grain | grain count << 16
};
// Step 3 in the grain-major form (sparse_grain_major), written once the window's cells are read.
struct PwSparseGrainMajor {
    float4 ent[kPwKChunk];                       // the offsets by phase bin: o.x, o.y, o.x * zoom, o.y * zoom
    unsigned short k[kPwKChunk];                 // the entry's offset (index into the x-sorted offsets)
    unsigned short start[PwSparse::kGmBins * PwSparse::kGmBins + 8];  // first entry of each bin, then n
    int base[kPwKChunk];                         // first bit of each offset's owned samples
    unsigned int bits[PwSparse::kGmBitsWords];   // one per owned sample: covered by a grain already
    unsigned int hits[PwSparse::kGmHitMax];      // (grain, entry) pairs that passed the disk test
    unsigned short pairs[(PwSparse::kThreads / 32) * PwSparse::kGmPairs];  // per warp: lane << 8 | entry
};

struct PwSparseShared {
    float4 grains[PwSparse::kGrainMax];          // centre, r^2, window cell (i - wi0) | (j - wj0) << 16 as bits
    union {
        PwSparseWindow w;
        PwSparseGrainMajor gm;
    };
    int4 rect[kPwKChunk];                       // owned pixel rectangle per offset: xa, xe, ya, ye
    // cell ranges (sparse_range_code) of the first kRangeSlots columns and rows of each offset's
    // rectangle: entry [slot * n + k]
    unsigned short range_x[PwSparse::kRangeSlots * kPwKChunk], range_y[PwSparse::kRangeSlots * kPwKChunk];
    unsigned int cnt[kPwFootMax];
    int wsum[40];
    int wi0, wi1, wj0, wj1, Wc, Hc, hw, hs;     // the window: cells [wi0, wi1] x [wj0, wj1], hw words per
                                                // column stored hs = sparse_col_stride(hw) words apart
    int fx0, fx1, fy0, fy1, nsamples;           // owned-pixel footprint, owned samples
    int rw_min, rw_max, rh_min, rh_max;         // extremes of the offsets' rectangle widths and heights
    int stop, ngrains, any_slow;                // any_slow: a tabulated range code is kRangeSlow
    int nhits;                                  // disk tests passed in the grain-major form
    float est_grains, est_cells;
};

static_assert(sizeof(PwSparseGrainMajor) <= sizeof(PwSparseWindow), "the grain-major tables fit the window's space");
static_assert(PwSparse::kGrainMax <= 2048, "a listed hit holds the grain in 11 bits");
static_assert(kPwKChunk <= 256, "a queued candidate holds the entry in 8 bits");

// The CTA's PwSparseShared: the start of its dynamic shared memory, named through the shared array
// itself, so that the out-of-line functions below address it as shared memory (a reference passed in
// would reach them as a generic address).
__device__ __forceinline__ PwSparseShared &sparse_smem() {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    return *reinterpret_cast<PwSparseShared *>(smem_raw);
}

// Geometry of the sparse pass: block edge `bs` (input pixels) = ratio x the fat grid's edge, block grid
// origin and width (the fat grid is (a.bx0, a.by0, a.nbx) with a.bsize); and the plane's emptiness
// bitmask: cells [gi0, gi0 + gw) x [gj0, gj0 + 32 ghw), word (c, k) = cellmask[k * gw + c] holding rows
// gj0 + 32k .. + 31 of column gi0 + c (bit r = row gj0 + 32k + r).
struct PwSparseGrid {
    float bs;
    int ratio;
    int sbx0, sby0, nsbx, nsby;
    const unsigned int *cellmask;
    int gi0, gj0, gw, ghw;
    // the grain-major form of step 3 (sparse_grain_major); gm_ent null when the plane does not allow it
    const float4 *gm_ent;   // [n] the x-sorted offsets by phase bin (PwSparseGrainMajor::ent)
    const int *gm_idx;      // [n] each entry's offset, then [kGmBins^2 + 1] each bin's first entry
    float gm_eps;           // rounding margin of a grain's phase band, in output pixels
    int gm_noslow;          // no sample's cell range can span more than 32 cells (none leaves its window)
    float gm_grain_cost, gm_sample_cost;  // modelled instructions per staged grain / per owned sample
};

// The plane's emptiness bitmask (step 0): thread t = (word row k = t / gw, column c = t % gw).
__device__ __forceinline__ void cell_mask_word(const PixelwiseArgs &a, const PwSparseGrid &g, long long t,
                                               unsigned int *cellmask) {
    const int c = (int)(t % g.gw), k = (int)(t / g.gw);
    const int i = g.gi0 + c;
    const uint64_t colh = cell_col_hash(a.seed, i);
    // the cell's lambda pixel, clamped to the plane (cell_pixel); cell coordinates stay far inside int,
    // so the clamp is done on floats and the conversion is a 32-bit one
    const int ix = (int)fminf(fmaxf(floorf(FG_FMUL((float)i, a.delta)), 0.0f), (float)(a.in_w - 1));
    auto iy_of = [&](int j) {
        return (int)fminf(fmaxf(floorf(FG_FMUL((float)j, a.delta)), 0.0f), (float)(a.in_h - 1));
    };
    const int jb = g.gj0 + 32 * k;
    // iy_of is nondecreasing in j (rounding and floor are monotone), so the word's 32 rows take at most
    // a few pixel rows: one when the first and last agree, two when they differ by one (the boundary
    // found by bisection); otherwise each row is looked up
    const int iy0 = iy_of(jb), iy1 = iy_of(jb + 31);
    const long long t0 = a.cells[(long long)iy0 * a.in_w + ix].thresh;
    // The row stage of mix3 is fmix64(rotl64(col + j, 41) + phi).  With base = col + jb, when adding
    // r < 32 carries nothing out of base's low 23 bits, rotl64(base + r, 41) = rotl64(base, 41) + r * 2^41,
    // so the row hash's input is one constant plus r * 2^41 (only its high word changes); a word whose
    // rows would carry (31 in 2^23) takes the row hash as is.
    const uint64_t base = colh + (uint64_t)(int64_t)jb;
    const uint64_t c0 = rotl64(base, 41) + kPhi;
    auto scan = [&](auto row_hash) {
        unsigned int word = 0;
        if (iy1 <= iy0 + 1) {
            int rb = 32;  // first row of pixel row iy1
            long long t1 = t0;
            if (iy1 != iy0) {
                int lo = 1, hi = 31;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (iy_of(jb + mid) == iy1) hi = mid;
                    else lo = mid + 1;
                }
                rb = lo;
                t1 = a.cells[(long long)iy1 * a.in_w + ix].thresh;
            }
            // the first-draw test as first_draw_screen: a cell whose seed words are all zero is listed and
            // counted exactly by the sparse pass (sparse_cell_count)
            auto bit = [&](int r, uint64_t m) -> unsigned { return (first_draw_screen(row_hash(r), m) ? 1u : 0u) << r; };
            // rows before rb take pixel row iy0's threshold, the others iy1's
            const uint64_t m0 = screen_bound(t0), m1 = screen_bound(t1);
#pragma unroll 4
            for (int r = 0; r < rb; r++) word |= bit(r, m0);
#pragma unroll 4
            for (int r = rb; r < 32; r++) word |= bit(r, m1);
        } else {
            int iy_prev = iy0;
            long long thresh = t0;
#pragma unroll 4
            for (int r = 0; r < 32; r++) {
                const int iy = iy_of(jb + r);
                if (iy != iy_prev) {
                    iy_prev = iy;
                    thresh = a.cells[(long long)iy * a.in_w + ix].thresh;
                }
                const long long v = (long long)(small_first_u64(row_hash(r)) >> 11);
                word |= (v > thresh ? 1u : 0u) << r;
            }
        }
        return word;
    };
    const unsigned int word = (base & 0x7FFFFFull) <= 0x7FFFFFull - 31
                                  ? scan([&](int r) { return fmix64(c0 + ((uint64_t)r << 41)); })
                                  : scan([&](int r) { return cell_row_hash(colh, jb + r); });
    cellmask[t] = word;
}

// The reference's per-sample loop for a sample the staged window cannot serve (out of line: rare).
__device__ __noinline__ bool sparse_regen_sample(const PixelwiseArgs &a, float xg, float yg, int i0, int i1, int j0,
                                                 int j1) {
    const UniformF32 U = uniform_f32_new(0.0f, a.delta);
    return eval_regen(a, U, xg, yg, i0, i1, j0, j1);
}

// Grain count of cell (i, j), which the emptiness bitmask lists as non-empty, with the stream left
// after the Poisson draws: cell_count_h with the seeded stream's first output as its first draw (no
// separate first-draw hash).
__device__ __forceinline__ uint32_t sparse_cell_count(const PixelwiseArgs &a, int i, int j, Xoshiro *rng) {
    const CellParam cp = a.cells[cell_pixel(a, i, j)];
    Xoshiro r = small_seed(cell_row_hash(cell_col_hash(a.seed, i), j));
    uint32_t q;
    if (cp.thresh >= 0) {
        // the first draw (above the threshold for every listed cell but one whose seed words 1, 2, 7 and
        // 8 are all zero, which the bitmask lists to be safe)
        const uint64_t v = r.next() >> 11;
        q = (long long)v > cp.thresh ? poisson_knuth_tail(u53_unit(v), cp.exp_lambda, r) : 0u;
    } else {
        const PoissonParams P = poisson_new(-cp.exp_lambda);
        q = poisson_rejection(P, r);
    }
    *rng = r;
    return q;
}

// The fat-grid blocks of sparse block (sbx, sby), appended to the deferred list (list[0] = count).
__device__ __forceinline__ void sparse_defer(const PixelwiseArgs &a, const PwSparseGrid &g, int sbx, int sby,
                                             int nby, int *list) {
    for (int q = 0; q < g.ratio * g.ratio; q++) {
        const int bx = sbx * g.ratio + q % g.ratio, by = sby * g.ratio + q / g.ratio;
        if (bx < a.bx0 || bx >= a.bx0 + a.nbx || by < a.by0 || by >= a.by0 + nby) continue;
        list[1 + atomicAdd(list, 1)] = (by - a.by0) * a.nbx + (bx - a.bx0);
    }
}

// Sample (xg, yg) with cell-range codes rx, ry (neither kRangeSlow): 1 covered, else 0.  For each cell
// column of the range (src/pixelwise.rs:55-58) one 64-bit shared load gives the bits of its rows; the
// grains of the non-empty cells get the disk test (src/pixelwise.rs:96-99).  The columns are scanned
// first, branch-free, into a mask of the ones holding non-empty cells, and only those are visited: a
// warp's lanes then diverge over their few non-empty columns instead of over every column.
__device__ __forceinline__ int sparse_sample_hit(const PwSparseShared &S, float xg, float yg, unsigned rx,
                                                 unsigned ry) {
    const int hs = S.hs;
    const int c0 = (int)(rx & 0x7FFu), ncol = (int)(rx >> 11);
    const int r0 = (int)(ry & 0x7FFu), b0 = r0 & 31;
    const unsigned keep = (2u << (ry >> 11)) - 1u;  // span <= 31: 2u << 31 wraps to 0 and keep is all ones
    const unsigned below = (1u << b0) - 1u;
    const int w0 = c0 * hs + (r0 >> 5);
    unsigned cols = 0u;
    for (int i = 0; i <= ncol; i++) {
        const uint2 m = S.w.mask2[w0 + i * hs];
        cols |= ((__funnelshift_r(m.x, m.y, b0) & keep) != 0u ? 1u : 0u) << i;
    }
    while (cols) {
        const int w = w0 + (__ffs(cols) - 1) * hs;
        cols &= cols - 1u;
        const uint2 m = S.w.mask2[w];
        unsigned bits = __funnelshift_r(m.x, m.y, b0) & keep;
        int rank = S.w.wrank[w] + __popc(m.x & below);
        do {  // the column's non-empty cells of the range, in row order
            bits &= bits - 1u;
            const unsigned sc = S.w.gsc[rank++];
            const int g0 = (int)(sc & 0xFFFFu), ge = g0 + (int)(sc >> 16);
            for (int g = g0; g < ge; g++) {
                const float4 G = S.grains[g];
                const float dx = FG_FSUB(xg, G.x), dy = FG_FSUB(yg, G.y);
                if (FG_FADD(FG_FMUL(dx, dx), FG_FMUL(dy, dy)) <= G.z) return 1;
            }
        } while (bits);
    }
    return 0;
}

// The second pass over a thread's samples: the ones whose range left the window.
__device__ __noinline__ void sparse_slow_sample(const PixelwiseArgs &a, float xg, float yg, int x, int y);

__device__ __forceinline__ void sparse_count_hit(const PixelwiseArgs &a, PwSparseShared &S, int x, int y) {
    const int fw = S.fx1 - S.fx0, fh = S.fy1 - S.fy0;
    if ((long long)fw * fh <= kPwFootMax && x >= S.fx0 && x - S.fx0 < fw && y >= S.fy0 && y - S.fy0 < fh)
        atomicAdd(&S.cnt[(y - S.fy0) * fw + (x - S.fx0)], 1u);
    else
        atomicAdd(&a.out[(long long)y * a.out_w + x], 1.0f);
}

// Step 3.  The offsets are sorted by x, and consecutive threads take consecutive offsets, each walking
// the pixels its offset owns (`parts` threads per offset, taking alternate rows, when N < the CTA
// size): a warp's lanes evaluate samples of about the same pixel whose points lie close together in x,
// so their mask loads fall on neighbouring columns.  Cell ranges come from the table the ownership pass
// filled when every rectangle fits it, else they are computed here.
// One pass over the thread's samples: pass 0 evaluates every sample from the staged window and counts
// the ones whose range leaves it; pass 1 sends exactly those to the per-sample loop (and counts them).
template <int kPass>
__device__ __forceinline__ unsigned sparse_sample_pass(const PixelwiseArgs &a, PwSparseShared &S) {
    using C = PwSparse;
    const int tid = threadIdx.x, nthreads = blockDim.x;
    unsigned slow = 0;
    const bool table = S.rw_max <= C::kRangeSlots && S.rh_max <= C::kRangeSlots;
    const int parts = a.n >= nthreads ? 1 : nthreads / a.n;
    const int wi0 = S.wi0, wi1 = S.wi1, wj0 = S.wj0, wj1 = S.wj1;
    for (int t = tid; t < a.n * parts; t += nthreads) {
        const int k = t % a.n, p = t / a.n;
        const int4 R = S.rect[k];
        const float2 o = a.offs[k];
        for (int y = R.z + p; y < R.w; y += parts) {
            const float yg = xg_of(y, a.inv_zoom, o.y);
            const unsigned ry = table ? S.range_y[(y - R.z) * a.n + k]
                                      : sparse_range_code(yg, a.rm, a.delta, wj0, wj1);
            for (int x = R.x; x < R.y; x++) {
                const float xg = xg_of(x, a.inv_zoom, o.x);
                const unsigned rx = table ? S.range_x[(x - R.x) * a.n + k]
                                          : sparse_range_code(xg, a.rm, a.delta, wi0, wi1);
                const bool out = rx == kRangeSlow || ry == kRangeSlow;
                if (kPass == 0) {
                    if (out) slow++;
                    else if (sparse_sample_hit(S, xg, yg, rx, ry)) sparse_count_hit(a, S, x, y);
                } else if (out) {
                    slow++;
                    sparse_slow_sample(a, xg, yg, x, y);
                }
            }
        }
    }
    return slow;
}

__device__ __noinline__ void sparse_samples(const PixelwiseArgs &a) {
    PwSparseShared &S = sparse_smem();
    if (!(a.rm > 0.0f)) return;  // a grain radius is at most rm: nothing can cover a sample
    const unsigned slow = sparse_sample_pass<0>(a, S);
    if (__syncthreads_or(slow != 0)) {
        if (slow) atomicAdd(&a.diag[0], (unsigned long long)slow);
        sparse_sample_pass<1>(a, S);
    }
}

// A disk test of the grain-major form passed: grain (window cell `cell`) covers the sample of offset
// entry e at pixel (rx, ry).  The sample counts when this block owns it, its cell ranges lie inside the
// window (else pass 1 decides it), the grain's cell lies in its ranges -- the cells the reference
// visits for it (src/pixelwise.rs:55-58) -- and no other grain covered it before.  The ranges come
// from the table, or beyond its slots are computed as the table's entries are.
__device__ __forceinline__ void sparse_gm_hit(const PixelwiseArgs &a, PwSparseShared &S, int e, unsigned cell, float rx,
                                              float ry) {
    using C = PwSparse;
    const int k = S.gm.k[e];
    const int x = (int)rx, y = (int)ry;
    const int4 R = S.rect[k];
    if (x < R.x || x >= R.y || y < R.z || y >= R.w) return;  // another block's sample
    const int sx = x - R.x, sy = y - R.z;
    unsigned cx, cy;
    if (sx < C::kRangeSlots) cx = S.range_x[sx * a.n + k];
    else cx = sparse_range_code(xg_of(x, a.inv_zoom, S.gm.ent[e].x), a.rm, a.delta, S.wi0, S.wi1);
    if (sy < C::kRangeSlots) cy = S.range_y[sy * a.n + k];
    else cy = sparse_range_code(xg_of(y, a.inv_zoom, S.gm.ent[e].y), a.rm, a.delta, S.wj0, S.wj1);
    if (cx == kRangeSlow || cy == kRangeSlow) return;
    if ((cell & 0xFFFFu) - (cx & 0x7FFu) > (cx >> 11) || (cell >> 16) - (cy & 0x7FFu) > (cy >> 11)) return;
    const int idx = S.gm.base[k] + sy * (R.y - R.x) + sx;
    const unsigned bit = 1u << (idx & 31);
    if (!(atomicOr(&S.gm.bits[idx >> 5], bit) & bit)) sparse_count_hit(a, S, x, y);
}

// Step 3, grain-major: each thread takes staged grains and finds the owned samples within their radius.
// Sample k of pixel x lies at xg = (x + 0.5) / zoom - o.x, so a grain at gx can cover only the pixel
// x = rint(gx * zoom - 0.5 + o.x * zoom) of each offset (its reach r * zoom is below half a pixel), and
// only offsets whose phase frac(o.x * zoom) lies within r * zoom + eps of frac(0.5 - gx * zoom) reach
// it: the offsets are binned by their two phases (kGmBins^2 bins), and a grain visits the bins its
// phase band covers.  Every candidate gets the reference's disk test on the reference's xg, yg
// (src/pixelwise.rs:96-99); the band only has to contain every pixel that can pass it.  A sample's
// covering grains are OR-ed through its bit, so the count equals the sample-major form's.
// The pixel coordinate of offset entry O that grain coordinate p = g * zoom - 0.5 can reach, as a float:
// p + o * zoom rounded to an integer by adding and removing 1.5 * 2^23.
__device__ __forceinline__ float gm_pixel(float p, float oz) {
    constexpr float kRint = 12582912.0f;
    return FG_FSUB(FG_FADD(FG_FADD(p, oz), kRint), kRint);
}

// A passed disk test is listed as grain | entry << 11 and decided after the pass, the list dealt across
// all lanes (the decision reads the rectangle, the ranges and the bit; in the pass a warp would run it
// for a few lanes at a time, and a lane deciding its own tests leaves the warp as slow as its busiest
// lane: both measured slower); once the list is full a test is decided on the spot.
__device__ __forceinline__ void gm_pass_test(const PixelwiseArgs &a, PwSparseShared &S, int t, int e) {
    using C = PwSparse;
    const float4 G = S.grains[t];
    const float4 O = S.gm.ent[e];
    const float px = FG_FSUB(FG_FMUL(G.x, a.zoom), 0.5f), py = FG_FSUB(FG_FMUL(G.y, a.zoom), 0.5f);
    const float rx = gm_pixel(px, O.z), ry = gm_pixel(py, O.w);
    // xg_of of pixel (rx, ry): rx + 0.5 is exact
    const float dx = FG_FSUB(FG_FSUB(FG_FMUL(FG_FADD(rx, 0.5f), a.inv_zoom), O.x), G.x);
    const float dy = FG_FSUB(FG_FSUB(FG_FMUL(FG_FADD(ry, 0.5f), a.inv_zoom), O.y), G.y);
    if (FG_FADD(FG_FMUL(dx, dx), FG_FMUL(dy, dy)) <= G.z) {
        const int slot = atomicAdd(&S.nhits, 1);
        if (slot < C::kGmHitMax) S.gm.hits[slot] = (unsigned)t | ((unsigned)e << 11);
        else sparse_gm_hit(a, S, e, __float_as_uint(G.w), rx, ry);
    }
}

// A warp takes 32 grains at a time, one per lane: each lane finds its grain's band of bins and counts
// the entries in them (3.5 on the large frame, 0 to 8 typically), the warp lists its (grain, entry)
// candidates in its queue at the lanes' prefix of the counts, and then tests the listed candidates 32
// at a time, every lane busy (a lane testing its own grain's candidates leaves the warp waiting for its
// busiest lane); a round with more candidates than the queue holds is tested lane by lane.
__device__ __noinline__ void sparse_grain_pass(const PixelwiseArgs &a, const PwSparseGrid &g) {
    PwSparseShared &S = sparse_smem();
    using C = PwSparse;
    constexpr int B = PwSparse::kGmBins;
    PwSparseGrainMajor &M = S.gm;
    const float z = a.zoom, zr = a.zoom * 1.0000039f;  // (1 + 2^-18): sqrt's rounding
    const int ng = S.ngrains, lane = threadIdx.x & 31;
    unsigned short *Q = M.pairs + (threadIdx.x >> 5) * C::kGmPairs;
    for (int t0 = threadIdx.x & ~31; t0 < ng; t0 += blockDim.x) {  // warp-uniform bounds (the shuffles)
        const int t = t0 + lane;
        int bx0 = 0, bx1 = -1, by0 = 0, by1 = -1;  // an empty band unless the grain can cover a sample
        if (t < ng) {
            const float4 G = S.grains[t];
            if (G.z >= 0.0f) {  // a radius <= 0 (r^2 = -1) covers nothing
                const float w = fmaf(sqrtf(G.z), zr, g.gm_eps);  // half-width of the phase band
                const float px = FG_FSUB(FG_FMUL(G.x, z), 0.5f), py = FG_FSUB(FG_FMUL(G.y, z), 0.5f);
                float lx = FG_FSUB(FG_FSUB(floorf(px), px), w), ly = FG_FSUB(FG_FSUB(floorf(py), py), w);
                lx = FG_FSUB(lx, floorf(lx));  // the band starts at phase lx in [0, 1) and spans 2w
                ly = FG_FSUB(ly, floorf(ly));
                bx0 = min((int)(lx * (float)B), B - 1);
                bx1 = (int)((lx + 2.0f * w) * (float)B);
                by0 = min((int)(ly * (float)B), B - 1);
                by1 = (int)((ly + 2.0f * w) * (float)B);
            }
        }
        // the band's entries: bins bx0..bx1 of bin rows by0..by1, bins past the last wrapping to the first
        auto for_each_range = [&](auto f) {
            for (int by = by0; by <= by1; by++) {
                const int row = (by & (B - 1)) * B;
                f(M.start[row + bx0], M.start[row + min(bx1, B - 1) + 1]);
                if (bx1 >= B) f(M.start[row], M.start[row + bx1 - B + 1]);
            }
        };
        int cnt = 0;
        for_each_range([&](int e0, int e1) { cnt += e1 - e0; });
        int incl = cnt;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        const int total = __shfl_sync(0xffffffffu, incl, 31);
        if (total <= C::kGmPairs) {
            int q = incl - cnt;
            for_each_range([&](int e0, int e1) {
                for (int e = e0; e < e1; e++) Q[q++] = (unsigned short)((lane << 8) | e);
            });
            __syncwarp();
            for (int i = lane; i < total; i += 32) {
                const unsigned pr = Q[i];
                gm_pass_test(a, S, t0 + (int)(pr >> 8), (int)(pr & 0xFFu));
            }
            __syncwarp();  // the queue is read before the next round writes it
        } else {
            for_each_range([&](int e0, int e1) {
                for (int e = e0; e < e1; e++) gm_pass_test(a, S, t, e);
            });
        }
    }
    __syncthreads();
    const int nh = min(S.nhits, C::kGmHitMax);
    for (int h = threadIdx.x; h < nh; h += blockDim.x) {
        const unsigned tok = M.hits[h];
        const int e = (int)(tok >> 11);
        const float4 G = S.grains[tok & 0x7FFu];
        const float4 O = M.ent[e];
        const float rx = gm_pixel(FG_FSUB(FG_FMUL(G.x, z), 0.5f), O.z);
        const float ry = gm_pixel(FG_FSUB(FG_FMUL(G.y, z), 0.5f), O.w);
        sparse_gm_hit(a, S, e, __float_as_uint(G.w), rx, ry);
    }
}

// Step 3 in the grain-major form: the owned samples' bit bases (a scan of the rectangles' areas), the
// phase-binned offsets, then the grains' pass.  Samples whose range leaves the window go to the
// per-sample loop as in the sample-major form: with every rectangle inside the range table the
// ownership pass saw them (any_slow); otherwise the plane's ranges span too few cells for any
// (gm_noslow).
__device__ __noinline__ void sparse_grain_major(const PixelwiseArgs &a, const PwSparseGrid &g) {
    PwSparseShared &S = sparse_smem();
    using C = PwSparse;
    const int tid = threadIdx.x, nthreads = blockDim.x;
    PwSparseGrainMajor &M = S.gm;
    int area = 0;
    if (tid < a.n) {  // n <= kPwKChunk = the CTA size
        const int4 R = S.rect[tid];
        if (R.y > R.x && R.w > R.z) area = (R.y - R.x) * (R.w - R.z);
    }
    int total;
    const int base = block_excl_scan(area, S.wsum, &total);
    if (tid < a.n) M.base[tid] = base;
    for (int e = tid; e < a.n; e += nthreads) {
        M.ent[e] = g.gm_ent[e];
        M.k[e] = (unsigned short)g.gm_idx[e];
    }
    for (int b = tid; b <= C::kGmBins * C::kGmBins; b += nthreads) M.start[b] = (unsigned short)g.gm_idx[a.n + b];
    for (int w = tid; w < (total + 31) >> 5; w += nthreads) M.bits[w] = 0u;
    if (tid == 0) S.nhits = 0;
    __syncthreads();
    if (!(a.rm > 0.0f)) return;  // a grain radius is at most rm: nothing can cover a sample
    sparse_grain_pass(a, g);
    if (S.any_slow) {  // uniform
        const unsigned slow = sparse_sample_pass<1>(a, S);
        if (slow) atomicAdd(&a.diag[0], (unsigned long long)slow);
    }
}

__device__ __noinline__ void sparse_slow_sample(const PixelwiseArgs &a, float xg, float yg, int x, int y) {
    PwSparseShared &S = sparse_smem();
    const int i0 = f2i_floor(FG_FDIV(FG_FSUB(xg, a.rm), a.delta));
    const int i1 = f2i_floor(FG_FDIV(FG_FADD(xg, a.rm), a.delta));
    const int j0 = f2i_floor(FG_FDIV(FG_FSUB(yg, a.rm), a.delta));
    const int j1 = f2i_floor(FG_FDIV(FG_FADD(yg, a.rm), a.delta));
    if (sparse_regen_sample(a, xg, yg, i0, i1, j0, j1)) sparse_count_hit(a, S, x, y);
}

// Step 2, out of line: the list of non-empty cells (column-major) with the rank before each mask
// word, then their grain counts, CSR prefix and grains.  Returns false (uniformly) when the list or
// the grains overflow their shared-memory buffers.
__device__ __noinline__ bool sparse_stage(const PixelwiseArgs &a) {
    PwSparseShared &S = sparse_smem();
    using C = PwSparse;
    const int tid = threadIdx.x, nthreads = blockDim.x, lane = tid & 31;
    const int Wc = S.Wc, Hc = S.Hc, hs = S.hs, wi0 = S.wi0, wj0 = S.wj0;
    if (tid == 0) S.ngrains = 0;  // read after the list's barrier
    const int nwords = Wc * hs;
    int nlist;
    {
        const int per = (nwords + nthreads - 1) / nthreads;
        const int b = tid * per, e = min(nwords, b + per);
        int local = 0;
        for (int w = b; w < e; w++) local += __popc(S.w.mask2[w].x);
        int total;
        int run = block_excl_scan(local, S.wsum, &total);
        nlist = total;
        if (total <= C::kListMax) {
            for (int w = b; w < e; w++) {
                S.w.wrank[w] = (unsigned short)run;
                unsigned m = S.w.mask2[w].x;
                const int col = w / hs, row0 = (w - col * hs) * 32;
                while (m) {
                    const int bit = __ffs(m) - 1;
                    m &= m - 1u;
                    S.w.list[run++] = (unsigned short)(col * Hc + row0 + bit);
                }
            }
        }
    }
    __syncthreads();
    if (nlist > C::kListMax) return false;
    // counts and grains in one pass: a warp takes 32 consecutive listed cells at a time, each lane counts
    // its cell's grains (the Poisson draws of src/pixelwise.rs:77-82), the lanes reserve their grains'
    // slots with a warp scan and one shared counter, and each lane regenerates its grains from the
    // stream the Poisson draws left (src/pixelwise.rs:84-95)
    const UniformF32 U = uniform_f32_new(0.0f, a.delta);
    for (int t0 = tid & ~31; t0 < nlist; t0 += nthreads) {  // warp-uniform bounds (the shuffles below)
        const int t = t0 + lane;
        int i = 0, j = 0;
        uint32_t q = 0u;
        Xoshiro rng;
        if (t < nlist) {
            const int c = S.w.list[t];
            i = wi0 + c / Hc;
            j = wj0 + c % Hc;
            q = sparse_cell_count(a, i, j, &rng);
        }
        const float cellw = __uint_as_float((unsigned)(i - wi0) | ((unsigned)(j - wj0) << 16));
        const int qc = (int)min(q, (uint32_t)C::kGrainMax + 1u);
        int incl = qc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += y;
        }
        int base = 0;
        if (lane == 31) base = atomicAdd(&S.ngrains, incl);  // lane 31 holds the warp's total
        base = __shfl_sync(0xffffffffu, base, 31);
        const int first = base + incl - qc;
        if (t < nlist) {
            S.w.gsc[t] = (unsigned)(first & 0xFFFF) | ((unsigned)min(qc, 0xFFFF) << 16);
            if (first + qc <= C::kGrainMax) {
                const float sx = FG_FMUL((float)i, a.delta), sy = FG_FMUL((float)j, a.delta);
                for (int k = 0; k < qc; k++) {
                    const float cx = FG_FADD(sx, uniform_f32_from(U, rng.next()));
                    const float cy = FG_FADD(sy, uniform_f32_from(U, rng.next()));
                    float r = radius_draw(a, rng);
                    if (r > a.rm) r = a.rm;
                    const float rr = (r <= 0.0f) ? -1.0f : FG_FMUL(r, r);  // -1 never passes the disk test
                    S.grains[first + k] = make_float4(cx, cy, rr, cellw);
                }
            }
        }
    }
    __syncthreads();
    return S.ngrains <= C::kGrainMax;  // an overflow wrote no grain past the buffer; the block is redone
}

// One block of edge bs at block coordinates (bx, by) (all threads of the CTA; the dynamic shared memory
// holds PwSparseShared): 0 rendered (or nothing to render), 1 left undone (its buffers would overflow:
// nothing written), 2 stopped by cancellation.
__device__ __noinline__ int pixelwise_sparse_block(const PixelwiseArgs &a, const PwSparseGrid &g, float bs, int bx,
                                                   int by) {
    using C = PwSparse;
    PwSparseShared &S = sparse_smem();
    const int tid = threadIdx.x, nthreads = blockDim.x, lane = tid & 31;
    // the cancellation word, read now and tested after the ownership pass (its latency overlaps it)
    int cancel_seen = 0;
    if (tid == 0 && a.cancel) cancel_seen = *(volatile int *)a.cancel;

    const float X0 = FG_FMUL((float)bx, bs), X1 = FG_FMUL((float)(bx + 1), bs);
    const float Y0 = FG_FMUL((float)by, bs), Y1 = FG_FMUL((float)(by + 1), bs);
    // Every owned sample has xg in [X0, X1) and computes its cell range with these same rounded,
    // monotone operations, so its range lies inside [wi0, wi1] x [wj0, wj1].
    const int wi0 = f2i_floor(FG_FDIV(FG_FSUB(X0, a.rm), a.delta));
    const int wi1 = f2i_floor(FG_FDIV(FG_FADD(X1, a.rm), a.delta));
    const int wj0 = f2i_floor(FG_FDIV(FG_FSUB(Y0, a.rm), a.delta));
    const int wj1 = f2i_floor(FG_FDIV(FG_FADD(Y1, a.rm), a.delta));
    const int Wc = wi1 - wi0 + 1, Hc = wj1 - wj0 + 1;
    const int hw = (Hc + 31) >> 5;  // mask words per window column
    const int hs = sparse_col_stride(hw);
    const bool fits = Wc > 0 && Hc > 0 && Hc <= C::kRowsMax && Wc * hs <= C::kMaskWords &&
                      wi0 >= g.gi0 && wi1 < g.gi0 + g.gw && wj0 >= g.gj0 && wj1 < g.gj0 + 32 * (g.ghw - 1);

    if (tid == 0) {
        S.wi0 = wi0; S.wi1 = wi1; S.wj0 = wj0; S.wj1 = wj1; S.Wc = Wc; S.Hc = Hc; S.hw = hw; S.hs = hs;
        S.est_grains = 0.0f;
        S.est_cells = 0.0f;
        S.fx0 = 0x7fffffff; S.fx1 = -1; S.fy0 = 0x7fffffff; S.fy1 = -1; S.nsamples = 0;
        S.rw_min = 0x7fffffff; S.rw_max = -1; S.rh_min = 0x7fffffff; S.rh_max = -1;
        S.any_slow = 0;
    }
    __syncthreads();
    // ---- expected grains and non-empty cells of the window: lambda integrated over its rectangle (a
    // cell takes the lambda of the pixel containing its origin; edge pixels extend outwards)
    if (fits) {
        const float wx0 = FG_FMUL((float)wi0, a.delta), wx1 = FG_FMUL((float)(wi1 + 1), a.delta);
        const float wy0 = FG_FMUL((float)wj0, a.delta), wy1 = FG_FMUL((float)(wj1 + 1), a.delta);
        const int px0 = (int)floorf(wx0), px1 = (int)floorf(wx1), py0 = (int)floorf(wy0), py1 = (int)floorf(wy1);
        const int nx = px1 - px0 + 1, npx = nx * (py1 - py0 + 1);
        float ge = 0.0f, ce = 0.0f;
        const float inv_cell = 1.0f / (a.delta * a.delta);
        for (int t = tid; t < npx; t += nthreads) {
            const int px = px0 + t % nx, py = py0 + t / nx;
            const float ox = fminf((float)(px + 1), wx1) - fmaxf((float)px, wx0);
            const float oy = fminf((float)(py + 1), wy1) - fmaxf((float)py, wy0);
            if (ox > 0.0f && oy > 0.0f) {
                const int cx = min(max(px, 0), a.in_w - 1), cy = min(max(py, 0), a.in_h - 1);
                const float lam = a.lam[(long long)cy * a.in_w + cx];
                ge += lam * ox * oy;
                ce += (1.0f - __expf(-lam * a.delta * a.delta)) * ox * oy * inv_cell;
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            ge += __shfl_xor_sync(0xffffffffu, ge, o);
            ce += __shfl_xor_sync(0xffffffffu, ce, o);
        }
        if (lane == 0 && (ge > 0.0f || ce > 0.0f)) {
            atomicAdd(&S.est_grains, ge);
            atomicAdd(&S.est_cells, ce);
        }
    }
    // ---- ownership: rectangles per offset, sample total, pixel footprint, rectangle size extremes
    // (N <= kPwKChunk)
    {
        int lx0 = 0x7fffffff, lx1 = -1, ly0 = 0x7fffffff, ly1 = -1, ns = 0;
        int wmin = 0x7fffffff, wmax = -1, hmin = 0x7fffffff, hmax = -1;
        bool slow = false;
        for (int k = tid; k < a.n; k += nthreads) {
            const float2 o = a.offs[k];
            const int xa = first_at_least(X0, a.out_w, a.inv_zoom, a.zoom, o.x);
            const int xe = first_at_least(X1, a.out_w, a.inv_zoom, a.zoom, o.x);
            const int ya = first_at_least(Y0, a.out_h, a.inv_zoom, a.zoom, o.y);
            const int ye = first_at_least(Y1, a.out_h, a.inv_zoom, a.zoom, o.y);
            S.rect[k] = make_int4(xa, xe, ya, ye);
            // the cell ranges of the rectangle's first columns and rows (pixelwise_sparse_block's table)
            for (int s2 = 0; s2 < min(xe - xa, C::kRangeSlots); s2++) {
                const unsigned c = sparse_range_code(xg_of(xa + s2, a.inv_zoom, o.x), a.rm, a.delta, wi0, wi1);
                S.range_x[s2 * a.n + k] = (unsigned short)c;
                slow |= c == kRangeSlow;
            }
            for (int s2 = 0; s2 < min(ye - ya, C::kRangeSlots); s2++) {
                const unsigned c = sparse_range_code(xg_of(ya + s2, a.inv_zoom, o.y), a.rm, a.delta, wj0, wj1);
                S.range_y[s2 * a.n + k] = (unsigned short)c;
                slow |= c == kRangeSlow;
            }
            wmin = min(wmin, xe - xa); wmax = max(wmax, xe - xa);
            hmin = min(hmin, ye - ya); hmax = max(hmax, ye - ya);
            if (xe > xa && ye > ya) {
                ns += (xe - xa) * (ye - ya);
                lx0 = min(lx0, xa); lx1 = max(lx1, xe);
                ly0 = min(ly0, ya); ly1 = max(ly1, ye);
            }
        }
        ns = __reduce_add_sync(0xffffffffu, ns);
        lx0 = __reduce_min_sync(0xffffffffu, lx0);
        lx1 = __reduce_max_sync(0xffffffffu, lx1);
        ly0 = __reduce_min_sync(0xffffffffu, ly0);
        ly1 = __reduce_max_sync(0xffffffffu, ly1);
        wmin = __reduce_min_sync(0xffffffffu, wmin);
        wmax = __reduce_max_sync(0xffffffffu, wmax);
        hmin = __reduce_min_sync(0xffffffffu, hmin);
        hmax = __reduce_max_sync(0xffffffffu, hmax);
        slow = __any_sync(0xffffffffu, slow);
        if (lane == 0) {
            if (slow) S.any_slow = 1;
            if (ns > 0) {
                atomicAdd(&S.nsamples, ns);
                atomicMin(&S.fx0, lx0); atomicMax(&S.fx1, lx1);
                atomicMin(&S.fy0, ly0); atomicMax(&S.fy1, ly1);
            }
            if (wmax >= 0) {  // the warp saw offsets
                atomicMin(&S.rw_min, wmin); atomicMax(&S.rw_max, wmax);
                atomicMin(&S.rh_min, hmin); atomicMax(&S.rh_max, hmax);
            }
        }
    }
    if (tid == 0) {
        S.stop = cancel_seen;
        if (cancel_seen) *(volatile int *)(a.cancel + 1) = 1;
    }
    __syncthreads();
    if (S.stop) return 2;
    if (S.nsamples == 0) return 0;
    if (!fits || S.est_grains > 0.75f * (float)C::kGrainMax || S.est_cells > 0.75f * (float)C::kListMax)
        return 1;
    const int fw = S.fx1 - S.fx0, fh = S.fy1 - S.fy0;
    const bool use_cnt = (long long)fw * fh <= kPwFootMax;
    if (use_cnt)
        for (int t = tid; t < fw * fh; t += nthreads) S.cnt[t] = 0u;

    // ---- 1. the window's bits from the plane's bitmask (word k of window column c: rows 32k .. 32k + 31)
    {
        const int rb = wj0 - g.gj0, rw = rb >> 5, rs = rb & 31;
        const unsigned tail = (Hc & 31) ? ((1u << (Hc & 31)) - 1u) : 0xffffffffu;
        for (int idx = tid; idx < Wc * hs; idx += nthreads) {
            const int k = idx / Wc, c = idx - k * Wc;  // consecutive threads: consecutive columns
            unsigned word = 0u;                        // the pad word of an even hw stays empty
            if (k < hw) {
                const int gc = wi0 - g.gi0 + c;
                const unsigned lo = g.cellmask[(long long)(rw + k) * g.gw + gc];
                const unsigned hi = rs ? g.cellmask[(long long)(rw + k + 1) * g.gw + gc] : 0u;
                word = __funnelshift_r(lo, hi, rs);
                if (k == hw - 1) word &= tail;
            }
            S.w.mask2[c * hs + k].x = word;
        }
        __syncthreads();
        for (int w = tid; w < Wc * hs; w += nthreads) {
            const int k = w % hs;
            S.w.mask2[w].y = k + 1 < hw ? S.w.mask2[w + 1].x : 0u;
        }
        __syncthreads();
    }

    // ---- 2. non-empty cells, their counts and grains
    if (!sparse_stage(a)) return 1;

    // ---- 3. the owned samples: grain-major when the plane allows it, the samples whose range leaves the
    // window are known (the plane has none, or every rectangle fits the range table), the samples fit the
    // bit array and the cost model favours it; else sample-major
    const bool gm = g.gm_ent && (g.gm_noslow || (S.rw_max <= C::kRangeSlots && S.rh_max <= C::kRangeSlots)) &&
                    S.nsamples <= 32 * C::kGmBitsWords &&
                    (float)S.ngrains * g.gm_grain_cost < (float)S.nsamples * g.gm_sample_cost;
    if (gm) sparse_grain_major(a, g);
    else sparse_samples(a);
    __syncthreads();

    // ---- 4. flush the per-pixel counts
    if (use_cnt) {
        for (int t = tid; t < fw * fh; t += nthreads) {
            const unsigned c = S.cnt[t];
            if (c) atomicAdd(&a.out[(long long)(S.fy0 + t / fw) * a.out_w + (S.fx0 + t % fw)], (float)c);
        }
    }
    if (tid == 0) {
        atomicAdd(&a.diag[3], 1ull);
        atomicAdd(&a.diag[gm ? 5 : 4], 1ull);
    }
    return 0;
}

// Sparse block (sbx, sby): whole, or -- when it overflows -- as its fat-grid blocks one after another;
// a fat-grid block that overflows too is appended to the deferred list for the fat pass (each fat-grid
// block is either rendered here or listed, never both).
__device__ __forceinline__ void pixelwise_sparse_root(const PixelwiseArgs &a, const PwSparseGrid &g, int sbx, int sby,
                                                      int nby, int *list) {
    const int st = pixelwise_sparse_block(a, g, g.bs, sbx, sby);
    if (st != 1) return;
    if (g.ratio == 1) {
        if (threadIdx.x == 0) sparse_defer(a, g, sbx, sby, nby, list);
        return;
    }
    for (int q = 0; q < g.ratio * g.ratio; q++) {
        const int bx = sbx * g.ratio + q % g.ratio, by = sby * g.ratio + q / g.ratio;
        if (bx < a.bx0 || bx >= a.bx0 + a.nbx || by < a.by0 || by >= a.by0 + nby) continue;
        __syncthreads();  // the previous block's shared state is no longer read
        const int sq = pixelwise_sparse_block(a, g, a.bsize, bx, by);
        if (sq == 2) return;
        if (sq == 1 && threadIdx.x == 0) list[1 + atomicAdd(list, 1)] = (by - a.by0) * a.nbx + (bx - a.bx0);
    }
}

}  // namespace fg
