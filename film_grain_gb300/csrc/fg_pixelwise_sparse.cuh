// fg_pixelwise_sparse.cuh -- the sparse block pass of the pixel-wise coverage estimator
// (src/pixelwise.rs:11-106): the first pass over every block of a plane whose grains are sparse
// enough to stage a large window in shared memory.  Blocks that turn out denser are left to the fat
// block pass (pixelwise_block<PwFat>), as the fat-grid blocks they cover.
//
// A CTA owns a square block of input space [X0, X1) x [Y0, Y1) (edge a power of two, `ratio` fat-grid
// blocks per side) and evaluates every sample (pixel, offset) whose point xg = ((x + 0.5) * inv_zoom) -
// offsets_input[k] lands in it:
//   1. the emptiness of every cell of the window that the owned samples can reach becomes one bit of
//      a row-major bitmask: each lane owns one of 32 consecutive columns (its column stage of the cell
//      hash computed once per run of rows), and per row the warp's ballot is one mask word; a cell is
//      empty when its first uniform does not exceed its Knuth threshold (cell_count_h);
//   2. the set bits, ranked in row-major order, list the non-empty cells; their grain counts (the
//      Poisson draws of src/pixelwise.rs:77-82) are prefix-summed into a CSR over the list and their
//      grains (centre, radius^2) regenerated into shared memory;
//   3. each thread takes the owned pixels of one offset (or a share of them) and runs the reference's
//      per-sample test: for each cell row j0..j1 of the sample's range (src/pixelwise.rs:55-58), the
//      bits of columns i0..i1 are cut from the mask, and when any is set their grains -- contiguous in
//      the CSR, since cells of one row follow each other in the list -- get the disk test
//      dx*dx + dy*dy <= r*r (src/pixelwise.rs:96-99);
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
    static constexpr int kMaskWords = 1024;  // window bitmask (32768 cells)
    static constexpr int kRowsMax = 256;     // window rows
    static constexpr int kRowBand = 8;       // rows one warp hashes per work unit
};

struct PwSparseShared {
    float4 grains[PwSparse::kGrainMax];
    unsigned int mask[PwSparse::kMaskWords];
    unsigned short wrank[PwSparse::kMaskWords];  // non-empty cells before each mask word (row-major)
    unsigned short list[PwSparse::kListMax];     // non-empty cells: window index j * Wc + i, row-major
    unsigned short gstart[PwSparse::kListMax + 1];
    int4 rect[kPwKChunk];                       // owned pixel rectangle per offset: xa, xe, ya, ye
    unsigned int cnt[kPwFootMax];
    int wsum[40];
    int fx0, fx1, fy0, fy1, nsamples;
    int stop;
    float est_grains, est_cells;
};

// Geometry of the sparse pass: block edge `bs` (input pixels) = ratio x the fat grid's edge, block grid
// origin and width; the fat grid is (a.bx0, a.by0, a.nbx) with a.bsize.
struct PwSparseGrid {
    float bs;
    int ratio;
    int sbx0, sby0, nsbx, nsby;
};

// The reference's per-sample loop for a sample the staged window cannot serve (out of line: rare).
__device__ __noinline__ bool sparse_regen_sample(const PixelwiseArgs &a, float xg, float yg, int i0, int i1, int j0,
                                                 int j1) {
    const UniformF32 U = uniform_f32_new(0.0f, a.delta);
    return eval_regen(a, U, xg, yg, i0, i1, j0, j1);
}

// One grain radius (out of line: the lognormal draw is long and runs once per staged grain).
__device__ __noinline__ float sparse_radius(const PixelwiseArgs &a, Xoshiro &rng) { return radius_draw(a, rng); }

// Grain count of cell (i, j) with the stream left after the Poisson draws (out of line: the rejection
// regime is long).
__device__ __noinline__ uint32_t sparse_cell_count(const PixelwiseArgs &a, int i, int j, Xoshiro *rng) {
    const CellParam cp = a.cells[cell_pixel(a, i, j)];
    Xoshiro r;
    const uint32_t q = cell_count(a.seed, i, j, cp, r);
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

// One sparse block (all threads of the CTA; `smem_raw` holds PwSparseShared).  Returns true when the
// block was left to the fat pass (nothing rendered).
__device__ __forceinline__ bool pixelwise_sparse_block(const PixelwiseArgs &a, const PwSparseGrid &g, int sbx,
                                                       int sby, unsigned char *smem_raw) {
    using C = PwSparse;
    PwSparseShared &S = *reinterpret_cast<PwSparseShared *>(smem_raw);
    const int tid = threadIdx.x, nthreads = blockDim.x, lane = tid & 31, warp = tid >> 5, nwarps = nthreads >> 5;
    // the cancellation word, read now and tested after the ownership pass (its latency overlaps it)
    int cancel_seen = 0;
    if (tid == 0 && a.cancel) cancel_seen = *(volatile int *)a.cancel;

    const float X0 = FG_FMUL((float)sbx, g.bs), X1 = FG_FMUL((float)(sbx + 1), g.bs);
    const float Y0 = FG_FMUL((float)sby, g.bs), Y1 = FG_FMUL((float)(sby + 1), g.bs);
    // Every owned sample has xg in [X0, X1) and computes its cell range with these same rounded,
    // monotone operations, so its range lies inside [wi0, wi1] x [wj0, wj1].
    const int wi0 = f2i_floor(FG_FDIV(FG_FSUB(X0, a.rm), a.delta));
    const int wi1 = f2i_floor(FG_FDIV(FG_FADD(X1, a.rm), a.delta));
    const int wj0 = f2i_floor(FG_FDIV(FG_FSUB(Y0, a.rm), a.delta));
    const int wj1 = f2i_floor(FG_FDIV(FG_FADD(Y1, a.rm), a.delta));
    const int Wc = wi1 - wi0 + 1, Hc = wj1 - wj0 + 1;
    const int wpr = (Wc + 31) >> 5;
    const bool fits = Wc > 0 && Hc > 0 && Hc <= C::kRowsMax && wpr * Hc <= C::kMaskWords;

    // ---- expected grains and non-empty cells of the window: lambda integrated over its rectangle (a
    // cell takes the lambda of the pixel containing its origin; edge pixels extend outwards)
    if (tid == 0) {
        S.est_grains = 0.0f;
        S.est_cells = 0.0f;
        S.fx0 = 0x7fffffff; S.fx1 = -1; S.fy0 = 0x7fffffff; S.fy1 = -1; S.nsamples = 0;
    }
    __syncthreads();
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
    // ---- ownership: rectangles per offset, sample total and pixel footprint (N <= kPwKChunk)
    {
        int lx0 = 0x7fffffff, lx1 = -1, ly0 = 0x7fffffff, ly1 = -1, ns = 0;
        for (int k = tid; k < a.n; k += nthreads) {
            const float2 o = a.offs[k];
            const int xa = first_at_least(X0, a.out_w, a.inv_zoom, a.zoom, o.x);
            const int xe = first_at_least(X1, a.out_w, a.inv_zoom, a.zoom, o.x);
            const int ya = first_at_least(Y0, a.out_h, a.inv_zoom, a.zoom, o.y);
            const int ye = first_at_least(Y1, a.out_h, a.inv_zoom, a.zoom, o.y);
            S.rect[k] = make_int4(xa, xe, ya, ye);
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
        if (lane == 0 && ns > 0) {
            atomicAdd(&S.nsamples, ns);
            atomicMin(&S.fx0, lx0); atomicMax(&S.fx1, lx1);
            atomicMin(&S.fy0, ly0); atomicMax(&S.fy1, ly1);
        }
    }
    if (tid == 0) {
        S.stop = cancel_seen;
        if (cancel_seen) *(volatile int *)(a.cancel + 1) = 1;
    }
    __syncthreads();
    if (S.nsamples == 0 || S.stop) return false;
    if (!fits || S.est_grains > 0.75f * (float)C::kGrainMax || S.est_cells > 0.75f * (float)C::kListMax)
        return true;  // the fat pass takes the block's fat-grid blocks
    const int fx0 = S.fx0, fy0 = S.fy0, fw = S.fx1 - S.fx0, fh = S.fy1 - S.fy0;
    const bool use_cnt = (long long)fw * fh <= kPwFootMax;
    if (use_cnt)
        for (int t = tid; t < fw * fh; t += nthreads) S.cnt[t] = 0u;

    // ---- 1. emptiness bitmask: unit u = (column group u % wpr, row band u / wpr), one per warp in turn
    {
        const int nbands = (Hc + C::kRowBand - 1) / C::kRowBand;
        for (int u = warp; u < wpr * nbands; u += nwarps) {
            const int cg = u % wpr, band = u / wpr;
            const int ci = cg * 32 + lane;
            const bool valid = ci < Wc;
            const int i = wi0 + (valid ? ci : Wc - 1);
            const uint64_t colh = cell_col_hash(a.seed, i);
            long long ix = (long long)floorf(FG_FMUL((float)i, a.delta));
            ix = ix < 0 ? 0 : (ix > a.in_w - 1 ? a.in_w - 1 : ix);
            int iy_prev = -1;
            long long thresh = 0;
            const int r0 = band * C::kRowBand, r1 = min(Hc, r0 + C::kRowBand);
            for (int r = r0; r < r1; r++) {
                const int j = wj0 + r;
                long long iy = (long long)floorf(FG_FMUL((float)j, a.delta));
                iy = iy < 0 ? 0 : (iy > a.in_h - 1 ? a.in_h - 1 : iy);
                if ((int)iy != iy_prev) {
                    iy_prev = (int)iy;
                    thresh = a.cells[iy * a.in_w + ix].thresh;
                }
                const long long v = (long long)(small_first_u64(cell_row_hash(colh, j)) >> 11);
                const unsigned word = __ballot_sync(0xffffffffu, valid && v > thresh);
                if (lane == 0) S.mask[r * wpr + cg] = word;
            }
        }
    }
    __syncthreads();

    // ---- 2. list of the non-empty cells (row-major), the rank before each mask word
    const int nwords = wpr * Hc;
    int nlist;
    {
        const int per = (nwords + nthreads - 1) / nthreads;
        const int b = tid * per, e = min(nwords, b + per);
        int local = 0;
        for (int w = b; w < e; w++) local += __popc(S.mask[w]);
        int total;
        int run = block_excl_scan(local, S.wsum, &total);
        nlist = total;
        if (total <= C::kListMax) {
            for (int w = b; w < e; w++) {
                S.wrank[w] = (unsigned short)run;
                unsigned m = S.mask[w];
                const int row = w / wpr, col0 = (w - row * wpr) * 32;
                while (m) {
                    const int bit = __ffs(m) - 1;
                    m &= m - 1u;
                    S.list[run++] = (unsigned short)(row * Wc + col0 + bit);
                }
            }
        }
    }
    __syncthreads();
    if (nlist > C::kListMax) return true;

    // ---- grain counts of the listed cells, their CSR prefix, then the grains
    for (int t = tid; t < nlist; t += nthreads) {
        const int c = S.list[t];
        Xoshiro rng;
        const uint32_t q = sparse_cell_count(a, wi0 + c % Wc, wj0 + c / Wc, &rng);
        S.gstart[t] = (unsigned short)(q > 65535u ? 65535u : q);
    }
    __syncthreads();
    int ngrains;
    {
        const int per = (nlist + nthreads - 1) / nthreads;
        const int b = tid * per, e = min(nlist, b + per);
        int local = 0;
        for (int t = b; t < e; t++) local += S.gstart[t];
        int total;
        int run = block_excl_scan(local, S.wsum, &total);
        ngrains = total;
        if (total <= C::kGrainMax) {
            for (int t = b; t < e; t++) {
                const int q = S.gstart[t];
                S.gstart[t] = (unsigned short)run;
                run += q;
            }
            if (tid == 0) S.gstart[nlist] = (unsigned short)total;
        }
    }
    __syncthreads();
    if (ngrains > C::kGrainMax) return true;
    {
        const UniformF32 U = uniform_f32_new(0.0f, a.delta);
        for (int t = tid; t < nlist; t += nthreads) {
            const int c = S.list[t];
            const int i = wi0 + c % Wc, j = wj0 + c / Wc;
            const CellParam cp = a.cells[cell_pixel(a, i, j)];
            const int base = S.gstart[t];
            uint32_t q = (uint32_t)(S.gstart[t + 1] - base);
            Xoshiro rng;
            if (cp.thresh >= 0) {
                // Knuth regime: the Poisson draw consumed exactly q + 1 uniforms; skip them.
                rng = small_seed(cell_row_hash(cell_col_hash(a.seed, i), j));
                for (uint32_t k = 0; k <= q; k++) (void)rng.next();
            } else {
                q = min(q, sparse_cell_count(a, i, j, &rng));
            }
            const float sx = FG_FMUL((float)i, a.delta), sy = FG_FMUL((float)j, a.delta);
            for (uint32_t k = 0; k < q; k++) {
                const float cx = FG_FADD(sx, uniform_f32_from(U, rng.next()));
                const float cy = FG_FADD(sy, uniform_f32_from(U, rng.next()));
                float r = a.lognorm ? sparse_radius(a, rng) : a.radius_mean;
                if (r > a.rm) r = a.rm;
                const float rr = (r <= 0.0f) ? -1.0f : FG_FMUL(r, r);  // -1 never passes the disk test
                S.grains[base + k] = make_float4(cx, cy, rr, 0.0f);
            }
        }
    }
    __syncthreads();

    // ---- 3. the owned samples: offset k's pixel rectangle, shared by `parts` threads by rows
    {
        const int parts = a.n >= nthreads ? 1 : nthreads / a.n;
        unsigned long long slow = 0;
        for (int t = tid; t < a.n * parts; t += nthreads) {
            const int k = t / parts, p = t % parts;
            const int4 R = S.rect[k];
            const float2 o = a.offs[k];
            for (int y = R.z + p; y < R.w; y += parts) {
                const float yg = xg_of(y, a.inv_zoom, o.y);
                const int j0 = f2i_floor(FG_FDIV(FG_FSUB(yg, a.rm), a.delta));
                const int j1 = f2i_floor(FG_FDIV(FG_FADD(yg, a.rm), a.delta));
                for (int x = R.x; x < R.y; x++) {
                    const float xg = xg_of(x, a.inv_zoom, o.x);
                    bool hit = false;
                    if (a.rm > 0.0f) {
                        const int i0 = f2i_floor(FG_FDIV(FG_FSUB(xg, a.rm), a.delta));
                        const int i1 = f2i_floor(FG_FDIV(FG_FADD(xg, a.rm), a.delta));
                        if (i0 <= i1 && j0 <= j1) {
                            if (i0 >= wi0 && i1 <= wi1 && j0 >= wj0 && j1 <= wj1 && i1 - i0 < 32) {
                                const int c0 = i0 - wi0, w0 = c0 >> 5, b0 = c0 & 31;
                                const unsigned span = (unsigned)(i1 - i0);
                                const unsigned keep = span == 31u ? 0xffffffffu : ((2u << span) - 1u);
                                for (int j = j0; j <= j1 && !hit; j++) {
                                    const int wbase = (j - wj0) * wpr + w0;
                                    const unsigned lo = S.mask[wbase];
                                    const unsigned hi = (w0 + 1 < wpr) ? S.mask[wbase + 1] : 0u;
                                    const unsigned bits = __funnelshift_r(lo, hi, b0) & keep;
                                    if (!bits) continue;
                                    const int rank = S.wrank[wbase] + __popc(lo & ((1u << b0) - 1u));
                                    const int gs = S.gstart[rank], ge = S.gstart[rank + __popc(bits)];
                                    for (int gi = gs; gi < ge; gi++) {
                                        const float4 G = S.grains[gi];
                                        const float dx = FG_FSUB(xg, G.x), dy = FG_FSUB(yg, G.y);
                                        if (FG_FADD(FG_FMUL(dx, dx), FG_FMUL(dy, dy)) <= G.z) {
                                            hit = true;
                                            break;
                                        }
                                    }
                                }
                            } else {
                                slow++;
                                hit = sparse_regen_sample(a, xg, yg, i0, i1, j0, j1);
                            }
                        }
                    }
                    if (hit) {
                        const bool in_foot = use_cnt && x >= fx0 && x - fx0 < fw && y >= fy0 && y - fy0 < fh;
                        if (in_foot) atomicAdd(&S.cnt[(y - fy0) * fw + (x - fx0)], 1u);
                        else atomicAdd(&a.out[(long long)y * a.out_w + x], 1.0f);
                    }
                }
            }
        }
        if (slow) atomicAdd(&a.diag[0], slow);
    }
    __syncthreads();

    // ---- 4. flush the per-pixel counts
    if (use_cnt) {
        for (int t = tid; t < fw * fh; t += nthreads) {
            const unsigned c = S.cnt[t];
            if (c) atomicAdd(&a.out[(long long)(fy0 + t / fw) * a.out_w + (fx0 + t % fw)], (float)c);
        }
    }
    if (tid == 0) atomicAdd(&a.diag[3], 1ull);
    return false;
}

}  // namespace fg
