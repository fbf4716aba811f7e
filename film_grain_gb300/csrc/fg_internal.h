// fg_internal.h -- planning and enqueue helpers shared by the C-ABI translation units.
#pragma once
#include <cuda_runtime.h>
#include "../../include/film_grain_gb300.h"
#include "fg_kernels.cuh"

namespace fg {

// Pixel-wise launch plan: block edge (input pixels, a power of two), block grid and offset extents.
struct PwPlan {
    float bsize;
    int bx0, by0, nbx, nby;
    float ext[4];  // offset x min, x max, y min, y max
};

fg_status cuda_error(cudaError_t e, const char *what);
fg_status check_render_args(const fg_params *p, const fg_derived *d);
bool is_device_ptr(const void *p);
void offset_extents(const float *offs, uint32_t n, float ext[4]);
PwPlan plan_pixelwise(const fg_params &p, const fg_derived &d, const float *h_offs_in, int max_block_log2);
PixelwiseArgs pixelwise_args(const fg_params &p, const fg_derived &d, const PwPlan &pl, const float *d_lam,
                             const CellParam *d_cells, const float *d_offs_in, float *d_out, unsigned long long *d_diag);
fg_status enqueue_pixelwise(const float *d_lam, const fg_params &p, const fg_derived &d, const float *h_offs_in,
                            const float *d_offs_in, float *d_out, CellParam *d_cells, unsigned long long *d_diag,
                            const EpilogueArgs *colour, cudaStream_t s, bool may_allocate = true,
                            int *d_cancel = nullptr);
// The grain-wise offset table: n entries (frac(offy), offx, offy, k) sorted by frac(offx), followed by
// the bucket index over frac(offx) (kGwBucketCount + 1 ints).
size_t grain_table_bytes(uint32_t n);
void grain_table(const float *h_offs, uint32_t n, void *blob);
GrainwiseArgs grainwise_args(const fg_params &p, const fg_derived &d, const float *h_offs, const float *d_lam,
                             const void *d_table, unsigned int *d_gmask, int mask_words);
bool grainwise_small_coords(const GrainwiseArgs &a);
size_t grainwise_mask_bytes(const fg_params &p, const fg_derived &d);
fg_status enqueue_grainwise(const GrainwiseArgs &a, cudaStream_t s);
fg_status enqueue_grainwise_epilogue(const GrainwiseArgs &a, float *d_out, int mode, unsigned char *d_rgb8,
                                     const float *d_cb, const float *d_cr, cudaStream_t s);

// Device prelude of the whole-image render (fg_lambda.cu): the colour split of the cropped interleaved
// RGB (n_in pixels) into d_planes (3 x n_in: Y, Cb, Cr or R, G, B), the plane maxima (d_max: 3 words)
// and lambda of the rendered planes (1 or 3) into d_lam.
fg_status enqueue_split_lambda(const float *d_rgb, long long n_in, int luma, float *d_planes, unsigned int *d_max,
                               float inv_e_pi_r2, float *d_lam, cudaStream_t s);
// normalize_plane (normalize), lambda_plane (lambda) or both on device memory; max_out receives the
// plane maximum when normalizing.
fg_status device_plane_pass(const float *src, int64_t n, int normalize, int lambda, float inv_e_pi_r2, float *dst,
                            float *max_out);
fg_status device_logf_table(LogfTableDev *out);

}  // namespace fg
