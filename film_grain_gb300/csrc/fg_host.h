// fg_host.h -- internal declarations of the host-side parameter resolution (fg_host.cpp).
#pragma once
#include <stdint.h>
#include <string>
#include <vector>
#include "../../include/film_grain_gb300.h"

namespace fg {

fg_status set_error(fg_status code, const std::string &msg);
void clear_error();
const char *last_error();

float default_cell_delta(float radius_mean);
fg_status params_build(const fg_params_builder &b, fg_params *out);
float radius_quantile(const fg_params &p, float prob);
void make_offsets(uint64_t seed, uint32_t n, float sigma, float *out);
fg_status derive(const fg_params &p, int64_t in_w, int64_t in_h, fg_derived *d, float *offsets, float *offsets_input);
int32_t choose_algorithm(const fg_params &p, const fg_derived &d);
float normalize_plane(const float *src, int64_t n, float *dst);
void lambda_plane(const float *norm, int64_t n, float inv_e_pi_r2, float *dst);
float lambda_from_plane(const float *src, int64_t n, float inv_e_pi_r2, float *dst);
void split_planes(const float *rgb, int64_t w, int64_t x0, int64_t y0, int64_t cw, int64_t ch, int luma, float *p0,
                  float *p1, float *p2);
void fill_stats(const fg_params &p, const fg_derived &d, int32_t algo, fg_render_stats *s);

// The platform logf (what the crate's f32::ln calls in lambda_plane) on every input lambda_plane can
// produce, as the inputs where it differs from RN_f32(log((double)x)): sorted keys (input bit
// patterns) with their logf bit patterns, bucketed by (bits - lo_bits) >> shift.  Built once per
// process from this process's own logf (16.8 million evaluations spread over the host cores).
struct LogfTable {
    uint32_t lo_bits, hi_bits;           // the domain [1e-6f, 1.0f] as f32 bit patterns
    int shift;
    std::vector<uint32_t> bucket_start;  // ((hi_bits - lo_bits) >> shift) + 2 entries
    std::vector<uint32_t> keys, vals;
};
const LogfTable &logf_table();

}  // namespace fg
