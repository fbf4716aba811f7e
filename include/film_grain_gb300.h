/*
 * film_grain_gb300.h -- C-ABI of the GB300 (sm_103a) film-grain integrators.
 *
 * A drop-in for the CPU hot path of joseph-wardle/film_grain (Rust crate film_grain 0.1.1): the
 * pixel-wise and grain-wise Monte Carlo integrators, the deterministic RNG streams they consume,
 * and the host arithmetic the crate's render entry points run around them.  Coverage counts are
 * bit-identical to the crate's CPU path on the same inputs and seed.
 *
 * Conventions
 *   - Plain C types only: no CUDA or torch types cross this boundary.  `stream` is a cudaStream_t
 *     passed as void* (NULL = the legacy default stream).
 *   - Planes are row-major f32, width x height, no padding.  Offsets are [n][2] f32 (x, y).
 *   - Pointers may be host or device memory; the library detects which.  Every render call is
 *     synchronous on return when any of its buffers is host memory; the *_async variants take
 *     device pointers only and return after enqueueing on `stream`.
 *   - Every call returns an fg_status; fg_last_error_message() gives the thread's last message.
 *   - `cancel` (may be NULL) is polled before and between kernel launches; a non-zero value makes
 *     the call return FG_ERR_CANCELLED (the crate's RenderError::Cancelled, src/lib.rs:41).
 *   - Thread safety: calls on different streams may run concurrently; the library keeps no state
 *     but a per-device cache of launch limits and the thread-local error message.
 */
#ifndef FILM_GRAIN_GB300_H
#define FILM_GRAIN_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define FG_API __attribute__((visibility("default")))
#else
#define FG_API
#endif

/* RenderError (src/lib.rs:28-44) mapped to status codes. */
typedef enum fg_status {
    FG_OK = 0,
    FG_ERR_PARAMS = 1,      /* RenderError::Params(ParamsError) */
    FG_ERR_CANCELLED = 2,   /* RenderError::Cancelled */
    FG_ERR_CUDA = 3,        /* RenderError::Gpu(String) */
    FG_ERR_INVALID = 4,     /* RenderError::Message: bad sizes, null pointers, empty input */
    FG_ERR_UNSUPPORTED = 5, /* RenderError::Unsupported */
    FG_ERR_NOMEM = 6,       /* device allocation failed */
    FG_ERR_INTERNAL = 7     /* a kernel reported an inconsistent state (never expected) */
} fg_status;

/* Enums of src/params.rs:6-28. */
typedef enum fg_radius_dist { FG_RADIUS_CONST = 0, FG_RADIUS_LOGNORM = 1 } fg_radius_dist;
typedef enum fg_algo { FG_ALGO_AUTO = 0, FG_ALGO_GRAIN = 1, FG_ALGO_PIXEL = 2 } fg_algo;
typedef enum fg_color_mode { FG_COLOR_LUMA = 0, FG_COLOR_RGB = 1 } fg_color_mode;
typedef enum fg_max_radius_kind { FG_MAXR_ABSOLUTE = 0, FG_MAXR_QUANTILE = 1 } fg_max_radius_kind;

/* ParamsBuilder (src/params.rs:70-91) without the path / output-format / CLI-only fields. */
typedef struct fg_params_builder {
    int32_t radius_dist;      /* fg_radius_dist */
    float radius_mean;        /* mu_r, input pixels */
    float radius_stddev;      /* sigma_r, input pixels (lognorm only) */
    float zoom;               /* output scale s */
    float sigma_px;           /* Gaussian filter sigma, output pixels */
    uint32_t n_samples;       /* N (0 is raised to 1, as ParamsBuilder::build does) */
    int32_t algo;             /* fg_algo */
    int32_t max_radius_kind;  /* fg_max_radius_kind */
    float max_radius_value;   /* absolute radius or quantile p in (0,1) */
    float cell_delta;         /* <= 0 or NaN: None -> default_cell_delta(radius_mean) */
    int32_t color_mode;       /* fg_color_mode */
    int32_t has_roi;          /* crop [roi_x0, roi_x1) x [roi_y0, roi_y1) of the input (before zoom) */
    uint32_t roi_x0, roi_y0, roi_x1, roi_y1;
    uint32_t size_w, size_h;  /* forced output size; size_w == 0: none; size_h == 0: keep aspect */
    uint64_t seed;
} fg_params_builder;

/* Params (src/params.rs:45-68), resolved by ParamsBuilder::build. */
typedef struct fg_params {
    int32_t radius_dist;
    float radius_mean;
    float radius_stddev;      /* 0 for Const (derive_radius_parameters) */
    float radius_log_mu;      /* valid when has_log_params */
    float radius_log_sigma;
    int32_t has_log_params;
    float zoom;
    float sigma_px;
    uint32_t n_samples;
    int32_t algo;
    int32_t max_radius_kind;
    float max_radius_value;
    float cell_delta;         /* always resolved (Some) after build */
    int32_t color_mode;
    int32_t has_roi;
    uint32_t roi_x0, roi_y0, roi_x1, roi_y1;
    uint32_t size_w, size_h;
    uint64_t seed;
} fg_params;

/* Derived (src/model.rs:167-179) minus its Vecs: offsets live in caller-owned [n][2] buffers. */
typedef struct fg_derived {
    int64_t input_width, input_height;
    int64_t output_width, output_height;
    float inv_e_pi_r2;
    float rm;
    float delta;
    uint32_t n_offsets;
} fg_derived;

/* RenderStats (src/lib.rs:46-55). */
typedef struct fg_render_stats {
    int32_t algorithm;        /* FG_ALGO_GRAIN or FG_ALGO_PIXEL */
    int64_t input_width, input_height, output_width, output_height;
    uint32_t n_samples;
    float sigma_ratio;
    float rm_ratio;
} fg_render_stats;

/* ---------------------------------------------------------------------------------------------
 * Host-side parameter resolution (no GPU needed).
 * ------------------------------------------------------------------------------------------- */

/* ParamsBuilder::build (src/params.rs:141-179): validation plus the lognormal mu/sigma
 * derivation (src/params.rs:223-253).  FG_ERR_PARAMS with the field named in the message. */
FG_API fg_status fg_params_build(const fg_params_builder *builder, fg_params *out);

/* derive_common (src/model.rs:181-226): sizes, inv_e_pi_r2, rm, delta and make_offsets
 * (src/rng.rs:9-24).  offsets / offsets_input receive [n_samples][2] f32 (host memory, may be NULL). */
FG_API fg_status fg_derive(const fg_params *params, int64_t input_width, int64_t input_height,
                           fg_derived *out, float *offsets, float *offsets_input);

/* choose_algorithm (src/choose.rs:4-26): FG_ALGO_PIXEL or FG_ALGO_GRAIN. */
FG_API int32_t fg_choose_algorithm(const fg_params *params, const fg_derived *derived);

/* default_cell_delta (src/params.rs:255-261). */
FG_API float fg_default_cell_delta(float radius_mean);

/* normalize_plane (src/model.rs:228-250); returns the plane maximum.  src and dst are both host
 * memory (a pass over the host cores) or both device memory (a synchronous pass on the GPU, same bits;
 * NaN is returned, with the message set, if it fails). */
FG_API float fg_normalize_plane(const float *src, int64_t n, float *dst);

/* lambda_plane (src/model.rs:252-265).  Host or device buffers as for fg_normalize_plane.  The crate
 * takes the logarithm with f32::ln, the platform logf; the device pass reproduces this process's logf
 * bit for bit (a table of the inputs where it differs from the correctly rounded logarithm, built once
 * per process from logf itself). */
FG_API void fg_lambda_plane(const float *normalized, int64_t n, float inv_e_pi_r2, float *dst);

/* lambda_plane(normalize_plane(src)) in one pass (the same per-element operations, so the same bits),
 * without the normalised plane in memory; returns the plane maximum as fg_normalize_plane does.  The
 * crate runs the two steps in turn (src/lib.rs:140-166 via src/model.rs:228-265).  Host or device
 * buffers as for fg_normalize_plane. */
FG_API float fg_lambda_from_plane(const float *src, int64_t n, float inv_e_pi_r2, float *dst);

/* ---------------------------------------------------------------------------------------------
 * The integrators.
 * ------------------------------------------------------------------------------------------- */

/* render_pixelwise (src/pixelwise.rs:11-45): per output pixel, the fraction of the N offset
 * samples (offsets_input, input-pixel units) covered by a grain of the cell-seeded Boolean model.
 * lambda: input_width x input_height; out: output_width x output_height. */
FG_API fg_status fg_render_pixelwise(const float *lambda, const fg_params *params, const fg_derived *derived,
                                     const float *offsets_input, float *out, const volatile int32_t *cancel,
                                     void *stream);

/* render_grainwise (src/grainwise.rs:12-124): per output pixel, popcount of the N-bit sample mask
 * that the pixel-seeded grains' offset disks (offsets, output-pixel units) set, times 1/N. */
FG_API fg_status fg_render_grainwise(const float *lambda, const fg_params *params, const fg_derived *derived,
                                     const float *offsets, float *out, const volatile int32_t *cancel,
                                     void *stream);

/* Device-pointer variants: enqueue on `stream` and return (no host synchronisation). */
FG_API fg_status fg_render_pixelwise_async(const float *d_lambda, const fg_params *params,
                                           const fg_derived *derived, const float *d_offsets_input,
                                           float *d_out, void *stream);
FG_API fg_status fg_render_grainwise_async(const float *d_lambda, const fg_params *params,
                                           const fg_derived *derived, const float *d_offsets, float *d_out,
                                           void *stream);

/* Pixel-wise render that allocates no device memory.  No counterpart in the crate: it exists for
 * callers that may not allocate GPU memory themselves (a host that budgets all device memory and
 * only lends a plug-in its own buffers, or a real-time preview loop that cannot afford cudaMalloc /
 * cudaFree between frames).  d_lambda and d_out are device memory owned by the caller; offsets_input
 * is host memory.  The kernel's scratch is one fixed-size array compiled into this library (present
 * on every GPU that loads it, until process exit), so the call is limited to input planes of at
 * most FG_NOALLOC_MAX_INPUT_PIXELS pixels and N <= FG_NOALLOC_MAX_SAMPLES (FG_ERR_UNSUPPORTED
 * beyond).  The first call on each device, and the first after that device's CUDA context has been
 * destroyed and recreated (cudaDeviceReset), looks up the array's device address; make that call
 * before any stream capture begins.  Every call, the first included, enqueues on `stream` a
 * host-to-device copy of offsets_input (read from the caller's host memory), a clear of the
 * counters and the render kernels.  Every call on a device shares the array, which keeps the last
 * call's contents, so calls whose work overlaps on the GPU (concurrent streams, or host threads)
 * race; serialise them. */
#define FG_NOALLOC_MAX_INPUT_PIXELS (512u * 512u)
#define FG_NOALLOC_MAX_SAMPLES 4096u
FG_API fg_status fg_render_pixelwise_noalloc(const float *d_lambda, const fg_params *params,
                                             const fg_derived *derived, const float *offsets_input, float *d_out,
                                             void *stream);

/* ---------------------------------------------------------------------------------------------
 * Whole-image orchestration (render_with_input_image, src/lib.rs:78-84 / 134-173).
 * ------------------------------------------------------------------------------------------- */

/* rgb: interleaved f32 RGB, height x width x 3 (what image::to_rgb32f yields; host memory); the
 * params' ROI, when set, is cropped first (apply_roi, src/color.rs:215-231).
 * out_rgb8: output_height x output_width x 3 u8 (host memory), sized from fg_dry_run or fg_derive.
 * Luma mode renders Y only and recombines it with nearest-resized Cb/Cr; RGB mode renders the three
 * planes with the same seed.  Only the cropped RGB goes to the GPU: the colour split, normalize_plane,
 * lambda_plane, the integrators, the colour recombination and the u8 packing all run there. */
FG_API fg_status fg_render_image(const float *rgb, int64_t width, int64_t height, const fg_params *params,
                                 uint8_t *out_rgb8, fg_render_stats *stats, const volatile int32_t *cancel,
                                 void *stream);

/* dry_run_with_input_image (src/lib.rs:100-104): derive + choose only. */
FG_API fg_status fg_dry_run(int64_t width, int64_t height, const fg_params *params, fg_render_stats *stats);

/* ---------------------------------------------------------------------------------------------
 * Batches: many images of uneven sizes and parameters in one persistent launch behind a CUDA graph.
 * No counterpart in the crate (which renders one image per call); results equal the per-image
 * fg_render_pixelwise / fg_render_grainwise outputs bit for bit.
 * ------------------------------------------------------------------------------------------- */

typedef struct fg_batch_image {
    int32_t algo;                  /* FG_ALGO_PIXEL or FG_ALGO_GRAIN (resolved, e.g. by fg_choose_algorithm) */
    const fg_params *params;       /* read at fg_batch_create */
    const fg_derived *derived;     /* read at fg_batch_create */
    const float *offsets;          /* host [n][2]: offsets_input for pixel-wise, offsets for grain-wise */
    const float *d_lambda;         /* device, input_width x input_height (read at every run) */
    float *d_out;                  /* device, output_width x output_height (written at every run) */
    const float *h_lambda;         /* optional host copy of lambda, used only to estimate tile costs */
} fg_batch_image;

typedef struct fg_batch_tuning {
    int32_t grain_mask_words;      /* shared-memory mask words per grain-wise tile (sets the tile edge) */
    int32_t pixel_max_block_log2;  /* largest pixel-wise block edge, log2 of input pixels */
    int32_t ctas_per_sm;           /* persistent CTAs per SM */
} fg_batch_tuning;

typedef struct fg_batch fg_batch;

/* Plans the images, allocates the batch's scratch, uploads the work list and captures the graph.
 * tuning may be NULL (defaults).  Synchronous. */
FG_API fg_status fg_batch_create(const fg_batch_image *images, int32_t n_images, const fg_batch_tuning *tuning,
                                 fg_batch **out);
/* Replays the graph on `stream` (asynchronous): every image's d_out is rendered from its d_lambda. */
FG_API fg_status fg_batch_run(fg_batch *batch, void *stream);
FG_API fg_status fg_batch_destroy(fg_batch *batch);
FG_API fg_status fg_batch_get_tuning(const fg_batch *batch, fg_batch_tuning *out);
/* Kernel launches one fg_batch_run makes (the kernel nodes of its graph).  No counterpart in the crate. */
FG_API fg_status fg_batch_kernel_count(const fg_batch *batch, int32_t *out);
/* Times candidate tunings on these images (creating and running a batch for each) and returns the
 * fastest, with its graph time in milliseconds when best_ms is not NULL.  Synchronous. */
FG_API fg_status fg_batch_autotune(const fg_batch_image *images, int32_t n_images, void *stream,
                                   fg_batch_tuning *best, float *best_ms);

/* ---------------------------------------------------------------------------------------------
 * Surrogate: a residual 3x3-conv network that predicts the rendered plane from the normalised
 * intensity u, a seeded N(0,1) noise field and the grain radius.  No counterpart in the crate: it
 * stands in for the MC integrators in interactive previews, while fg_render_* remain the method of
 * record.  Layout: activations NHWC bf16 (channel stride 16 or 32), weights [cout][9 taps][cin] bf16
 * with tap = 3*ky + kx, biases f32.  Every pointer is device memory; every call is asynchronous on
 * `stream`.  Network:
 *   x   = (u, noise, radius * radius_scale, 0 ...)          16 channels
 *   h0  = relu(conv_in(x) + b_in)                          w_in  [32][9][16]
 *   h_l = h_{l-1} + relu(conv_l(h_{l-1}) + b_l)            w_res [n_res][32][9][32]
 *   y   = u + conv_out(h_L)[channel 0] + b_out[0]          w_out [8][9][32] (rows 1..7 zero)
 * ------------------------------------------------------------------------------------------- */

enum {
    FG_SG_CONV_INPUT = 0,           /* 16 -> 32, out = relu(z + b) */
    FG_SG_CONV_RESIDUAL = 1,        /* 32 -> 32, out = res + relu(z + b); aux (if not NULL) = relu(z + b) */
    FG_SG_CONV_OUTPUT = 2,          /* 32 -> 8, out_f32 = res_f32 + z[0] + b[0] */
    FG_SG_CONV_DGRAD_RESIDUAL = 3,  /* 32 -> 32, out = res + z (no bias): data gradient of a residual conv */
    FG_SG_CONV_DGRAD_OUTPUT = 4     /* 16 -> 32, out = z (no bias): data gradient of the output conv */
};

typedef struct fg_sg_net {
    int32_t n_res;                 /* residual layers */
    float radius_scale;            /* radius input channel = radius * radius_scale */
    const void *w_in;              /* bf16 [32][9][16] */
    const float *b_in;             /* [32] */
    const void *w_res;             /* bf16 [n_res][32][9][32] */
    const float *b_res;            /* [n_res][32] */
    const void *w_out;             /* bf16 [8][9][32] */
    const float *b_out;            /* [8] */
} fg_sg_net;

/* One 3x3 conv over nb images of height x width (kind above; in_cstride = input channel stride, a
 * multiple of 8 and at least the kind's input channels; in and w 16-byte aligned). */
FG_API fg_status fg_sg_conv_forward(int32_t kind, const void *in, int32_t in_cstride, const void *w, const float *bias,
                                    const void *res, const float *res_f32, void *out, void *aux, float *out_f32,
                                    int32_t nb, int32_t height, int32_t width, void *stream);
/* Adds the weight and bias gradients of a forward conv of `kind` (INPUT, RESIDUAL or OUTPUT) into the
 * f32 buffers dw [cout][9][cin] and db [cout]: gout is the gradient at the conv output (before the
 * bias, channel stride g_cstride), x the conv input (channel stride x_cstride). */
FG_API fg_status fg_sg_conv_wgrad(int32_t kind, const void *gout, int32_t g_cstride, const void *x, int32_t x_cstride,
                                  float *dw, float *db, int32_t nb, int32_t height, int32_t width, void *stream);
/* g[i] = relu[i] > 0 ? dh[i] : 0 over n bf16 elements. */
FG_API fg_status fg_sg_mask_grad(const void *dh, const void *relu, void *g, int64_t n, void *stream);
/* wt[ci][8 - tap][co] = w[co][tap][ci] (zero in the padding), the weights of the data-gradient conv. */
FG_API fg_status fg_sg_flip_weights(const void *w, void *wt, int32_t cout, int32_t cin, int32_t cout_pad,
                                    int32_t cin_pad, void *stream);
/* One Adam step (bias-corrected with `step` >= 1) on f32 weights w with moments m, v and decoupled
 * weight decay w -= lr * decay[i] * w (decay may be NULL: none); also writes the bf16 copy w_bf16 when
 * it is not NULL, and the weight average ema = ema_decay * ema + (1 - ema_decay) * w when ema is not NULL. */
FG_API fg_status fg_sg_adam(float *w, float *m, float *v, const float *grad, const float *decay, void *w_bf16,
                            float *ema, float ema_decay, int64_t n, float lr, float beta1, float beta2, float eps,
                            int32_t step, void *stream);
/* Builds the 16-channel network input from u [nb][h][w] and one radius per image; the noise field is
 * a function of (seed, pixel index in the batch) only. */
FG_API fg_status fg_sg_make_input(const float *u, const float *radius, float radius_scale, uint64_t seed, void *x,
                                  int32_t nb, int32_t height, int32_t width, void *stream);
/* dy16[p] = (scale * (y[p] - target[p]), 0 x 15) in bf16, and *loss_sum += sum (y - target)^2. */
FG_API fg_status fg_sg_mse_grad(const float *y, const float *target, void *dy16, float *loss_sum, int64_t n,
                                float scale, void *stream);
/* Scratch needed by fg_sg_infer. */
FG_API size_t fg_sg_infer_workspace_bytes(int32_t nb, int32_t height, int32_t width);
/* The whole network forward: out [nb][h][w] f32 from u [nb][h][w] and radius [nb]. */
FG_API fg_status fg_sg_infer(const fg_sg_net *net, const float *u, const float *radius, uint64_t seed, float *out,
                             int32_t nb, int32_t height, int32_t width, void *workspace, size_t workspace_bytes,
                             void *stream);

/* ---------------------------------------------------------------------------------------------
 * Diagnostics.
 * ------------------------------------------------------------------------------------------- */

/* Last error message of the calling thread ("" if none). */
FG_API const char *fg_last_error_message(void);

/* Counters of the calling thread's last synchronous fg_render_pixelwise: [0] samples evaluated on the
 * per-sample regeneration path, [1] blocks without a staged cell window, [2] block subdivisions on
 * shared-memory overflow, [3] blocks processed.  No counterpart in the crate (diagnostics only). */
FG_API void fg_pixelwise_diagnostics(unsigned long long out[4]);
/* Blocks of the calling thread's last synchronous fg_render_pixelwise that the sparse block pass ran,
 * by the form of their sample step: [0] sample-major (each sample scans the cells of its range),
 * [1] grain-major (each staged grain tests the samples within its radius).  The two forms give
 * identical counts.  No counterpart in the crate (diagnostics only). */
FG_API void fg_pixelwise_sparse_forms(unsigned long long out[2]);
/* Kernel launches one pixel-wise render of these params makes: 3 when the plane takes the per-sample
 * kernel (cell table, per-sample kernel, epilogue), 6 when it takes the sparse block pass (cell table,
 * the plane's cell-emptiness bitmask, the offsets sorted by x and binned by phase, sparse and fat block
 * passes, epilogue), 4 when it takes the lean block pass (cell table, lean and fat block passes,
 * epilogue).  offsets_input as for fg_render_pixelwise.  No counterpart in the crate (diagnostics
 * only). */
FG_API fg_status fg_pixelwise_kernel_count(const fg_params *params, const fg_derived *derived,
                                           const float *offsets_input, int32_t *out);

/* Library version string. */
FG_API const char *fg_version(void);

#ifdef __cplusplus
} /* extern "C" */
#endif

#endif /* FILM_GRAIN_GB300_H */
