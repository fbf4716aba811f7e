//! Raw FFI of the GB300 film-grain library: `#[repr(C)]` mirrors of every struct and `extern "C"`
//! declaration of every entry point in include/film_grain_gb300.h, in the header's order.  Kept in
//! step with the header by a test that parses both files (tests/test_rust_shim.py in the library's
//! repository).  Safe wrappers for the crate's integrator dispatch are in gb300_render.rs.
#![allow(non_camel_case_types, dead_code)]

use std::os::raw::{c_char, c_void};

pub const FG_OK: i32 = 0;
pub const FG_ERR_PARAMS: i32 = 1;
pub const FG_ERR_CANCELLED: i32 = 2;
pub const FG_ERR_CUDA: i32 = 3;
pub const FG_ERR_INVALID: i32 = 4;
pub const FG_ERR_UNSUPPORTED: i32 = 5;
pub const FG_ERR_NOMEM: i32 = 6;
pub const FG_ERR_INTERNAL: i32 = 7;

pub const FG_RADIUS_CONST: i32 = 0;
pub const FG_RADIUS_LOGNORM: i32 = 1;
pub const FG_ALGO_AUTO: i32 = 0;
pub const FG_ALGO_GRAIN: i32 = 1;
pub const FG_ALGO_PIXEL: i32 = 2;
pub const FG_COLOR_LUMA: i32 = 0;
pub const FG_COLOR_RGB: i32 = 1;
pub const FG_MAXR_ABSOLUTE: i32 = 0;
pub const FG_MAXR_QUANTILE: i32 = 1;

pub const FG_NOALLOC_MAX_INPUT_PIXELS: u32 = 512 * 512;
pub const FG_NOALLOC_MAX_SAMPLES: u32 = 4096;

pub const FG_SG_CONV_INPUT: i32 = 0;
pub const FG_SG_CONV_RESIDUAL: i32 = 1;
pub const FG_SG_CONV_OUTPUT: i32 = 2;
pub const FG_SG_CONV_DGRAD_RESIDUAL: i32 = 3;
pub const FG_SG_CONV_DGRAD_OUTPUT: i32 = 4;

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct FgParamsBuilder {
    pub radius_dist: i32,
    pub radius_mean: f32,
    pub radius_stddev: f32,
    pub zoom: f32,
    pub sigma_px: f32,
    pub n_samples: u32,
    pub algo: i32,
    pub max_radius_kind: i32,
    pub max_radius_value: f32,
    pub cell_delta: f32,
    pub color_mode: i32,
    pub has_roi: i32,
    pub roi_x0: u32,
    pub roi_y0: u32,
    pub roi_x1: u32,
    pub roi_y1: u32,
    pub size_w: u32,
    pub size_h: u32,
    pub seed: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct FgParams {
    pub radius_dist: i32,
    pub radius_mean: f32,
    pub radius_stddev: f32,
    pub radius_log_mu: f32,
    pub radius_log_sigma: f32,
    pub has_log_params: i32,
    pub zoom: f32,
    pub sigma_px: f32,
    pub n_samples: u32,
    pub algo: i32,
    pub max_radius_kind: i32,
    pub max_radius_value: f32,
    pub cell_delta: f32,
    pub color_mode: i32,
    pub has_roi: i32,
    pub roi_x0: u32,
    pub roi_y0: u32,
    pub roi_x1: u32,
    pub roi_y1: u32,
    pub size_w: u32,
    pub size_h: u32,
    pub seed: u64,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct FgDerived {
    pub input_width: i64,
    pub input_height: i64,
    pub output_width: i64,
    pub output_height: i64,
    pub inv_e_pi_r2: f32,
    pub rm: f32,
    pub delta: f32,
    pub n_offsets: u32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct FgRenderStats {
    pub algorithm: i32,
    pub input_width: i64,
    pub input_height: i64,
    pub output_width: i64,
    pub output_height: i64,
    pub n_samples: u32,
    pub sigma_ratio: f32,
    pub rm_ratio: f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct FgBatchImage {
    pub algo: i32,
    pub params: *const FgParams,
    pub derived: *const FgDerived,
    pub offsets: *const f32,
    pub d_lambda: *const f32,
    pub d_out: *mut f32,
    pub h_lambda: *const f32,
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct FgBatchTuning {
    pub grain_mask_words: i32,
    pub pixel_max_block_log2: i32,
    pub ctas_per_sm: i32,
}

/// Opaque batch handle (fg_batch).
pub enum FgBatch {}

#[repr(C)]
#[derive(Clone, Copy, Debug)]
pub struct FgSgNet {
    pub n_res: i32,
    pub radius_scale: f32,
    pub w_in: *const c_void,
    pub b_in: *const f32,
    pub w_res: *const c_void,
    pub b_res: *const f32,
    pub w_out: *const c_void,
    pub b_out: *const f32,
}

extern "C" {
    pub fn fg_params_build(builder: *const FgParamsBuilder, out: *mut FgParams) -> i32;
    pub fn fg_derive(params: *const FgParams, input_width: i64, input_height: i64, out: *mut FgDerived,
                     offsets: *mut f32, offsets_input: *mut f32) -> i32;
    pub fn fg_choose_algorithm(params: *const FgParams, derived: *const FgDerived) -> i32;
    pub fn fg_default_cell_delta(radius_mean: f32) -> f32;
    pub fn fg_normalize_plane(src: *const f32, n: i64, dst: *mut f32) -> f32;
    pub fn fg_lambda_plane(normalized: *const f32, n: i64, inv_e_pi_r2: f32, dst: *mut f32);
    pub fn fg_lambda_from_plane(src: *const f32, n: i64, inv_e_pi_r2: f32, dst: *mut f32) -> f32;

    pub fn fg_render_pixelwise(lambda: *const f32, params: *const FgParams, derived: *const FgDerived,
                               offsets_input: *const f32, out: *mut f32, cancel: *const i32,
                               stream: *mut c_void) -> i32;
    pub fn fg_render_grainwise(lambda: *const f32, params: *const FgParams, derived: *const FgDerived,
                               offsets: *const f32, out: *mut f32, cancel: *const i32,
                               stream: *mut c_void) -> i32;
    pub fn fg_render_pixelwise_async(d_lambda: *const f32, params: *const FgParams, derived: *const FgDerived,
                                     d_offsets_input: *const f32, d_out: *mut f32, stream: *mut c_void) -> i32;
    pub fn fg_render_grainwise_async(d_lambda: *const f32, params: *const FgParams, derived: *const FgDerived,
                                     d_offsets: *const f32, d_out: *mut f32, stream: *mut c_void) -> i32;
    pub fn fg_render_pixelwise_noalloc(d_lambda: *const f32, params: *const FgParams, derived: *const FgDerived,
                                       offsets_input: *const f32, d_out: *mut f32, stream: *mut c_void) -> i32;

    pub fn fg_render_image(rgb: *const f32, width: i64, height: i64, params: *const FgParams, out_rgb8: *mut u8,
                           stats: *mut FgRenderStats, cancel: *const i32, stream: *mut c_void) -> i32;
    pub fn fg_dry_run(width: i64, height: i64, params: *const FgParams, stats: *mut FgRenderStats) -> i32;

    pub fn fg_batch_create(images: *const FgBatchImage, n_images: i32, tuning: *const FgBatchTuning,
                           out: *mut *mut FgBatch) -> i32;
    pub fn fg_batch_run(batch: *mut FgBatch, stream: *mut c_void) -> i32;
    pub fn fg_batch_destroy(batch: *mut FgBatch) -> i32;
    pub fn fg_batch_get_tuning(batch: *const FgBatch, out: *mut FgBatchTuning) -> i32;
    pub fn fg_batch_kernel_count(batch: *const FgBatch, out: *mut i32) -> i32;
    pub fn fg_batch_autotune(images: *const FgBatchImage, n_images: i32, stream: *mut c_void,
                             best: *mut FgBatchTuning, best_ms: *mut f32) -> i32;

    pub fn fg_sg_conv_forward(kind: i32, input: *const c_void, in_cstride: i32, w: *const c_void, bias: *const f32,
                              res: *const c_void, res_f32: *const f32, out: *mut c_void, aux: *mut c_void,
                              out_f32: *mut f32, nb: i32, height: i32, width: i32, stream: *mut c_void) -> i32;
    pub fn fg_sg_conv_wgrad(kind: i32, gout: *const c_void, g_cstride: i32, x: *const c_void, x_cstride: i32,
                            dw: *mut f32, db: *mut f32, nb: i32, height: i32, width: i32, stream: *mut c_void) -> i32;
    pub fn fg_sg_mask_grad(dh: *const c_void, relu: *const c_void, g: *mut c_void, n: i64, stream: *mut c_void) -> i32;
    pub fn fg_sg_flip_weights(w: *const c_void, wt: *mut c_void, cout: i32, cin: i32, cout_pad: i32, cin_pad: i32,
                              stream: *mut c_void) -> i32;
    pub fn fg_sg_adam(w: *mut f32, m: *mut f32, v: *mut f32, grad: *const f32, decay: *const f32, w_bf16: *mut c_void,
                      ema: *mut f32, ema_decay: f32, n: i64, lr: f32, beta1: f32, beta2: f32, eps: f32, step: i32,
                      stream: *mut c_void) -> i32;
    pub fn fg_sg_make_input(u: *const f32, radius: *const f32, radius_scale: f32, seed: u64, x: *mut c_void, nb: i32,
                            height: i32, width: i32, stream: *mut c_void) -> i32;
    pub fn fg_sg_mse_grad(y: *const f32, target: *const f32, dy16: *mut c_void, loss_sum: *mut f32, n: i64, scale: f32,
                          stream: *mut c_void) -> i32;
    pub fn fg_sg_infer_workspace_bytes(nb: i32, height: i32, width: i32) -> usize;
    pub fn fg_sg_infer(net: *const FgSgNet, u: *const f32, radius: *const f32, seed: u64, out: *mut f32, nb: i32,
                       height: i32, width: i32, workspace: *mut c_void, workspace_bytes: usize,
                       stream: *mut c_void) -> i32;

    pub fn fg_last_error_message() -> *const c_char;
    pub fn fg_pixelwise_diagnostics(out: *mut u64);
    pub fn fg_pixelwise_sparse_forms(out: *mut u64);
    pub fn fg_pixelwise_kernel_count(params: *const FgParams, derived: *const FgDerived, offsets_input: *const f32,
                                     out: *mut i32) -> i32;
    pub fn fg_version() -> *const c_char;
}
