//! The crate's integrators on the GB300 library: drop-in replacements for `render_pixelwise`
//! (src/pixelwise.rs:11-45) and `render_grainwise` (src/grainwise.rs:12-124) with the same arguments,
//! result and errors, for the `(Device::Gpu, Algo::*)` arms of `render_from_workspace_impl`
//! (src/lib.rs:151-165) when the `gb300` feature is on.  `Params` and `Derived` are converted field
//! by field and the offsets passed are the crate's own (`derived.offsets` / `derived.offsets_input`),
//! so the library draws the crate's RNG streams at the crate's sample positions.
//!
//! The cancel closure is polled every millisecond by a scoped thread while the library call runs and
//! mirrored into the flag the library reads; the library mirrors that flag into its running kernels,
//! which stop at their next work item, and the call returns `RenderError::Cancelled`.
use std::ffi::CStr;
use std::sync::atomic::{AtomicBool, AtomicI32, Ordering};
use std::time::Duration;

use crate::gb300 as ffi;
use crate::model::{Derived, Plane};
use crate::params::{Algo, ColorMode, MaxRadius, Params, RadiusDist};
use crate::{RenderError, RenderResult};

type CancelCheck<'a> = Option<&'a (dyn Fn() -> bool + Send + Sync)>;

/// `Params` -> `fg_params` (include/film_grain_gb300.h), the already-built values.
pub fn to_fg_params(p: &Params) -> ffi::FgParams {
    let (max_radius_kind, max_radius_value) = match p.max_radius {
        MaxRadius::Absolute(v) => (ffi::FG_MAXR_ABSOLUTE, v),
        MaxRadius::Quantile(q) => (ffi::FG_MAXR_QUANTILE, q),
    };
    let (has_roi, roi) = match p.roi {
        Some(r) => (1, (r.x0, r.y0, r.x1, r.y1)),
        None => (0, (0, 0, 0, 0)),
    };
    let (size_w, size_h) = match p.size {
        Some((w, h)) => (w, h.unwrap_or(0)),
        None => (0, 0),
    };
    ffi::FgParams {
        radius_dist: match p.radius_dist {
            RadiusDist::Const => ffi::FG_RADIUS_CONST,
            RadiusDist::Lognorm => ffi::FG_RADIUS_LOGNORM,
        },
        radius_mean: p.radius_mean,
        radius_stddev: p.radius_stddev,
        radius_log_mu: p.radius_log_mu.unwrap_or(0.0),
        radius_log_sigma: p.radius_log_sigma.unwrap_or(0.0),
        has_log_params: (p.radius_log_mu.is_some() && p.radius_log_sigma.is_some()) as i32,
        zoom: p.zoom,
        sigma_px: p.sigma_px,
        n_samples: p.n_samples,
        algo: match p.algo {
            Algo::Auto => ffi::FG_ALGO_AUTO,
            Algo::Grain => ffi::FG_ALGO_GRAIN,
            Algo::Pixel => ffi::FG_ALGO_PIXEL,
        },
        max_radius_kind,
        max_radius_value,
        cell_delta: p.cell_delta.unwrap_or(0.0),
        color_mode: match p.color_mode {
            ColorMode::Luma => ffi::FG_COLOR_LUMA,
            ColorMode::Rgb => ffi::FG_COLOR_RGB,
        },
        has_roi,
        roi_x0: roi.0,
        roi_y0: roi.1,
        roi_x1: roi.2,
        roi_y1: roi.3,
        size_w,
        size_h,
        seed: p.seed,
    }
}

/// `Derived` -> `fg_derived` (the offsets travel separately).
pub fn to_fg_derived(d: &Derived) -> ffi::FgDerived {
    ffi::FgDerived {
        input_width: d.input_width as i64,
        input_height: d.input_height as i64,
        output_width: d.output_width as i64,
        output_height: d.output_height as i64,
        inv_e_pi_r2: d.inv_e_pi_r2,
        rm: d.rm,
        delta: d.delta,
        n_offsets: d.offsets.len() as u32,
    }
}

fn last_error() -> String {
    unsafe {
        let m = ffi::fg_last_error_message();
        if m.is_null() { String::new() } else { CStr::from_ptr(m).to_string_lossy().into_owned() }
    }
}

/// fg_status -> RenderError (src/lib.rs:28-44).
fn check(rc: i32) -> RenderResult<()> {
    match rc {
        ffi::FG_OK => Ok(()),
        ffi::FG_ERR_CANCELLED => Err(RenderError::Cancelled),
        ffi::FG_ERR_CUDA | ffi::FG_ERR_NOMEM | ffi::FG_ERR_INTERNAL => Err(RenderError::Gpu(last_error())),
        _ => Err(RenderError::Message(last_error())),
    }
}

/// Runs `call` with the flag the library polls, set by a watcher thread once `cancel` returns true.
fn with_cancel<T>(cancel: CancelCheck<'_>, call: impl FnOnce(*const i32) -> T) -> T {
    let Some(cancel) = cancel else { return call(std::ptr::null()) };
    let flag = AtomicI32::new(cancel() as i32);
    let done = AtomicBool::new(false);
    std::thread::scope(|s| {
        s.spawn(|| {
            while !done.load(Ordering::Acquire) {
                if cancel() {
                    flag.store(1, Ordering::Release);
                    return;
                }
                std::thread::sleep(Duration::from_millis(1));
            }
        });
        let r = call(flag.as_ptr() as *const i32);
        done.store(true, Ordering::Release);
        r
    })
}

fn flat(offsets: &[[f32; 2]]) -> Vec<f32> {
    offsets.iter().flat_map(|o| [o[0], o[1]]).collect()
}

/// render_pixelwise (src/pixelwise.rs:11-45) on the GPU: the same output plane, bit for bit.
pub fn render_pixelwise_gb300(lambda: &Plane, params: &Params, derived: &Derived, cancel: CancelCheck<'_>)
    -> RenderResult<Plane> {
    let (p, d) = (to_fg_params(params), to_fg_derived(derived));
    let offs = flat(&derived.offsets_input);
    let mut out = vec![0.0f32; derived.output_width * derived.output_height];
    let rc = with_cancel(cancel, |flag| unsafe {
        ffi::fg_render_pixelwise(lambda.data.as_ptr(), &p, &d, offs.as_ptr(), out.as_mut_ptr(), flag,
                                 std::ptr::null_mut())
    });
    check(rc)?;
    Ok(Plane::from_vec(derived.output_width, derived.output_height, out))
}

/// render_grainwise (src/grainwise.rs:12-124) on the GPU: the same output plane, bit for bit.
pub fn render_grainwise_gb300(lambda: &Plane, params: &Params, derived: &Derived, cancel: CancelCheck<'_>)
    -> RenderResult<Plane> {
    let (p, d) = (to_fg_params(params), to_fg_derived(derived));
    let offs = flat(&derived.offsets);
    let mut out = vec![0.0f32; derived.output_width * derived.output_height];
    let rc = with_cancel(cancel, |flag| unsafe {
        ffi::fg_render_grainwise(lambda.data.as_ptr(), &p, &d, offs.as_ptr(), out.as_mut_ptr(), flag,
                                 std::ptr::null_mut())
    });
    check(rc)?;
    Ok(Plane::from_vec(derived.output_width, derived.output_height, out))
}
