// fg_color.cuh -- the colour workspace's per-pixel output arithmetic (src/color.rs), fused into the
// integrators' epilogues.
#pragma once
#include "fg_rng.cuh"

namespace fg {

// src/color.rs:233-235 clamp01 and :237-239 to_u8
__device__ __forceinline__ float clamp01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }
__device__ __forceinline__ unsigned char to_u8(float v) {
    return (unsigned char)__float2int_rz(floorf(FG_FADD(FG_FMUL(clamp01(v), 255.0f), 0.5f)));
}
// Plane::resize_nearest source index (src/model.rs:87-95)
__device__ __forceinline__ int nearest_src(int x, float scale, int w) {
    float f = FG_FSUB(FG_FMUL(FG_FADD((float)x, 0.5f), scale), 0.5f);
    float hi = (float)(w - 1);
    f = f < 0.0f ? 0.0f : (f > hi ? hi : f);
    return (int)roundf(f);
}
// into_rgb_image luma arm (src/color.rs:75-96)
__device__ __forceinline__ void luma_rgb8(float yv, float cbv, float crv, unsigned char *o) {
    const float YR = 0.2126f, YG = 0.7152f, YB = 0.0722f, CBD = 1.8556f, CRD = 1.5748f;
    float r = clamp01(FG_FADD(yv, FG_FMUL(CRD, crv)));
    float b = clamp01(FG_FADD(yv, FG_FMUL(CBD, cbv)));
    float gu = FG_FDIV(FG_FSUB(FG_FSUB(yv, FG_FMUL(YR, r)), FG_FMUL(YB, b)), YG);
    float g = clamp01(gu);
    o[0] = to_u8(r); o[1] = to_u8(g); o[2] = to_u8(b);
}

}  // namespace fg
