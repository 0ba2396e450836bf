// hl_indirect.cuh — radiance-cascade indirect diffuse light of Helio's deferred pass
// for sm_103a: sample_rc_irradiance (deferred_lighting.wgsl:822-917) over the
// rc_cascade0 probe texture (Rgba16Float, 16^3 probes of 4x4 octahedral directions).
#pragma once

#include <cuda_fp16.h>

#include "hl_common.cuh"
#include "hl_internal.h"

namespace hl {
namespace rc {

constexpr uint32_t kProbeDim = HL_RC_PROBE_DIM;  // RC_PROBE_DIM, :824
constexpr uint32_t kDirDim = HL_RC_DIR_DIM;      // RC_DIR_DIM, :825

// rc_oct_decode (:827-840) of the centre of direction cell (ddx, ddy).
__device__ __forceinline__ void oct_dir(uint32_t ddx, uint32_t ddy, float& x, float& y, float& z) {
    const float fx = (float(ddx) + 0.5f) / float(kDirDim) * 2.0f - 1.0f;
    const float fy = (float(ddy) + 0.5f) / float(kDirDim) * 2.0f - 1.0f;
    const float ax = fabsf(fx), ay = fabsf(fy), l = ax + ay;
    if (l > 1.0f) {
        x = (1.0f - ay) * (fx >= 0.0f ? 1.0f : -1.0f);
        y = 1.0f - l;
        z = (1.0f - ax) * (fy >= 0.0f ? 1.0f : -1.0f);
    } else {
        x = fx;
        y = 1.0f - l;
        z = fy;
    }
    const float in = rsqrtf(x * x + y * y + z * z);
    x *= in;
    y *= in;
    z *= in;
}

__device__ __forceinline__ float smooth01(float lo, float hi, float x) {
    const float t = fminf(fmaxf((x - lo) / (hi - lo), 0.0f), 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// rc_corner_irradiance_precomp (:842-864): the cosine-weighted mean of one probe's
// directions (those with weight > 0.001). The 4 directions dx of one row dy are 32
// contiguous bytes, so a probe is read as 8 unconditional 16-byte loads and the skipped
// directions are masked after loading.
__device__ __forceinline__ void corner(const ExtView& ev, uint32_t px, uint32_t py, uint32_t pz, const float* cw,
                                       float& r, float& g, float& b) {
    const uint32_t cpx = min(px, kProbeDim - 1u), cpy = min(py, kProbeDim - 1u), cpz = min(pz, kProbeDim - 1u);
    const unsigned char* base = ev.rc + 8ull * (cpx * kDirDim) + ev.rc_pitch * ((cpy * kProbeDim + cpz) * kDirDim);
    uint4 t[kDirDim][2];
#pragma unroll
    for (uint32_t ddy = 0; ddy < kDirDim; ++ddy) {
        const uint4* row = reinterpret_cast<const uint4*>(base + ev.rc_pitch * ddy);
        t[ddy][0] = __ldg(row);
        t[ddy][1] = __ldg(row + 1);
    }
    float ir = 0.0f, ig = 0.0f, ib = 0.0f, ws = 0.0f;
#pragma unroll
    for (uint32_t ddx = 0; ddx < kDirDim; ++ddx) {
#pragma unroll
        for (uint32_t ddy = 0; ddy < kDirDim; ++ddy) {
            const float w = cw[ddx * kDirDim + ddy];
            const uint4 q = t[ddy][ddx >> 1];
            const uint32_t lo = (ddx & 1u) ? q.z : q.x, hi = (ddx & 1u) ? q.w : q.y;
            const float2 rg = __half22float2(*reinterpret_cast<const __half2*>(&lo));
            const float2 bb = __half22float2(*reinterpret_cast<const __half2*>(&hi));
            const bool use = w > 0.001f;
            ir += use ? rg.x * w : 0.0f;
            ig += use ? rg.y * w : 0.0f;
            ib += use ? bb.x * w : 0.0f;
            ws += use ? w : 0.0f;
        }
    }
    const float d = fmaxf(ws, 0.001f);
    r = ir / d;
    g = ig / d;
    b = ib / d;
}

__device__ __forceinline__ float mix_(float a, float b, float t) { return a * (1.0f - t) + b * t; }

// sample_rc_irradiance (:866-917) at world position w with unit normal n.
static __device__ __noinline__ void irradiance(const ExtView& ev, const DeferredGlobals* glb, float wx, float wy,
                                               float wz, float nx, float ny, float nz, float& r, float& g, float& b) {
    r = g = b = 0.0f;
    if (glb->has_rc_gi == 0u) return;
    const float mn[3] = {glb->rc_world_min[0], glb->rc_world_min[1], glb->rc_world_min[2]};
    const float size[3] = {glb->rc_world_max[0] - mn[0], glb->rc_world_max[1] - mn[1], glb->rc_world_max[2] - mn[2]};
    if (size[0] <= 0.0f || size[1] <= 0.0f || size[2] <= 0.0f) return;
    const float w[3] = {wx, wy, wz};
    float vw = 1.0f, pf[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        const float t = (w[k] - mn[k]) / size[k];
        vw *= smooth01(0.0f, 0.05f, t) * smooth01(1.0f, 1.0f - 0.05f, t);
        const float cell = size[k] / float(kProbeDim);
        pf[k] = fminf(fmaxf((w[k] - mn[k]) / cell - 0.5f, 0.0f), float(kProbeDim) - 1.0f);
    }
    if (vw <= 0.0f) return;
    float cw[kDirDim * kDirDim];
#pragma unroll
    for (uint32_t ddx = 0; ddx < kDirDim; ++ddx) {
#pragma unroll
        for (uint32_t ddy = 0; ddy < kDirDim; ++ddy) {
            float dx, dy, dz;
            oct_dir(ddx, ddy, dx, dy, dz);
            cw[ddx * kDirDim + ddy] = fmaxf(0.0f, nx * dx + ny * dy + nz * dz);
        }
    }
    const uint32_t ix = uint32_t(pf[0]), iy = uint32_t(pf[1]), iz = uint32_t(pf[2]);
    const float fx = pf[0] - floorf(pf[0]), fy = pf[1] - floorf(pf[1]), fz = pf[2] - floorf(pf[2]);
    float c[8][3];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        corner(ev, ix + uint32_t(k >> 2), iy + uint32_t((k >> 1) & 1), iz + uint32_t(k & 1), cw, c[k][0], c[k][1],
               c[k][2]);
    float out[3];
#pragma unroll
    for (int ch = 0; ch < 3; ++ch) {
        const float c0 = mix_(mix_(c[0][ch], c[1][ch], fz), mix_(c[2][ch], c[3][ch], fz), fy);
        const float c1 = mix_(mix_(c[4][ch], c[5][ch], fz), mix_(c[6][ch], c[7][ch], fz), fy);
        out[ch] = mix_(c0, c1, fx) * vw;
    }
    r = out[0];
    g = out[1];
    b = out[2];
}

// The ambient term of fs_main with radiance-cascade GI (:1159-1163, 1197-1209): the
// hemisphere ambient h (times albedo) blended with kD_ibl * rc_irradiance * albedo by
// w = clamp(4 |rc_irradiance|, 0, 1), kD_ibl = (1 - fresnel_schlick_roughness(NdV, F0,
// roughness)) (1 - metallic) (pbr_eval.wgsl:63-66). h is replaced in place.
static __device__ __noinline__ void ambient(const ExtView& ev, const DeferredGlobals* glb, float wx, float wy,
                                            float wz, float nx, float ny, float nz, float ndv, float rough, float metal,
                                            float f0r, float f0g, float f0b, float ar, float ag, float ab, float& hr,
                                            float& hg, float& hb) {
    float ir, ig, ib;
    irradiance(ev, glb, wx, wy, wz, nx, ny, nz, ir, ig, ib);
    const float x = fminf(fmaxf(1.0f - ndv, 0.0f), 1.0f);
    const float p5 = x * x * x * x * x, omr = 1.0f - rough;
    const float fr = f0r + (fmaxf(omr, f0r) - f0r) * p5, fg = f0g + (fmaxf(omr, f0g) - f0g) * p5,
                fb = f0b + (fmaxf(omr, f0b) - f0b) * p5;
    const float km = 1.0f - metal;
    const float dr = (1.0f - fr) * km * ir * ar, dg = (1.0f - fg) * km * ig * ag, db = (1.0f - fb) * km * ib * ab;
    const float w = fminf(fmaxf(sqrtf(ir * ir + ig * ig + ib * ib) * 4.0f, 0.0f), 1.0f);
    hr = hr * (1.0f - w) + dr * w;
    hg = hg * (1.0f - w) + dg * w;
    hb = hb * (1.0f - w) + db * w;
}

}  // namespace rc
}  // namespace hl
