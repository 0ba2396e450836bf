// hl_shadow.cuh — shadow_factor of Helio's deferred lighting pass for sm_103a
// (deferred_lighting.wgsl:237-565): normal-offset bias, cube-face / cascade / spot layer
// selection, Vogel-disk PCF and PCSS over the dynamic and static Depth32Float atlases.
//
// The light-space projection, the per-pixel hash and the tap positions are f32 with
// correctly rounded, uncontracted operations in the shader's order, so the texel
// coordinates of every tap follow from the same f32 values the oracle forms; the
// comparison (LessEqual against the texel, bilinear over the four texels around the tap,
// clamp-to-edge) is exact, its weights f32.
#pragma once

#include "hl_common.cuh"
#include "hl_internal.h"

namespace hl {

namespace shadow {

constexpr float kNormalOffset = 0.01f;        // NORMAL_OFFSET_SCALE, deferred_lighting.wgsl:277
constexpr float kGoldenAngle = 2.39996323f;   // vogel_disk_sample, :240
constexpr float kTwoPi = 6.28318530718f;      // :287

__device__ __forceinline__ float fract_(float x) { return __fsub_rn(x, floorf(x)); }

// hash22 (:246-250) in f32, operations in the shader's order.
__device__ __forceinline__ float hash22(float px, float py) {
    const float p3x = fract_(__fmul_rn(px, 0.1031f)), p3y = fract_(__fmul_rn(py, 0.1031f));
    const float p3z = p3x;  // vec3(p.x, p.y, p.x) * 0.1031
    const float d = __fadd_rn(__fadd_rn(__fmul_rn(p3x, __fadd_rn(p3y, 33.33f)), __fmul_rn(p3y, __fadd_rn(p3z, 33.33f))),
                              __fmul_rn(p3z, __fadd_rn(p3x, 33.33f)));
    return fract_(__fmul_rn(__fadd_rn(p3x, p3y), d));
}

// vogel_disk_sample (:238-243) scaled by `radius`.
__device__ __forceinline__ void vogel(uint32_t i, uint32_t n, float theta, float radius, float& ox, float& oy) {
    const float r = __fdiv_rn(__fsqrt_rn(__fadd_rn(float(i), 0.5f)), __fsqrt_rn(float(n)));
    const float angle = __fadd_rn(__fmul_rn(float(i), kGoldenAngle), theta);
    float s, c;
    sincosf(angle, &s, &c);
    ox = __fmul_rn(__fmul_rn(c, r), radius);
    oy = __fmul_rn(__fmul_rn(s, r), radius);
}

// textureSampleCompareLevel with a LessEqual, linear, clamp-to-edge comparison sampler:
// the four texels around u*S - 0.5 compared with ref (1 when ref <= texel), blended
// bilinearly.
__device__ __forceinline__ float compare(const float* layer_texels, uint32_t S, float fs, float u, float v, float ref) {
    const float fx = __fmaf_rn(u, fs, -0.5f), fy = __fmaf_rn(v, fs, -0.5f);
    const float x0 = floorf(fx), y0 = floorf(fy);
    const float ax = fx - x0, ay = fy - y0;
    const float hi = fs - 1.0f;
    const uint32_t i0 = uint32_t(fminf(fmaxf(x0, 0.0f), hi)), i1 = uint32_t(fminf(fmaxf(x0 + 1.0f, 0.0f), hi));
    const uint32_t j0 = uint32_t(fminf(fmaxf(y0, 0.0f), hi)), j1 = uint32_t(fminf(fmaxf(y0 + 1.0f, 0.0f), hi));
    const float* r0 = layer_texels + size_t(j0) * S;
    const float* r1 = layer_texels + size_t(j1) * S;
    const float t00 = ref <= __ldg(r0 + i0) ? 1.0f : 0.0f, t10 = ref <= __ldg(r0 + i1) ? 1.0f : 0.0f;
    const float t01 = ref <= __ldg(r1 + i0) ? 1.0f : 0.0f, t11 = ref <= __ldg(r1 + i1) ? 1.0f : 0.0f;
    const float bx = 1.0f - ax, by = 1.0f - ay;
    return fmaf(t11, ax * ay, fmaf(t01, bx * ay, fmaf(t10, ax * by, t00 * (bx * by))));
}

// The light-space position of a layer: clip = M * (p, 1) (column major, summed in column
// order), ndc = clip.xyz / clip.w, uv = (ndc.x * 0.5 + 0.5, -ndc.y * 0.5 + 0.5).
// Returns false when the point is outside the layer (w <= 0, uv or depth outside [0,1]).
__device__ __forceinline__ bool project(const float* m, float px, float py, float pz, float& u, float& v, float& z) {
    float c[4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
        c[r] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(__ldg(m + r), px), __fmul_rn(__ldg(m + 4 + r), py)),
                                   __fmul_rn(__ldg(m + 8 + r), pz)),
                         __ldg(m + 12 + r));
    if (!(c[3] > 0.0f)) return false;
    const float nx = __fdiv_rn(c[0], c[3]), ny = __fdiv_rn(c[1], c[3]);
    z = __fdiv_rn(c[2], c[3]);
    u = __fadd_rn(__fmul_rn(nx, 0.5f), 0.5f);
    v = __fadd_rn(__fmul_rn(-ny, 0.5f), 0.5f);
    return u >= 0.0f && v >= 0.0f && u <= 1.0f && v <= 1.0f && z >= 0.0f && z <= 1.0f;
}

__device__ __forceinline__ bool layer_ok(const ExtView& sv, uint32_t layer) {
    if (layer < sv.layers) return true;
    raise_status(sv.status, HL_ERR_DEVICE_BOUNDS);
    return false;
}

// Vogel-disk PCF over both atlases at ref, lit = min(dynamic, static) per tap. Sample
// counts above kMaxSamples are rejected (lit, HL_ERR_SIZE) so that no launch loops for
// long on a corrupt configuration.
constexpr uint32_t kMaxSamples = 1024;
__device__ __forceinline__ float pcf(const ExtView& sv, uint32_t layer, float u, float v, float ref, float radius,
                                     uint32_t count, float theta) {
    if (count > kMaxSamples) {
        raise_status(sv.status, HL_ERR_SIZE);
        return 1.0f;
    }
    const size_t off = size_t(layer) * sv.size * sv.size;
    const float* dyn = sv.dyn + off;
    const float* sta = sv.sta + off;
    float lit = 0.0f;
    for (uint32_t i = 0; i < count; ++i) {
        float ox, oy;
        vogel(i, count, theta, radius, ox, oy);
        const float su = __fadd_rn(u, ox), sv_ = __fadd_rn(v, oy);
        lit += fminf(compare(dyn, sv.size, sv.fsize, su, sv_, ref), compare(sta, sv.size, sv.fsize, su, sv_, ref));
    }
    return lit / float(count);
}

__device__ __forceinline__ uint32_t cfg_u32(const ExtView& sv, int word) {
    return __ldg(reinterpret_cast<const uint32_t*>(sv.cfg) + word);
}
__device__ __forceinline__ float cfg_f32(const ExtView& sv, int word) {
    return __ldg(reinterpret_cast<const float*>(sv.cfg) + word);
}

// sample_cascade_shadow (:264-329).
static __device__ float sample_cascade(const ExtView& sv, uint32_t layer, uint32_t cascade, float scale, float px,
                                float py, float pz, float fx, float fy) {
    if (!layer_ok(sv, layer)) return 1.0f;
    float u, v, z;
    if (!project(sv.mats + 16ull * layer, px, py, pz, u, v, z)) return 1.0f;
    const float radius = __fmul_rn(__fdiv_rn(2.0f, sv.fsize), scale);
    const float theta = __fmul_rn(hash22(fx, fy), kTwoPi);
    const uint32_t base = cfg_u32(sv, 19);
    const uint32_t count = cascade == 0u ? base
                         : cascade == 1u ? max(base * 3u / 4u, 4u)
                         : cascade == 2u ? max(base / 2u, 4u)
                                         : max(base / 4u, 4u);
    return pcf(sv, layer, u, v, z, radius, count, theta);  // no samples: 0 / 0, as the shader
}

// sample_cascade_shadow_pcss (:393-450) with pcss_blocker_search (:334-377).
static __device__ float sample_cascade_pcss(const ExtView& sv, uint32_t layer, uint32_t cascade, float px, float py,
                                     float pz, float fx, float fy) {
    if (!layer_ok(sv, layer)) return 1.0f;
    float u, v, z;
    if (!project(sv.mats + 16ull * layer, px, py, pz, u, v, z)) return 1.0f;
    const float filter_radius = cfg_f32(sv, 4 * int(cascade) + 2), light_size = cfg_f32(sv, 4 * int(cascade) + 3);
    const float theta = __fmul_rn(hash22(fx, fy), kTwoPi);
    const float search = __fdiv_rn(light_size, sv.fsize);
    const uint32_t nb = cfg_u32(sv, 17), nf = cfg_u32(sv, 18);
    if (nb > kMaxSamples) {
        raise_status(sv.status, HL_ERR_SIZE);
        return 1.0f;
    }
    const size_t off = size_t(layer) * sv.size * sv.size;
    float bsum = 0.0f, bcount = 0.0f;
    const float ref = __fsub_rn(z, 0.0001f);
    for (uint32_t i = 0; i < nb; ++i) {
        float ox, oy;
        vogel(i, nb, theta, search, ox, oy);
        const int ix = __float2int_rz(__fmul_rn(__fadd_rn(u, ox), sv.fsize));
        const int iy = __float2int_rz(__fmul_rn(__fadd_rn(v, oy), sv.fsize));
        if (ix < 0 || iy < 0 || ix >= int(sv.size) || iy >= int(sv.size)) continue;
        const size_t t = off + size_t(iy) * sv.size + size_t(ix);
        const float occ = fminf(__ldg(sv.dyn + t), __ldg(sv.sta + t));
        if (occ < ref) {
            bsum += occ;
            bcount += 1.0f;
        }
    }
    if (bcount < 0.5f) return 1.0f;
    const float avg = bsum / bcount;
    const float penumbra = (z - avg) / fmaxf(avg, 0.001f) * light_size;
    const float radius = fminf(fmaxf(penumbra / sv.fsize, filter_radius / sv.fsize), filter_radius * 3.0f / sv.fsize);
    return pcf(sv, layer, u, v, z, radius, nf, theta);
}

// point_light_face (:252-261).
__device__ __forceinline__ uint32_t point_face(float dx, float dy, float dz) {
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    if (ax >= ay && ax >= az) return dx < 0.0f ? 1u : 0u;
    if (ay >= ax && ay >= az) return dy < 0.0f ? 3u : 2u;
    return dz < 0.0f ? 5u : 4u;
}

__device__ __forceinline__ float smoothstep_(float lo, float hi, float x) {
    const float t = fminf(fmaxf((x - lo) / (hi - lo), 0.0f), 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// One directional cascade: PCSS when enabled for it, else PCF with its scale.
static __device__ float directional_cascade(const ExtView& sv, uint32_t shadow_index, uint32_t c, float bx, float by,
                                     float bz, float fx, float fy) {
    const bool pcss = cfg_u32(sv, 16) != 0u && cfg_f32(sv, 4 * int(c) + 3) > 0.0f;
    if (pcss) return sample_cascade_pcss(sv, shadow_index + c, c, bx, by, bz, fx, fy);
    return sample_cascade(sv, shadow_index + c, c, __fadd_rn(1.0f, __fmul_rn(float(c), 1.5f)), bx, by, bz, fx, fy);
}

}  // namespace shadow

// shadow_factor (:452-565) of light `li` at world position w with unit normal n, for the
// fragment at pixel centre (fx, fy). Out of line: the shading kernels call it for lit
// pairs of shadow-casting lights only.
static __device__ __noinline__ float shadow_factor(const ExtView& sv, uint32_t li, float4 pos_range, float4 dir_outer,
                                            uint32_t shadow_index, uint32_t type, float wx, float wy, float wz,
                                            float nx, float ny, float nz, float fx, float fy, float camx, float camy,
                                            float camz, float4 csm) {
    using namespace shadow;
    if (li >= sv.max_lights || shadow_index == HL_NO_SHADOW) return 1.0f;
    float lx, ly, lz;
    if (type == 0u) {
        lx = -dir_outer.x;
        ly = -dir_outer.y;
        lz = -dir_outer.z;
    } else {
        lx = pos_range.x - wx;
        ly = pos_range.y - wy;
        lz = pos_range.z - wz;
    }
    const float il = rsqrtf(lx * lx + ly * ly + lz * lz);
    const float ndl = fmaxf((nx * lx + ny * ly + nz * lz) * il, 0.0f);
    const float k = kNormalOffset * (1.0f - ndl);
    const float bx = wx + nx * k, by = wy + ny * k, bz = wz + nz * k;
    if (type == 1u) {  // point: the cube face of the offset from the light
        const uint32_t face = point_face(__fsub_rn(bx, pos_range.x), __fsub_rn(by, pos_range.y), __fsub_rn(bz, pos_range.z));
        return sample_cascade(sv, shadow_index + face, 0u, 1.0f, bx, by, bz, fx, fy);
    }
    if (type != 0u)  // spot (and any other type): one layer
        return sample_cascade(sv, shadow_index, 0u, 1.0f, bx, by, bz, fx, fy);
    // directional: cascade of the distance to the camera, 10 % blend zones
    const float dx = wx - camx, dy = wy - camy, dz = wz - camz;
    const float dist = sqrtf(dx * dx + dy * dy + dz * dz);
    const float lo0 = csm.x * 0.95f, hi0 = csm.x * 1.05f, lo1 = csm.y * 0.95f, hi1 = csm.y * 1.05f;
    const float lo2 = csm.z * 0.95f, hi2 = csm.z * 1.05f;
    uint32_t ca = 3u, cb = 3u;
    float blend = 0.0f;
    if (dist < lo0) {
        ca = 0u;
    } else if (dist < hi0) {
        ca = 0u; cb = 1u; blend = smoothstep_(lo0, hi0, dist);
    } else if (dist < lo1) {
        ca = 1u;
    } else if (dist < hi1) {
        ca = 1u; cb = 2u; blend = smoothstep_(lo1, hi1, dist);
    } else if (dist < lo2) {
        ca = 2u;
    } else if (dist < hi2) {
        ca = 2u; cb = 3u; blend = smoothstep_(lo2, hi2, dist);
    }
    const float sa = directional_cascade(sv, shadow_index, ca, bx, by, bz, fx, fy);
    if (blend <= 0.001f || cb == ca) return sa;
    const float sb = directional_cascade(sv, shadow_index, cb, bx, by, bz, fx, fy);
    return sa * (1.0f - blend) + sb * blend;
}

}  // namespace hl
