// shadow_factor.h — CPU restatement of shadow_factor of Helio's deferred lighting pass
// (crates/passes/3d/helio-pass-deferred-light/shaders/deferred_lighting.wgsl:237-565),
// included by oracle.cpp.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle; see oracle.cpp).
//
// The normal-offset bias and the cascade distance are in the oracle's arithmetic type
// T (f64 for the accuracy oracle). The biased position is then rounded to f32 and the
// light-space projection, the per-pixel hash and the tap positions are formed in f32 in
// the shader's operation order without contraction (this file is compiled with
// -ffp-contract=off), because the shader forms them in f32 and the depth comparisons
// and texel choices follow from them; cos and sin of the f32 tap angle are the f64
// functions rounded once to f32. The comparison (LessEqual against the texel, four
// texels around u*S - 0.5, clamp-to-edge) is exact; its bilinear weights and the sums
// are f64.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace shadow_oracle {

struct ShadowDesc {  // hl_shadow_maps (include/helio_gb300.h), all memory on the host here
    const float* dyn;
    const float* sta;
    const float* mats;
    const void* cfg;
    uint32_t size, layers, max_lights, reserved;
};
static_assert(sizeof(ShadowDesc) == 48, "hl_shadow_maps is 48 bytes");

struct Config {  // ShadowConfig, libhelio/src/shadow.rs:33-64 (80 bytes)
    float cascades[4][4];  // split_distance, depth_bias, filter_radius, pcss_light_size
    uint32_t enable_pcss, pcss_blocker_samples, pcss_filter_samples, pcf_sample_count;
};
static_assert(sizeof(Config) == 80, "ShadowConfig is 80 bytes");

constexpr uint32_t kNoShadow = 0xFFFFFFFFu;

inline float fract_f(float x) { return x - std::floor(x); }

// hash22 (deferred_lighting.wgsl:246-250), f32.
inline float hash22(float px, float py) {
    const float p3x = fract_f(px * 0.1031f), p3y = fract_f(py * 0.1031f), p3z = p3x;
    const float d = (p3x * (p3y + 33.33f) + p3y * (p3z + 33.33f)) + p3z * (p3x + 33.33f);
    return fract_f((p3x + p3y) * d);
}

// vogel_disk_sample (:238-243) times radius, f32.
inline void vogel(uint32_t i, uint32_t n, float theta, float radius, float& ox, float& oy) {
    const float r = std::sqrt(float(i) + 0.5f) / std::sqrt(float(n));
    const float angle = float(i) * 2.39996323f + theta;
    const float c = float(std::cos(double(angle))), s = float(std::sin(double(angle)));
    ox = (c * r) * radius;
    oy = (s * r) * radius;
}

// clip = M (p, 1), ndc, uv (:281-290); false when outside the layer.
inline bool project(const float* m, float px, float py, float pz, float& u, float& v, float& z) {
    float c[4];
    for (int r = 0; r < 4; ++r) c[r] = ((m[r] * px + m[4 + r] * py) + m[8 + r] * pz) + m[12 + r];
    if (!(c[3] > 0.0f)) return false;
    const float nx = c[0] / c[3], ny = c[1] / c[3];
    z = c[2] / c[3];
    u = nx * 0.5f + 0.5f;
    v = -ny * 0.5f + 0.5f;
    return u >= 0.0f && v >= 0.0f && u <= 1.0f && v <= 1.0f && z >= 0.0f && z <= 1.0f;
}

// textureSampleCompareLevel, LessEqual, linear, clamp-to-edge.
inline double compare(const float* tex, uint32_t S, float u, float v, float ref) {
    const float fs = float(S);
    const float fx = std::fmaf(u, fs, -0.5f), fy = std::fmaf(v, fs, -0.5f);
    const double x0 = std::floor(double(fx)), y0 = std::floor(double(fy));
    const double ax = double(fx) - x0, ay = double(fy) - y0;
    auto cl = [&](double i) { return uint32_t(i < 0 ? 0.0 : (i > S - 1.0 ? S - 1.0 : i)); };
    const uint32_t i0 = cl(x0), i1 = cl(x0 + 1), j0 = cl(y0), j1 = cl(y0 + 1);
    auto t = [&](uint32_t i, uint32_t j) { return ref <= tex[size_t(j) * S + i] ? 1.0 : 0.0; };
    return (1 - ax) * (1 - ay) * t(i0, j0) + ax * (1 - ay) * t(i1, j0) + (1 - ax) * ay * t(i0, j1) + ax * ay * t(i1, j1);
}

inline double pcf(const ShadowDesc& sd, uint32_t layer, float u, float v, float ref, float radius, uint32_t count,
                  float theta) {
    const size_t off = size_t(layer) * sd.size * sd.size;
    double lit = 0.0;
    for (uint32_t i = 0; i < count; ++i) {
        float ox, oy;
        vogel(i, count, theta, radius, ox, oy);
        const float su = u + ox, sv = v + oy;
        lit += std::fmin(compare(sd.dyn + off, sd.size, su, sv, ref), compare(sd.sta + off, sd.size, su, sv, ref));
    }
    return lit / double(count);
}

// sample_cascade_shadow (:264-329). *bounds set for a layer beyond the atlas.
inline double sample_cascade(const ShadowDesc& sd, const Config& cf, uint32_t layer, uint32_t cascade, float scale,
                             float px, float py, float pz, float fx, float fy, int* bounds) {
    if (layer >= sd.layers) {
        *bounds = 1;
        return 1.0;
    }
    float u, v, z;
    if (!project(sd.mats + 16ull * layer, px, py, pz, u, v, z)) return 1.0;
    const float radius = (2.0f / float(sd.size)) * scale;
    const float theta = hash22(fx, fy) * 6.28318530718f;
    const uint32_t base = cf.pcf_sample_count;
    const uint32_t count = cascade == 0 ? base
                         : cascade == 1 ? std::max(base * 3u / 4u, 4u)
                         : cascade == 2 ? std::max(base / 2u, 4u)
                                        : std::max(base / 4u, 4u);
    return pcf(sd, layer, u, v, z, radius, count, theta);
}

// sample_cascade_shadow_pcss (:393-450) with pcss_blocker_search (:334-377).
inline double sample_cascade_pcss(const ShadowDesc& sd, const Config& cf, uint32_t layer, uint32_t cascade, float px,
                                  float py, float pz, float fx, float fy, int* bounds) {
    if (layer >= sd.layers) {
        *bounds = 1;
        return 1.0;
    }
    float u, v, z;
    if (!project(sd.mats + 16ull * layer, px, py, pz, u, v, z)) return 1.0;
    const float fs = float(sd.size);
    const double filter_radius = cf.cascades[cascade][2], light_size = cf.cascades[cascade][3];
    const float theta = hash22(fx, fy) * 6.28318530718f;
    const float search = cf.cascades[cascade][3] / fs;
    const size_t off = size_t(layer) * sd.size * sd.size;
    double bsum = 0.0, bcount = 0.0;
    const float ref = z - 0.0001f;
    for (uint32_t i = 0; i < cf.pcss_blocker_samples; ++i) {
        float ox, oy;
        vogel(i, cf.pcss_blocker_samples, theta, search, ox, oy);
        const int ix = int((u + ox) * fs), iy = int((v + oy) * fs);  // i32(f32): toward zero
        if (ix < 0 || iy < 0 || ix >= int(sd.size) || iy >= int(sd.size)) continue;
        const size_t t = off + size_t(iy) * sd.size + size_t(ix);
        const float occ = std::fmin(sd.dyn[t], sd.sta[t]);
        if (occ < ref) {
            bsum += occ;
            bcount += 1.0;
        }
    }
    if (bcount < 0.5) return 1.0;
    const double avg = bsum / bcount;
    const double penumbra = (double(z) - avg) / std::fmax(avg, 0.001) * light_size;
    const double radius = std::fmin(std::fmax(penumbra / fs, filter_radius / fs), filter_radius * 3.0 / fs);
    return pcf(sd, layer, u, v, z, float(radius), cf.pcss_filter_samples, theta);
}

inline uint32_t point_face(float dx, float dy, float dz) {  // :252-261
    const float ax = std::fabs(dx), ay = std::fabs(dy), az = std::fabs(dz);
    if (ax >= ay && ax >= az) return dx < 0.0f ? 1u : 0u;
    if (ay >= ax && ay >= az) return dy < 0.0f ? 3u : 2u;
    return dz < 0.0f ? 5u : 4u;
}

inline double directional_cascade(const ShadowDesc& sd, const Config& cf, uint32_t si, uint32_t c, float bx, float by,
                                  float bz, float fx, float fy, int* bounds) {
    if (cf.enable_pcss != 0u && cf.cascades[c][3] > 0.0f)
        return sample_cascade_pcss(sd, cf, si + c, c, bx, by, bz, fx, fy, bounds);
    return sample_cascade(sd, cf, si + c, c, 1.0f + float(c) * 1.5f, bx, by, bz, fx, fy, bounds);
}

// shadow_factor (:452-565) of light li (GpuLight fields as given) at world position P
// with unit normal N, fragment at pixel centre (fx, fy), camera at cam, CSM splits csm.
template <class T>
double shadow_factor(const ShadowDesc& sd, uint32_t li, const float pos[3], const float dir[3], uint32_t shadow_index,
                     uint32_t type, T Px, T Py, T Pz, T Nx, T Ny, T Nz, float fx, float fy, T cx, T cy, T cz,
                     const float csm[4], int* bounds) {
    if (li >= sd.max_lights || shadow_index == kNoShadow) return 1.0;
    Config cf;
    std::memcpy(&cf, sd.cfg, sizeof cf);
    T lx, ly, lz;
    if (type == 0u) {
        lx = -T(dir[0]);
        ly = -T(dir[1]);
        lz = -T(dir[2]);
    } else {
        lx = T(pos[0]) - Px;
        ly = T(pos[1]) - Py;
        lz = T(pos[2]) - Pz;
    }
    const T ll = std::sqrt(lx * lx + ly * ly + lz * lz);
    T ndl = (Nx * lx + Ny * ly + Nz * lz) / ll;
    if (ndl < T(0)) ndl = T(0);
    const T k = T(0.01) * (T(1) - ndl);
    const float bx = float(Px + Nx * k), by = float(Py + Ny * k), bz = float(Pz + Nz * k);
    if (type == 1u) {
        const uint32_t face = point_face(bx - pos[0], by - pos[1], bz - pos[2]);
        return sample_cascade(sd, cf, shadow_index + face, 0u, 1.0f, bx, by, bz, fx, fy, bounds);
    }
    if (type != 0u) return sample_cascade(sd, cf, shadow_index, 0u, 1.0f, bx, by, bz, fx, fy, bounds);
    const T dx = Px - cx, dy = Py - cy, dz = Pz - cz;
    const double dist = double(std::sqrt(dx * dx + dy * dy + dz * dz));
    const double lo0 = csm[0] * 0.95f, hi0 = csm[0] * 1.05f, lo1 = csm[1] * 0.95f, hi1 = csm[1] * 1.05f;
    const double lo2 = csm[2] * 0.95f, hi2 = csm[2] * 1.05f;
    auto smooth = [](double lo, double hi, double x) {
        double t = (x - lo) / (hi - lo);
        t = t < 0 ? 0 : (t > 1 ? 1 : t);
        return t * t * (3 - 2 * t);
    };
    uint32_t ca = 3, cb = 3;
    double blend = 0.0;
    if (dist < lo0) {
        ca = 0;
    } else if (dist < hi0) {
        ca = 0; cb = 1; blend = smooth(lo0, hi0, dist);
    } else if (dist < lo1) {
        ca = 1;
    } else if (dist < hi1) {
        ca = 1; cb = 2; blend = smooth(lo1, hi1, dist);
    } else if (dist < lo2) {
        ca = 2;
    } else if (dist < hi2) {
        ca = 2; cb = 3; blend = smooth(lo2, hi2, dist);
    }
    const double sa = directional_cascade(sd, cf, shadow_index, ca, bx, by, bz, fx, fy, bounds);
    if (blend <= 0.001 || cb == ca) return sa;
    const double sb = directional_cascade(sd, cf, shadow_index, cb, bx, by, bz, fx, fy, bounds);
    return sa * (1.0 - blend) + sb * blend;
}

}  // namespace shadow_oracle
