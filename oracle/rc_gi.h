// rc_gi.h — CPU restatement of the radiance-cascade indirect diffuse term of Helio's
// deferred lighting pass (crates/passes/3d/helio-pass-deferred-light/shaders/
// deferred_lighting.wgsl:822-917, composed at :1159-1163, 1197-1209; fresnel_schlick_
// roughness from crates/libhelio/shaders/pbr_eval.wgsl:63-66), included by oracle.cpp.
//
// TEST INFRASTRUCTURE ONLY (part of the oracle; see oracle.cpp). Arithmetic in the
// oracle's type T (f64 for the accuracy oracle); probe texels are Rgba16Float.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

namespace rc_oracle {

struct RcDesc {  // hl_rc_cascade (include/helio_gb300.h), texels in host memory here
    const void* texels;
    uint64_t pitch;
    uint32_t width, height;
};
static_assert(sizeof(RcDesc) == 24, "hl_rc_cascade is 24 bytes");

constexpr uint32_t kProbeDim = 16, kDirDim = 4;

inline double half_value(uint16_t h) {
    const uint32_t s = h >> 15, e = (h >> 10) & 31u, m = h & 1023u;
    double v;
    if (e == 0) v = std::ldexp(double(m), -24);
    else if (e == 31) v = m ? NAN : INFINITY;
    else v = std::ldexp(double(m | 1024u), int(e) - 25);
    return s ? -v : v;
}

template <class T> T smooth(T lo, T hi, T x) {
    T t = (x - lo) / (hi - lo);
    t = t < T(0) ? T(0) : (t > T(1) ? T(1) : t);
    return t * t * (T(3) - T(2) * t);
}

// sample_rc_irradiance at world position (wx, wy, wz), unit normal n; out[3].
template <class T>
void irradiance(const RcDesc& rc, const float* world_min, const float* world_max, T wx, T wy, T wz, T nx, T ny, T nz,
                T* out) {
    out[0] = out[1] = out[2] = T(0);
    const T mn[3] = {T(world_min[0]), T(world_min[1]), T(world_min[2])};
    const T size[3] = {T(world_max[0]) - mn[0], T(world_max[1]) - mn[1], T(world_max[2]) - mn[2]};
    if (size[0] <= T(0) || size[1] <= T(0) || size[2] <= T(0)) return;
    const T w[3] = {wx, wy, wz};
    T vw = T(1), pf[3];
    for (int k = 0; k < 3; ++k) {
        const T t = (w[k] - mn[k]) / size[k];
        vw *= smooth(T(0), T(0.05), t) * smooth(T(1), T(1) - T(0.05), t);
        const T cell = size[k] / T(kProbeDim);
        T p = (w[k] - mn[k]) / cell - T(0.5);
        pf[k] = p < T(0) ? T(0) : (p > T(kProbeDim - 1) ? T(kProbeDim - 1) : p);
    }
    if (vw <= T(0)) return;
    T cw[16];
    for (uint32_t ddx = 0; ddx < kDirDim; ++ddx) {
        for (uint32_t ddy = 0; ddy < kDirDim; ++ddy) {
            const T fx = (T(ddx) + T(0.5)) / T(kDirDim) * T(2) - T(1);
            const T fy = (T(ddy) + T(0.5)) / T(kDirDim) * T(2) - T(1);
            const T ax = std::fabs(fx), ay = std::fabs(fy), l = ax + ay;
            T d[3];
            if (l > T(1)) {
                d[0] = (T(1) - ay) * (fx >= T(0) ? T(1) : T(-1));
                d[1] = T(1) - l;
                d[2] = (T(1) - ax) * (fy >= T(0) ? T(1) : T(-1));
            } else {
                d[0] = fx; d[1] = T(1) - l; d[2] = fy;
            }
            const T dl = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            const T c = (nx * d[0] + ny * d[1] + nz * d[2]) / dl;
            cw[ddx * kDirDim + ddy] = c > T(0) ? c : T(0);
        }
    }
    const uint32_t ip[3] = {uint32_t(pf[0]), uint32_t(pf[1]), uint32_t(pf[2])};
    const T fr[3] = {pf[0] - std::floor(pf[0]), pf[1] - std::floor(pf[1]), pf[2] - std::floor(pf[2])};
    T c[8][3];
    for (int k = 0; k < 8; ++k) {
        const uint32_t px = std::min(ip[0] + uint32_t(k >> 2), kProbeDim - 1);
        const uint32_t py = std::min(ip[1] + uint32_t((k >> 1) & 1), kProbeDim - 1);
        const uint32_t pz = std::min(ip[2] + uint32_t(k & 1), kProbeDim - 1);
        T irr[3] = {T(0), T(0), T(0)}, ws = T(0);
        for (uint32_t ddx = 0; ddx < kDirDim; ++ddx) {
            for (uint32_t ddy = 0; ddy < kDirDim; ++ddy) {
                const T wgt = cw[ddx * kDirDim + ddy];
                if (!(wgt > T(0.001))) continue;
                const uint32_t ax = px * kDirDim + ddx, ay = (py * kProbeDim + pz) * kDirDim + ddy;
                uint16_t h[4];
                std::memcpy(h, static_cast<const unsigned char*>(rc.texels) + rc.pitch * ay + 8ull * ax, 8);
                for (int ch = 0; ch < 3; ++ch) irr[ch] += T(half_value(h[ch])) * wgt;
                ws += wgt;
            }
        }
        const T d = ws > T(0.001) ? ws : T(0.001);
        for (int ch = 0; ch < 3; ++ch) c[k][ch] = irr[ch] / d;
    }
    auto mix = [](T a, T b, T t) { return a * (T(1) - t) + b * t; };
    for (int ch = 0; ch < 3; ++ch) {
        const T c0 = mix(mix(c[0][ch], c[1][ch], fr[2]), mix(c[2][ch], c[3][ch], fr[2]), fr[1]);
        const T c1 = mix(mix(c[4][ch], c[5][ch], fr[2]), mix(c[6][ch], c[7][ch], fr[2]), fr[1]);
        out[ch] = mix(c0, c1, fr[0]) * vw;
    }
}

}  // namespace rc_oracle
