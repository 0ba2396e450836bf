// hl_texel.cuh — decoding one G-buffer texel of each supported layout
// (gbuffer.wgsl:323-328 for the metallic F0; the reference layout's planes follow
// deferred_lighting.wgsl:991-1040). Shared by the shading and adjoint kernels.
#pragma once

#include <cuda_fp16.h>

#include "hl_common.cuh"
#include "hl_internal.h"
#include "hl_shade_math.cuh"

namespace hl {
namespace gbuf {

using namespace sm;

__device__ __forceinline__ float h2f(uint16_t h) { return __half2float(__ushort_as_half(h)); }

template <uint32_t LAYOUT>
struct Texel {
    float depth;
    float ar, ag, ab, alpha;
    float nx, ny, nz;
    float ao, rough, metal;
    float f0r, f0g, f0b;
    float er, eg, eb;
};

// The texel's planes as loaded, before decoding: a kernel may issue the loads early and
// decode later (decode_texel), so that their latency overlaps other work.
struct RawTexel {
    uint4 a;      // reference: RGBA8 albedo (x); F32: albedo + roughness; F16: RGBA16F (x, y)
    uint4 n;      // reference: normal + F0.r (x, y); F32: normal + metallic; F16: oct normal (x)
    uint2 o;      // reference: RGBA8 ao, roughness, metallic, F0.g (x); F16: metallic (x)
    uint2 e;      // reference: emissive + F0.b
    float depth;  // 1 outside the view
};

template <uint32_t LAYOUT>
__device__ __forceinline__ RawTexel load_raw(const GBufView& g, uint32_t x, uint32_t y) {
    RawTexel r{};
    if (LAYOUT == HL_GBUF_REFERENCE) {
        r.a.x = *reinterpret_cast<const uint32_t*>(g.plane[0] + g.pitch[0] * y + 4ull * x);
        const uint2 nr = *reinterpret_cast<const uint2*>(g.plane[1] + g.pitch[1] * y + 8ull * x);
        r.n.x = nr.x;
        r.n.y = nr.y;
        r.o.x = *reinterpret_cast<const uint32_t*>(g.plane[2] + g.pitch[2] * y + 4ull * x);
        r.e = *reinterpret_cast<const uint2*>(g.plane[3] + g.pitch[3] * y + 8ull * x);
        r.depth = *reinterpret_cast<const float*>(g.plane[4] + g.pitch[4] * y + 4ull * x);
    } else if (LAYOUT == HL_GBUF_F32) {
        r.a = *reinterpret_cast<const uint4*>(g.plane[0] + g.pitch[0] * y + 16ull * x);
        r.n = *reinterpret_cast<const uint4*>(g.plane[1] + g.pitch[1] * y + 16ull * x);
        r.depth = *reinterpret_cast<const float*>(g.plane[2] + g.pitch[2] * y + 4ull * x);
    } else {
        const uint2 a = *reinterpret_cast<const uint2*>(g.plane[0] + g.pitch[0] * y + 8ull * x);
        r.a.x = a.x;
        r.a.y = a.y;
        r.n.x = *reinterpret_cast<const uint32_t*>(g.plane[1] + g.pitch[1] * y + 4ull * x);
        r.o.x = *reinterpret_cast<const uint16_t*>(g.plane[2] + g.pitch[2] * y + 2ull * x);
        r.depth = *reinterpret_cast<const float*>(g.plane[3] + g.pitch[3] * y + 4ull * x);
    }
    return r;
}

template <uint32_t LAYOUT>
__device__ __forceinline__ Texel<LAYOUT> decode_texel(const RawTexel& r) {
    Texel<LAYOUT> t;
    t.depth = r.depth;
    if (LAYOUT == HL_GBUF_REFERENCE) {
        // RGBA8 bytes in memory order: x in the low byte
        t.ar = div_(float(r.a.x & 0xffu), 255.0f);
        t.ag = div_(float((r.a.x >> 8) & 0xffu), 255.0f);
        t.ab = div_(float((r.a.x >> 16) & 0xffu), 255.0f);
        t.alpha = div_(float(r.a.x >> 24), 255.0f);
        t.nx = h2f(uint16_t(r.n.x & 0xffffu));
        t.ny = h2f(uint16_t(r.n.x >> 16));
        t.nz = h2f(uint16_t(r.n.y & 0xffffu));
        t.f0r = h2f(uint16_t(r.n.y >> 16));
        t.ao = div_(float(r.o.x & 0xffu), 255.0f);
        t.rough = div_(float((r.o.x >> 8) & 0xffu), 255.0f);
        t.metal = div_(float((r.o.x >> 16) & 0xffu), 255.0f);
        t.f0g = div_(float(r.o.x >> 24), 255.0f);
        t.er = h2f(uint16_t(r.e.x & 0xffffu));
        t.eg = h2f(uint16_t(r.e.x >> 16));
        t.eb = h2f(uint16_t(r.e.y & 0xffffu));
        t.f0b = h2f(uint16_t(r.e.y >> 16));
    } else if (LAYOUT == HL_GBUF_F32) {
        t.ar = __uint_as_float(r.a.x);
        t.ag = __uint_as_float(r.a.y);
        t.ab = __uint_as_float(r.a.z);
        t.rough = __uint_as_float(r.a.w);
        t.nx = __uint_as_float(r.n.x);
        t.ny = __uint_as_float(r.n.y);
        t.nz = __uint_as_float(r.n.z);
        t.metal = __uint_as_float(r.n.w);
    } else {
        t.ar = h2f(uint16_t(r.a.x & 0xffffu));
        t.ag = h2f(uint16_t(r.a.x >> 16));
        t.ab = h2f(uint16_t(r.a.y & 0xffffu));
        t.rough = h2f(uint16_t(r.a.y >> 16));
        oct_decode(h2f(uint16_t(r.n.x & 0xffffu)), h2f(uint16_t(r.n.x >> 16)), t.nx, t.ny, t.nz);
        t.metal = h2f(uint16_t(r.o.x));
    }
    if (LAYOUT != HL_GBUF_REFERENCE) {
        t.alpha = 1.0f;
        t.ao = 1.0f;
        t.er = t.eg = t.eb = 0.0f;
        t.f0r = metallic_f0(t.ar, t.metal);
        t.f0g = metallic_f0(t.ag, t.metal);
        t.f0b = metallic_f0(t.ab, t.metal);
    }
    return t;
}

// Loads and decodes in one step (the same values as decode_texel(load_raw(...)); the
// kernels that read their texel among other loads keep this form, whose code the compiler
// schedules with theirs).
template <uint32_t LAYOUT>
__device__ __forceinline__ Texel<LAYOUT> load_texel(const GBufView& g, uint32_t x, uint32_t y) {
    Texel<LAYOUT> t;
    if (LAYOUT == HL_GBUF_REFERENCE) {
        const uchar4 a = *reinterpret_cast<const uchar4*>(g.plane[0] + g.pitch[0] * y + 4ull * x);
        const uint2 nr = *reinterpret_cast<const uint2*>(g.plane[1] + g.pitch[1] * y + 8ull * x);
        const uchar4 o = *reinterpret_cast<const uchar4*>(g.plane[2] + g.pitch[2] * y + 4ull * x);
        const uint2 e = *reinterpret_cast<const uint2*>(g.plane[3] + g.pitch[3] * y + 8ull * x);
        t.depth = *reinterpret_cast<const float*>(g.plane[4] + g.pitch[4] * y + 4ull * x);
        t.ar = div_(float(a.x), 255.0f);
        t.ag = div_(float(a.y), 255.0f);
        t.ab = div_(float(a.z), 255.0f);
        t.alpha = div_(float(a.w), 255.0f);
        t.nx = h2f(uint16_t(nr.x & 0xffffu));
        t.ny = h2f(uint16_t(nr.x >> 16));
        t.nz = h2f(uint16_t(nr.y & 0xffffu));
        t.f0r = h2f(uint16_t(nr.y >> 16));
        t.ao = div_(float(o.x), 255.0f);
        t.rough = div_(float(o.y), 255.0f);
        t.metal = div_(float(o.z), 255.0f);
        t.f0g = div_(float(o.w), 255.0f);
        t.er = h2f(uint16_t(e.x & 0xffffu));
        t.eg = h2f(uint16_t(e.x >> 16));
        t.eb = h2f(uint16_t(e.y & 0xffffu));
        t.f0b = h2f(uint16_t(e.y >> 16));
    } else if (LAYOUT == HL_GBUF_F32) {
        const float4 a = *reinterpret_cast<const float4*>(g.plane[0] + g.pitch[0] * y + 16ull * x);
        const float4 n = *reinterpret_cast<const float4*>(g.plane[1] + g.pitch[1] * y + 16ull * x);
        t.depth = *reinterpret_cast<const float*>(g.plane[2] + g.pitch[2] * y + 4ull * x);
        t.ar = a.x;
        t.ag = a.y;
        t.ab = a.z;
        t.rough = a.w;
        t.nx = n.x;
        t.ny = n.y;
        t.nz = n.z;
        t.metal = n.w;
    } else {
        const uint2 a = *reinterpret_cast<const uint2*>(g.plane[0] + g.pitch[0] * y + 8ull * x);
        const uint32_t on = *reinterpret_cast<const uint32_t*>(g.plane[1] + g.pitch[1] * y + 4ull * x);
        const uint16_t m = *reinterpret_cast<const uint16_t*>(g.plane[2] + g.pitch[2] * y + 2ull * x);
        t.depth = *reinterpret_cast<const float*>(g.plane[3] + g.pitch[3] * y + 4ull * x);
        t.ar = h2f(uint16_t(a.x & 0xffffu));
        t.ag = h2f(uint16_t(a.x >> 16));
        t.ab = h2f(uint16_t(a.y & 0xffffu));
        t.rough = h2f(uint16_t(a.y >> 16));
        oct_decode(h2f(uint16_t(on & 0xffffu)), h2f(uint16_t(on >> 16)), t.nx, t.ny, t.nz);
        t.metal = h2f(m);
    }
    if (LAYOUT != HL_GBUF_REFERENCE) {
        t.alpha = 1.0f;
        t.ao = 1.0f;
        t.er = t.eg = t.eb = 0.0f;
        t.f0r = metallic_f0(t.ar, t.metal);
        t.f0g = metallic_f0(t.ag, t.metal);
        t.f0b = metallic_f0(t.ab, t.metal);
    }
    return t;
}

// Planes of each layout and their bytes per texel.
template <uint32_t LAYOUT>
__host__ __device__ constexpr int plane_count() {
    return LAYOUT == HL_GBUF_REFERENCE ? 5 : LAYOUT == HL_GBUF_F32 ? 3 : 4;
}
template <uint32_t LAYOUT>
__host__ __device__ constexpr uint32_t plane_bpp(int p) {
    return LAYOUT == HL_GBUF_REFERENCE ? (p == 1 || p == 3 ? 8u : 4u)
         : LAYOUT == HL_GBUF_F32       ? (p < 2 ? 16u : 4u)
                                       : (p == 0 ? 8u : p == 2 ? 2u : 4u);
}

__device__ __forceinline__ void prefetch_l2(const void* p) { asm volatile("prefetch.global.L2 [%0];" ::"l"(p)); }

// Asks L2 for the rows of a w x h pixel block at (x0, y0) of one plane (bpp bytes per
// pixel): one prefetch per 128-byte step of each row, all inside the block's bytes.
// Thread t of n takes every n-th (row, step).
__device__ __forceinline__ void prefetch_block(const unsigned char* plane, uint64_t pitch, uint32_t bpp,
                                               uint32_t width, uint32_t height, uint32_t x0, uint32_t y0, uint32_t w,
                                               uint32_t h, uint32_t t, uint32_t n) {
    if (x0 >= width || y0 >= height) return;
    const uint32_t xe = min(x0 + w, width), ye = min(y0 + h, height);
    const uint32_t b0 = x0 * bpp, b1 = xe * bpp;
    const uint32_t steps = (b1 - b0 + 127u) / 128u + 1u;  // the last step reaches the block's last byte
    for (uint32_t i = t; i < (ye - y0) * steps; i += n) {
        const unsigned char* row = plane + pitch * (y0 + i / steps);
        prefetch_l2(row + min(b0 + 128u * (i % steps), b1 - 1u));
    }
}

// The G-buffer rows of a w x h tile at (x0, y0), every plane of the layout.
template <uint32_t LAYOUT>
__device__ __forceinline__ void prefetch_tile(const GBufView& g, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h,
                                              uint32_t t, uint32_t n) {
#pragma unroll
    for (int p = 0; p < plane_count<LAYOUT>(); ++p)
        prefetch_block(g.plane[p], g.pitch[p], plane_bpp<LAYOUT>(p), g.width, g.height, x0, y0, w, h, t, n);
}

}  // namespace gbuf
}  // namespace hl
