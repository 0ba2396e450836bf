// hl_gbuffer_write.cu — the fragment stage of Helio's GBufferPass for sm_103a
// (gbuffer.wgsl:287-497 under the default PBR template), and its C-ABI entry point.
//
// One thread per pixel, 32x8-pixel CTAs: a warp reads one row of 32 consecutive
// 64-byte surface records (2 KB contiguous) and writes 32 consecutive texels of every
// target. Materials and their texture slots are small tables read through L1; texture
// texels are gathered from L2. The texture table (up to 256 entries) and the sRGB
// decode table travel in the kernel parameters, so the call allocates nothing.
//
// Texture sampling is done in software at level 0 (the level a magnified or 1:1 texel
// footprint selects): the texel coordinate is fma(u, W, -0.5) rounded once to f32, the
// integer texel and the weights follow from it exactly, addressing wraps each integer
// coordinate (repeat / clamp-to-edge / mirrored-repeat as Vulkan and WebGPU define
// them), and the four texels are blended in f32. UVs go through select_uv
// (gbuffer.wgsl:287-297) with correctly rounded, uncontracted operations, so the texel
// coordinates are bit-identical to the oracle's.
#include <cuda_fp16.h>

#include <cmath>

#include "hl_common.cuh"
#include "hl_host.h"
#include "hl_internal.h"

namespace hl {
namespace {

constexpr uint32_t kGbwThreadsX = 32, kGbwThreadsY = 8;
constexpr uint32_t kMaxTexDim = 16384;

// Byte offsets of GpuMaterialTextures (helio/src/material.rs:156-187): seven 48-byte
// slots (texture_index u32 at 0, offset_scale f32x4 at 16, rotation f32x4 at 32),
// then params f32x4 (normal_scale, occlusion_strength, alpha_cutoff, -).
enum Slot : uint32_t { S_BASE = 0, S_NORMAL, S_RM, S_EMISSIVE, S_OCCLUSION, S_SPEC_COLOR, S_SPEC_WEIGHT };
constexpr uint32_t kSlotBytes = 48, kParamsOffset = 336;
static_assert(kParamsOffset + 16 == HL_SIZEOF_MATERIAL_TEXTURES, "GpuMaterialTextures is 352 bytes");
static_assert(sizeof(hl_surface) == 64, "hl_surface is 64 bytes");

constexpr uint32_t kFlagHasNormalMap = 1u << 3;  // libhelio/src/material.rs:189
constexpr uint32_t kWorkflowSpecular = 1u;        // gbuffer.wgsl:283

// A texture as the kernel reads it: 32 bytes. mode = format | addr_u << 4 | addr_v << 8
// | filter << 12; inv_w, inv_h = 1/width, 1/height (for the wrap quotient estimate).
struct TexDev {
    const unsigned char* p;
    uint32_t pitch;
    uint16_t w, h;
    uint32_t mode;
    float inv_w, inv_h;
    uint32_t pad;
};
static_assert(sizeof(TexDev) == 32, "TexDev is 32 bytes");

struct GbwParams {
    const unsigned char* globals;
    const unsigned char* surfaces;
    uint64_t surf_pitch;
    const unsigned char* mats;
    const unsigned char* mtex;
    uint32_t n_mat, n_tex;
    uint32_t W, H;
    unsigned char* out[HL_GBUFFER_TARGETS];
    uint64_t pitch[HL_GBUFFER_TARGETS];
    int* status;
    float srgb[256];  // sRGB 8-bit code -> 255 x linear, from the f64 formula rounded once
    TexDev tex[HL_MAX_MATERIAL_TEXTURES];
};

__device__ __forceinline__ float4 ldg4(const unsigned char* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ uint32_t ldgu(const unsigned char* p) { return __ldg(reinterpret_cast<const uint32_t*>(p)); }

// Exact modulus of an integer-valued float fi by period (>= 1; inv = 1/period): for
// |fi| < 2^24 the quotient is estimated in f32 (off by at most one) and the remainder
// corrected in integers, so no integer division is needed.
__device__ __forceinline__ int mod_coord(float fi, int period, float inv) {
    int m;
    if (fabsf(fi) < 16777216.0f) {
        m = int(fi) - period * int(floorf(fi * inv));
        if (m < 0) m += period;
        if (m >= period) m -= period;
    } else {  // beyond 2^24 texels every f32 coordinate is an integer: 64-bit remainder
        m = int(__float2ll_rz(fi) % (long long)period);
        if (m < 0) m += period;
    }
    return m;
}

// The texel columns (or rows) i0 = wrap(f0) and i1 = wrap(f0 + 1) of a coordinate f0
// (an integer-valued float) under the sampler's address mode (Vulkan / WebGPU:
// repeat, clamp-to-edge, mirrored-repeat with period 2n); inv_n = 1/n.
__device__ __forceinline__ void wrap_pair(float f0, int n, float inv_n, uint32_t mode, int& i0, int& i1) {
    if (f0 >= 0.0f && f0 < float(n - 1)) {  // both inside: every mode agrees
        i0 = int(f0);
        i1 = i0 + 1;
        return;
    }
    if (mode == HL_ADDRESS_CLAMP_TO_EDGE) {  // fmaxf maps NaN to 0
        i0 = int(fminf(fmaxf(f0, 0.0f), float(n - 1)));
        i1 = int(fminf(fmaxf(f0 + 1.0f, 0.0f), float(n - 1)));
        return;
    }
    const bool mirror = mode == HL_ADDRESS_MIRROR_REPEAT;
    const int period = mirror ? 2 * n : n;
    const int m0 = mod_coord(f0, period, mirror ? 0.5f * inv_n : inv_n);
    const int m1 = m0 + 1 == period ? 0 : m0 + 1;
    i0 = mirror && m0 >= n ? period - 1 - m0 : m0;
    i1 = mirror && m1 >= n ? period - 1 - m1 : m1;
}

// One texel's raw channels: RGBA8 unorm as byte values 0..255, RGBA8 sRGB as 255 x the
// linear value (the table) and the alpha byte, f16 / f32 as stored. The 8-bit formats
// are scaled by 1/255 once after filtering.
template <uint32_t FMT>
__device__ __forceinline__ float4 fetch_raw(const unsigned char* row, int ix, const float* srgb255) {
    if (FMT == HL_TEX_RGBA32F) return __ldg(reinterpret_cast<const float4*>(row) + ix);
    if (FMT == HL_TEX_RGBA16F) {
        const uint2 v = __ldg(reinterpret_cast<const uint2*>(row) + ix);
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
        return make_float4(a.x, a.y, b.x, b.y);
    }
    const uint32_t v = __ldg(reinterpret_cast<const uint32_t*>(row) + ix);
    const uint32_t r = v & 0xffu, g = (v >> 8) & 0xffu, b = (v >> 16) & 0xffu, a = v >> 24;
    if (FMT == HL_TEX_RGBA8_SRGB) return make_float4(srgb255[r], srgb255[g], srgb255[b], float(a));
    return make_float4(float(r), float(g), float(b), float(a));
}

__device__ __forceinline__ float4 blend4(float4 a, float4 b, float4 c, float4 d, float wa, float wb, float wc,
                                         float wd) {
    return make_float4(fmaf(d.x, wd, fmaf(c.x, wc, fmaf(b.x, wb, a.x * wa))),
                       fmaf(d.y, wd, fmaf(c.y, wc, fmaf(b.y, wb, a.y * wa))),
                       fmaf(d.z, wd, fmaf(c.z, wc, fmaf(b.z, wb, a.z * wa))),
                       fmaf(d.w, wd, fmaf(c.w, wc, fmaf(b.w, wb, a.w * wa))));
}

template <uint32_t FMT>
__device__ __forceinline__ float4 sample_fmt(const TexDev& t, float u, float v, const float* srgb255) {
    const int W = t.w, H = t.h;
    const uint32_t au = (t.mode >> 4) & 0xfu, av = (t.mode >> 8) & 0xfu;
    float4 r;
    if (((t.mode >> 12) & 0xfu) == HL_FILTER_NEAREST) {
        int x0, x1, y0, y1;
        wrap_pair(floorf(__fmul_rn(u, float(W))), W, t.inv_w, au, x0, x1);
        wrap_pair(floorf(__fmul_rn(v, float(H))), H, t.inv_h, av, y0, y1);
        r = fetch_raw<FMT>(t.p + uint64_t(t.pitch) * uint32_t(y0), x0, srgb255);
    } else {
        const float fx = __fmaf_rn(u, float(W), -0.5f), fy = __fmaf_rn(v, float(H), -0.5f);
        const float fx0 = floorf(fx), fy0 = floorf(fy);
        const float ax = fx - fx0, ay = fy - fy0;  // exact
        int x0, x1, y0, y1;
        wrap_pair(fx0, W, t.inv_w, au, x0, x1);
        wrap_pair(fy0, H, t.inv_h, av, y0, y1);
        const unsigned char* r0 = t.p + uint64_t(t.pitch) * uint32_t(y0);
        const unsigned char* r1 = t.p + uint64_t(t.pitch) * uint32_t(y1);
        const float4 t00 = fetch_raw<FMT>(r0, x0, srgb255), t10 = fetch_raw<FMT>(r0, x1, srgb255);
        const float4 t01 = fetch_raw<FMT>(r1, x0, srgb255), t11 = fetch_raw<FMT>(r1, x1, srgb255);
        const float bx = 1.0f - ax, by = 1.0f - ay;
        r = blend4(t00, t10, t01, t11, bx * by, ax * by, bx * ay, ax * ay);
    }
    if (FMT == HL_TEX_RGBA8_UNORM || FMT == HL_TEX_RGBA8_SRGB) {
        constexpr float k = 1.0f / 255.0f;
        r = make_float4(r.x * k, r.y * k, r.z * k, r.w * k);
    }
    return r;
}

// textureSample at level 0 (see the file comment).
__device__ __forceinline__ float4 sample_tex(const TexDev& t, float u, float v, const float* srgb255) {
    switch (t.mode & 0xfu) {
        case HL_TEX_RGBA8_SRGB: return sample_fmt<HL_TEX_RGBA8_SRGB>(t, u, v, srgb255);
        case HL_TEX_RGBA16F: return sample_fmt<HL_TEX_RGBA16F>(t, u, v, srgb255);
        case HL_TEX_RGBA32F: return sample_fmt<HL_TEX_RGBA32F>(t, u, v, srgb255);
        default: return sample_fmt<HL_TEX_RGBA8_UNORM>(t, u, v, srgb255);
    }
}

// sample_texture (gbuffer.wgsl:300-306) with select_uv (:287-297).
__device__ __forceinline__ float4 sample_slot(const TexDev* tex, uint32_t n_tex, int* status, const float* srgb255,
                                              const unsigned char* slot, float u, float v, float4 fallback) {
    const uint32_t idx = ldgu(slot);
    if (idx == HL_NO_TEXTURE) return fallback;
    if (idx >= n_tex) {
        raise_status(status, HL_ERR_DEVICE_BOUNDS);
        return fallback;
    }
    const float4 os = ldg4(slot + 16), rot = ldg4(slot + 32);
    const float sx = __fmul_rn(u, os.z), sy = __fmul_rn(v, os.w);
    const float s = rot.x, c = rot.y;
    const float rx = __fsub_rn(__fmul_rn(sx, c), __fmul_rn(sy, s));
    const float ry = __fadd_rn(__fmul_rn(sx, s), __fmul_rn(sy, c));
    return sample_tex(tex[idx], __fadd_rn(rx, os.x), __fadd_rn(ry, os.y), srgb255);
}

__device__ __forceinline__ float3 normalize3(float x, float y, float z) {
    const float inv = rsqrtf(x * x + y * y + z * z);
    return make_float3(x * inv, y * inv, z * inv);
}

__device__ __forceinline__ uint32_t to_unorm8(float v) { return __float2uint_rn(__saturatef(v) * 255.0f); }
__device__ __forceinline__ uint32_t pack_unorm8(float r, float g, float b, float a) {
    return to_unorm8(r) | (to_unorm8(g) << 8) | (to_unorm8(b) << 16) | (to_unorm8(a) << 24);
}
__device__ __forceinline__ uint32_t pack_h2(float a, float b) {
    const __half2 h = __floats2half2_rn(a, b);
    return *reinterpret_cast<const uint32_t*>(&h);
}

struct GbOut {
    float albedo[4], normal[4], orm[4], emissive[4];
};

__device__ __forceinline__ void store_targets(const GbwParams& p, uint32_t x, uint32_t y, const GbOut& o, float lmu,
                                              float lmv, float velx, float vely) {
    *reinterpret_cast<uint32_t*>(p.out[0] + p.pitch[0] * y + 4ull * x) =
        pack_unorm8(o.albedo[0], o.albedo[1], o.albedo[2], o.albedo[3]);
    *reinterpret_cast<uint2*>(p.out[1] + p.pitch[1] * y + 8ull * x) =
        make_uint2(pack_h2(o.normal[0], o.normal[1]), pack_h2(o.normal[2], o.normal[3]));
    *reinterpret_cast<uint32_t*>(p.out[2] + p.pitch[2] * y + 4ull * x) =
        pack_unorm8(o.orm[0], o.orm[1], o.orm[2], o.orm[3]);
    *reinterpret_cast<uint2*>(p.out[3] + p.pitch[3] * y + 8ull * x) =
        make_uint2(pack_h2(o.emissive[0], o.emissive[1]), pack_h2(o.emissive[2], o.emissive[3]));
    if (p.out[4]) *reinterpret_cast<uint32_t*>(p.out[4] + p.pitch[4] * y + 4ull * x) = pack_h2(lmu, lmv);
    if (p.out[5]) *reinterpret_cast<uint2*>(p.out[5] + p.pitch[5] * y + 8ull * x) = make_uint2(0u, 0u);
    if (p.out[6]) *reinterpret_cast<uint2*>(p.out[6] + p.pitch[6] * y + 8ull * x) = make_uint2(0u, 0u);
    if (p.out[7]) *reinterpret_cast<uint32_t*>(p.out[7] + p.pitch[7] * y + 4ull * x) = pack_h2(velx, vely);
}

__global__ void __launch_bounds__(kGbwThreadsX * kGbwThreadsY, 4)
gbuffer_write_kernel(const __grid_constant__ GbwParams p) {
    __shared__ float srgb[256];
    __shared__ float4 samp[7][kGbwThreadsX * kGbwThreadsY];  // each thread's texture samples
    const uint32_t t = threadIdx.y * kGbwThreadsX + threadIdx.x;
    srgb[t] = p.srgb[t];
    __syncthreads();
    const uint32_t x = blockIdx.x * kGbwThreadsX + threadIdx.x, y = blockIdx.y * kGbwThreadsY + threadIdx.y;
    if (x >= p.W || y >= p.H) return;

    const unsigned char* rec = p.surfaces + p.surf_pitch * y + 64ull * x;
    const float4 s0 = ldg4(rec), s1 = ldg4(rec + 16), s2 = ldg4(rec + 32), s3 = ldg4(rec + 48);
    const uint32_t mid = __float_as_uint(s1.w);
    if (mid == HL_NO_FRAGMENT) return;
    if (mid >= p.n_mat) {
        raise_status(p.status, HL_ERR_DEVICE_BOUNDS);
        return;
    }
    const float u = s2.x, v = s2.y;

    // compute_velocity (gbuffer.wgsl:417-423) in f32 as the shader writes it, each
    // operation rounded once (no contraction); clip_position.xy is the pixel centre
    const float pnx = __fdiv_rn(s3.x, s3.w), pny = __fdiv_rn(s3.y, s3.w);
    const float velx = __fsub_rn(float(x) + 0.5f, __fmul_rn(__fadd_rn(__fmul_rn(pnx, 0.5f), 0.5f), float(p.W)));
    const float vely = __fsub_rn(float(y) + 0.5f, __fmul_rn(__fsub_rn(0.5f, __fmul_rn(pny, 0.5f)), float(p.H)));

    const unsigned char* mat = p.mats + 96ull * mid;
    const unsigned char* mt = p.mtex + uint64_t(HL_SIZEOF_MATERIAL_TEXTURES) * mid;
    const uint32_t debug = ldgu(p.globals + 80);
    const float4 one = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    const float4 base_color = ldg4(mat), emis = ldg4(mat + 16), rm = ldg4(mat + 32);
    const float4 prm = ldg4(mt + kParamsOffset);
    const uint32_t flags = ldgu(mat + 72);
    const bool specular = ldgu(mat + 68) == kWorkflowSpecular;
    const bool normal_mapped = (flags & kFlagHasNormalMap) != 0u && ldgu(mt + S_NORMAL * kSlotBytes) != HL_NO_TEXTURE;

    // The slots this pixel samples, base colour first (its alpha decides the discard
    // before anything else is sampled). One loop body holds the only copy of the
    // sampler; each result goes to this thread's column of samp.
    uint32_t need = 1u << S_BASE;
    if (debug == 1u) need = 0u;
    else if (debug == 3u) need |= 1u << S_RM;
    else if (debug != 2u) {
        need |= (1u << S_RM) | (1u << S_OCCLUSION) | (1u << S_EMISSIVE);
        if (normal_mapped) need |= 1u << S_NORMAL;
        if (specular) need |= (1u << S_SPEC_COLOR) | (1u << S_SPEC_WEIGHT);
    }
    for (uint32_t m = need; m != 0u; m &= m - 1u) {
        const uint32_t k = __ffs(m) - 1u;
        const float4 fb = k == S_NORMAL ? make_float4(0.5f, 0.5f, 1.0f, 1.0f) : one;
        const float4 r = sample_slot(p.tex, p.n_tex, p.status, srgb, mt + k * kSlotBytes, u, v, fb);
        samp[k][t] = r;
        // default_pbr_surface's alpha, and the discard of gbuffer.wgsl:484-485
        if (k == S_BASE && debug == 0u) {
            const float alpha = base_color.w * r.w;
            if (alpha <= 0.001f || alpha < prm.z) return;
        }
    }
    GbOut o;
    if (debug == 1u || debug == 2u) {  // gbuffer.wgsl:431-459
        float4 a = make_float4(u, v, 0.0f, 1.0f);
        if (debug == 2u) {
            const float4 b = samp[S_BASE][t];
            a = make_float4(b.x, b.y, b.z, 1.0f);
        }
        o = GbOut{{a.x, a.y, a.z, a.w}, {0.0f, 0.0f, 1.0f, 0.0f}, {0, 0, 0, 0}, {0, 0, 0, 0}};
        store_targets(p, x, y, o, 0.0f, 0.0f, velx, vely);
        return;
    }

    const float4 base = samp[S_BASE][t];
    const float4 albedo = make_float4(base_color.x * base.x, base_color.y * base.y, base_color.z * base.z,
                                      base_color.w * base.w);
    const float3 ng = normalize3(s0.x, s0.y, s0.z);
    const float4 orm_s = samp[S_RM][t];
    const float rough = fminf(fmaxf(rm.x * orm_s.y, 0.045f), 1.0f);
    const float metal = fminf(fmaxf(rm.y * orm_s.z, 0.0f), 1.0f);

    if (debug == 3u) {  // gbuffer.wgsl:461-478
        o = GbOut{{albedo.x, albedo.y, albedo.z, albedo.w}, {ng.x, ng.y, ng.z, 0.0f}, {1.0f, rough, metal, 0.0f},
                  {0, 0, 0, 0}};
        store_targets(p, x, y, o, 0.0f, 0.0f, velx, vely);
        return;
    }

    // default_pbr_surface (gbuffer.wgsl:333-364)
    const float alpha = albedo.w;
    float3 n = ng;
    if (normal_mapped) {
        const float tdn = s1.x * ng.x + s1.y * ng.y + s1.z * ng.z;
        const float3 tt = normalize3(s1.x - tdn * ng.x, s1.y - tdn * ng.y, s1.z - tdn * ng.z);
        const float bs = s0.w;
        const float3 bb = make_float3((ng.y * tt.z - ng.z * tt.y) * bs, (ng.z * tt.x - ng.x * tt.z) * bs,
                                      (ng.x * tt.y - ng.y * tt.x) * bs);
        const float4 ns = samp[S_NORMAL][t];
        const float tx = (ns.x * 2.0f - 1.0f) * prm.x, ty = (ns.y * 2.0f - 1.0f) * prm.x, tz = ns.z * 2.0f - 1.0f;
        n = normalize3(tt.x * tx + bb.x * ty + ng.x * tz, tt.y * tx + bb.y * ty + ng.y * tz,
                       tt.z * tx + bb.z * ty + ng.z * tz);
    }
    const float4 occ = samp[S_OCCLUSION][t];
    const float4 em_s = samp[S_EMISSIVE][t];
    const float ao = 1.0f + (occ.x - 1.0f) * prm.y;

    // resolve_specular_f0 (gbuffer.wgsl:308-329)
    float f0r, f0g, f0b;
    if (specular) {
        const float4 sc = samp[S_SPEC_COLOR][t];
        const float4 sw = samp[S_SPEC_WEIGHT][t];
        const float ior = fmaxf(rm.z, 1.0f);
        const float q = (ior - 1.0f) / (ior + 1.0f);
        const float k = rm.w * sw.w;
        const float d = q * q;
        f0r = k * sc.x * d;
        f0g = k * sc.y * d;
        f0b = k * sc.z * d;
    } else {
        // mix(0.04, albedo, metallic) = 0.04 (1 - metallic) + albedo metallic, clamped
        const float d = 0.04f * (1.0f - metal);
        f0r = fminf(fmaxf(fmaf(albedo.x, metal, d), 0.0f), 0.999f);
        f0g = fminf(fmaxf(fmaf(albedo.y, metal, d), 0.0f), 0.999f);
        f0b = fminf(fmaxf(fmaf(albedo.z, metal, d), 0.0f), 0.999f);
    }
    const float ew = emis.w;
    o = GbOut{{albedo.x, albedo.y, albedo.z, alpha},
              {n.x, n.y, n.z, f0r},
              {ao, rough, metal, f0g},
              {emis.x * ew * em_s.x, emis.y * ew * em_s.y, emis.z * ew * em_s.z, f0b}};
    store_targets(p, x, y, o, s2.z, s2.w, velx, vely);
}

}  // namespace
}  // namespace hl

namespace {

using namespace hl_host;

constexpr uint32_t kTargetBpp[HL_GBUFFER_TARGETS] = {4, 8, 4, 8, 4, 8, 8, 4};
constexpr uint32_t kTexBpp[4] = {4, 4, 8, 16};

// 255 x the f64 sRGB electro-optical transfer function of each 8-bit code, rounded to
// f32 (the kernel filters 8-bit texels in units of 1/255 and scales once).
void srgb_table(float* out) {
    for (int i = 0; i < 256; ++i) {
        const double c = double(i) / 255.0;
        out[i] = float(255.0 * (c <= 0.04045 ? c / 12.92 : std::pow((c + 0.055) / 1.055, 2.4)));
    }
}

}  // namespace

extern "C" hl_status hl_write_gbuffer(hl_ctx* ctx, const void* globals, const hl_surface* surfaces,
                                      uint64_t surfaces_pitch, const void* materials, const void* material_textures,
                                      uint32_t n_materials, const hl_texture* textures, uint32_t n_textures,
                                      const hl_gbuffer_targets* targets, void* stream) {
    if (!ctx) return HL_ERR_INVALID_ARGUMENT;
    if (!globals || !aligned(globals, 16)) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "globals is NULL or misaligned");
    if (!targets) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "targets is NULL");
    const uint32_t W = targets->width, H = targets->height;
    if (W == 0 || H == 0) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "targets are %ux%u", W, H);
    if (W > (1u << 16) || H > (1u << 16))
        return fail(ctx, HL_ERR_SIZE, "targets %ux%u exceed 65536 pixels per side", W, H);
    if (!surfaces || !aligned(surfaces, 16) || surfaces_pitch % 16 != 0)
        return fail(ctx, HL_ERR_LAYOUT, "surfaces NULL or pointer/pitch not 16-byte aligned");
    if (surfaces_pitch < uint64_t(W) * sizeof(hl_surface))
        return fail(ctx, HL_ERR_LAYOUT, "surfaces pitch %llu < %u x 64 bytes", (unsigned long long)surfaces_pitch, W);
    if (n_materials > 0 && (!materials || !material_textures))
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "materials or material_textures is NULL with n_materials=%u",
                    n_materials);
    if ((materials && !aligned(materials, 16)) || (material_textures && !aligned(material_textures, 16)))
        return fail(ctx, HL_ERR_LAYOUT, "materials / material_textures not 16-byte aligned");
    if (n_textures > HL_MAX_MATERIAL_TEXTURES)
        return fail(ctx, HL_ERR_SIZE, "n_textures %u exceeds %u", n_textures, HL_MAX_MATERIAL_TEXTURES);
    if (n_textures > 0 && !textures) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "textures is NULL with n_textures=%u", n_textures);

    hl::GbwParams p;
    std::memset(&p, 0, sizeof p);
    for (uint32_t i = 0; i < n_textures; ++i) {
        const hl_texture& t = textures[i];
        if (!t.texels) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "texture %u has no texels", i);
        if (t.format > HL_TEX_RGBA32F || t.address_u > HL_ADDRESS_MIRROR_REPEAT ||
            t.address_v > HL_ADDRESS_MIRROR_REPEAT || t.filter > HL_FILTER_LINEAR)
            return fail(ctx, HL_ERR_INVALID_ARGUMENT, "texture %u: unknown format, address mode or filter", i);
        if (t.width == 0 || t.height == 0 || t.width > hl::kMaxTexDim || t.height > hl::kMaxTexDim)
            return fail(ctx, HL_ERR_SIZE, "texture %u is %ux%u (1..%u per side)", i, t.width, t.height, hl::kMaxTexDim);
        const uint32_t bpp = kTexBpp[t.format];
        if (!aligned(t.texels, bpp) || t.pitch % bpp != 0)
            return fail(ctx, HL_ERR_LAYOUT, "texture %u pointer/pitch not %u-byte aligned", i, bpp);
        if (t.pitch < uint64_t(t.width) * bpp || t.pitch > 0xFFFFFFFFull)
            return fail(ctx, HL_ERR_LAYOUT, "texture %u pitch %llu out of range", i, (unsigned long long)t.pitch);
        p.tex[i] = hl::TexDev{static_cast<const unsigned char*>(t.texels), uint32_t(t.pitch), uint16_t(t.width),
                              uint16_t(t.height), t.format | (t.address_u << 4) | (t.address_v << 8) | (t.filter << 12),
                              1.0f / float(t.width), 1.0f / float(t.height), 0u};
    }
    for (int i = 0; i < HL_GBUFFER_TARGETS; ++i) {
        void* d = targets->planes[i];
        if (!d) {
            if (i < 4) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "G-buffer target %d is NULL", i);
            continue;
        }
        if (!aligned(d, kTargetBpp[i]) || targets->pitch[i] % kTargetBpp[i] != 0)
            return fail(ctx, HL_ERR_LAYOUT, "G-buffer target %d pointer/pitch not %u-byte aligned", i, kTargetBpp[i]);
        if (targets->pitch[i] < uint64_t(W) * kTargetBpp[i])
            return fail(ctx, HL_ERR_LAYOUT, "G-buffer target %d pitch too small", i);
        p.out[i] = static_cast<unsigned char*>(d);
        p.pitch[i] = targets->pitch[i];
    }
    p.globals = static_cast<const unsigned char*>(globals);
    p.surfaces = reinterpret_cast<const unsigned char*>(surfaces);
    p.surf_pitch = surfaces_pitch;
    p.mats = static_cast<const unsigned char*>(materials);
    p.mtex = static_cast<const unsigned char*>(material_textures);
    p.n_mat = n_materials;
    p.n_tex = n_textures;
    p.W = W;
    p.H = H;
    p.status = ctx->d_status;
    srgb_table(p.srgb);

    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    const dim3 block(hl::kGbwThreadsX, hl::kGbwThreadsY);
    const dim3 grid((W + hl::kGbwThreadsX - 1) / hl::kGbwThreadsX, (H + hl::kGbwThreadsY - 1) / hl::kGbwThreadsY);
    hl::gbuffer_write_kernel<<<grid, block, 0, as_stream(stream)>>>(p);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_fail(ctx, e, "G-buffer write launch");
    return HL_OK;
}
