// hl_reflect.cu — the reflection draw of Helio's deferred pass for sm_103a
// (fs_reflection, deferred_lighting.wgsl:1265-1341), and its C-ABI entry point.
//
// One thread per pixel, 32x8-pixel CTAs: the pass is a per-pixel read of the G-buffer,
// the SSR and planar hit images and the lightmap UVs, and a read-modify-write of the
// lit target (the additive blend of the reference's second draw: colour One + One,
// alpha kept). Only pixels rough enough for the radiance-cascade fallback
// (roughness > 0.6 with has_rc_gi) gather the 8 probe corners, through the same
// sampler as the ambient term of the lighting kernel (sample_rc_specular, :928-980, is
// sample_rc_irradiance along another direction). The world position is reconstructed
// in double-float as in the precise lighting paths and V normalised from it in f32, so
// the Fresnel term and the reflection vector carry f32 rounding only.
#include <cuda_fp16.h>

#include "hl_common.cuh"
#include "hl_host.h"
#include "hl_indirect.cuh"
#include "hl_internal.h"
#include "hl_shade_math.cuh"
#include "hl_texel.cuh"

namespace hl {
namespace {

using namespace sm;

constexpr uint32_t kRefThreadsX = 32, kRefThreadsY = 8;

// The reflection captures and their cube-map array (hl_reflection_env).
struct EnvView {
    const unsigned char* caps;    // GpuReflectionCapture[count], 112 B each; nullptr: none bound
    const unsigned char* texels;  // RGBA16F, layer-major, 6 faces, each face's mip chain
    uint32_t count, size, levels, layers;
    uint64_t chain;               // texels of one face's mip chain
};

struct ReflectParams {
    GBufView gb;
    TargetView out;
    const GpuCamera* camera;
    const DeferredGlobals* globals;
    const unsigned char* ssr;
    uint64_t ssr_pitch;
    const unsigned char* planar;
    uint64_t planar_pitch;
    const unsigned char* lmuv;
    uint64_t lmuv_pitch;
    ExtView rc;  // rc.rc == nullptr: no probes bound
    EnvView env;
    int* status;
};

__device__ __forceinline__ float4 load_h4(const unsigned char* p) {
    const uint2 v = __ldg(reinterpret_cast<const uint2*>(p));
    const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&v.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&v.y));
    return make_float4(a.x, a.y, b.x, b.y);
}

// The target texel as four floats, and its store (alpha carried through bit for bit).
template <uint32_t TARGET>
struct TargetTexel {
    float4 v;
    uint32_t alpha_bits;  // RGBA16F: the alpha half's bits
};

template <uint32_t TARGET>
__device__ __forceinline__ TargetTexel<TARGET> load_target(const unsigned char* o) {
    TargetTexel<TARGET> t;
    if (TARGET == HL_TARGET_RGBA32F) {
        t.v = *reinterpret_cast<const float4*>(o);
        t.alpha_bits = 0;
    } else {
        const uint2 q = *reinterpret_cast<const uint2*>(o);
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&q.y));
        t.v = make_float4(a.x, a.y, b.x, b.y);
        t.alpha_bits = q.y >> 16;
    }
    return t;
}

// Writes (r, g, b) and either the given alpha or the texel's own alpha bits.
template <uint32_t TARGET>
__device__ __forceinline__ void store_target(unsigned char* o, const TargetTexel<TARGET>& t, float r, float g, float b,
                                             const float* alpha) {
    if (TARGET == HL_TARGET_RGBA32F) {
        *reinterpret_cast<float4*>(o) = make_float4(r, g, b, alpha ? *alpha : t.v.w);
    } else {
        const __half2 rg = __floats2half2_rn(r, g);
        const uint32_t bb = uint32_t(__half_as_ushort(__float2half_rn(b)));
        const uint32_t ab = alpha ? uint32_t(__half_as_ushort(__float2half_rn(*alpha))) : t.alpha_bits;
        *reinterpret_cast<uint2*>(o) = make_uint2(*reinterpret_cast<const uint32_t*>(&rg), bb | (ab << 16));
    }
}

// One level of one cube layer sampled as the pass's env sampler does: the face of the
// direction's major axis (ties to z, then y), the face coordinates of the Vulkan /
// WebGPU cube-map table, bilinear within the face with the edge texels clamped.
__device__ __forceinline__ void cube_sample(const EnvView& e, float dx, float dy, float dz, uint32_t layer,
                                            uint32_t level, float& r, float& g, float& b) {
    const float ax = fabsf(dx), ay = fabsf(dy), az = fabsf(dz);
    uint32_t face;
    float sc, tc, ma;
    if (az >= ax && az >= ay) {
        face = dz >= 0.0f ? 4u : 5u;
        sc = dz >= 0.0f ? dx : -dx;
        tc = -dy;
        ma = az;
    } else if (ay >= ax) {
        face = dy >= 0.0f ? 2u : 3u;
        sc = dx;
        tc = dy >= 0.0f ? dz : -dz;
        ma = ay;
    } else {
        face = dx >= 0.0f ? 0u : 1u;
        sc = dx >= 0.0f ? -dz : dz;
        tc = -dy;
        ma = ax;
    }
    const float sf = ma > 0.0f ? 0.5f * (sc / ma + 1.0f) : 0.5f, tf = ma > 0.0f ? 0.5f * (tc / ma + 1.0f) : 0.5f;
    const uint32_t n = max(1u, e.size >> level);
    uint64_t off = 0;
    for (uint32_t m = 0; m < level; ++m) {
        const uint64_t nm = max(1u, e.size >> m);
        off += nm * nm;
    }
    const unsigned char* base = e.texels + 8ull * ((uint64_t(layer) * 6u + face) * e.chain + off);
    const float u = sf * float(n) - 0.5f, v = tf * float(n) - 0.5f;
    const float fu = floorf(u), fv = floorf(v);
    const float wu = u - fu, wv = v - fv;
    const int iu = int(fu), iv = int(fv), top = int(n) - 1;
    const int u0 = min(max(iu, 0), top), u1 = min(max(iu + 1, 0), top);
    const int v0 = min(max(iv, 0), top), v1 = min(max(iv + 1, 0), top);
    const float4 t00 = load_h4(base + 8ull * (uint64_t(v0) * n + u0)), t01 = load_h4(base + 8ull * (uint64_t(v0) * n + u1));
    const float4 t10 = load_h4(base + 8ull * (uint64_t(v1) * n + u0)), t11 = load_h4(base + 8ull * (uint64_t(v1) * n + u1));
    r = (t00.x * (1.0f - wu) + t01.x * wu) * (1.0f - wv) + (t10.x * (1.0f - wu) + t11.x * wu) * wv;
    g = (t00.y * (1.0f - wu) + t01.y * wu) * (1.0f - wv) + (t10.y * (1.0f - wu) + t11.y * wu) * wv;
    b = (t00.z * (1.0f - wu) + t01.z * wu) * (1.0f - wv) + (t10.z * (1.0f - wu) + t11.z * wu) * wv;
}

// The 16 floats of a column-major mat4 times (x, y, z, w), row r.
__device__ __forceinline__ float mrow(const float* m, int r, float x, float y, float z, float w) {
    return m[r] * x + m[4 + r] * y + m[8 + r] * z + m[12 + r] * w;
}

// sample_reflection_environment (deferred_lighting.wgsl:646-694) with capture_weight
// (:618-638), parallax_box (:596-616) and parallax_sphere (:575-588).
__device__ __noinline__ float3 reflection_environment(const EnvView& e, uint32_t count, float Px, float Py, float Pz,
                                                      float Rx, float Ry, float Rz, float lod, int* status) {
    // the env sampler's nearest level: ceil(lod + 0.5) - 1, within the chain
    const int lvl = int(ceilf(lod + 0.5f)) - 1;
    const uint32_t level = uint32_t(min(max(lvl, 0), int(e.levels) - 1));
    float ar = 0.0f, ag = 0.0f, ab = 0.0f, acc = 0.0f;
    const uint32_t n = min(min(count, 64u), e.count);
    for (uint32_t i = 0; i < n; ++i) {
        if (acc >= 0.999f) break;
        const float* c = reinterpret_cast<const float*>(e.caps + 112ull * i);
        const float4 pr = __ldg(reinterpret_cast<const float4*>(c));
        const float4 et = __ldg(reinterpret_cast<const float4*>(c + 4));
        float m[16];
#pragma unroll
        for (int k = 0; k < 16; ++k) m[k] = __ldg(c + 8 + k);
        const int layer = __ldg(reinterpret_cast<const int*>(c + 24));
        const uint32_t shape = __ldg(reinterpret_cast<const uint32_t*>(c + 25));
        const float brightness = __ldg(c + 27);
        if (layer < 0) continue;  // no cubemap resident
        if (uint32_t(layer) >= e.layers) {
            raise_status(status, HL_ERR_DEVICE_BOUNDS);
            continue;
        }
        float w;
        if (shape == 1u) {  // box: the distance inside the nearest pair of faces over the transition
            const float lx = mrow(m, 0, Px, Py, Pz, 1.0f), ly = mrow(m, 1, Px, Py, Pz, 1.0f),
                        lz = mrow(m, 2, Px, Py, Pz, 1.0f);
            const float gx = et.x - fabsf(lx), gy = et.y - fabsf(ly), gz = et.z - fabsf(lz);
            w = (gx < 0.0f || gy < 0.0f || gz < 0.0f)
                    ? 0.0f
                    : fminf(fmaxf(fminf(fminf(gx, gy), gz) / fmaxf(et.w, 1e-4f), 0.0f), 1.0f);
        } else {  // sphere: fade over the outer 10 % of the radius
            const float ox = Px - pr.x, oy = Py - pr.y, oz = Pz - pr.z;
            const float dist = sqrtf(ox * ox + oy * oy + oz * oz);
            w = dist > pr.w ? 0.0f : fminf(fmaxf((pr.w - dist) / fmaxf(pr.w * 0.1f, 1e-4f), 0.0f), 1.0f);
        }
        if (w <= 0.0f) continue;
        float dx = Rx, dy = Ry, dz = Rz;
        if (shape == 1u) {
            const float plx = mrow(m, 0, Px, Py, Pz, 1.0f), ply = mrow(m, 1, Px, Py, Pz, 1.0f),
                        plz = mrow(m, 2, Px, Py, Pz, 1.0f);
            const float rlx = mrow(m, 0, Rx, Ry, Rz, 0.0f), rly = mrow(m, 1, Rx, Ry, Rz, 0.0f),
                        rlz = mrow(m, 2, Rx, Ry, Rz, 0.0f);
            const float ix = 1.0f / rlx, iy = 1.0f / rly, iz = 1.0f / rlz;
            const float tx = fmaxf((-et.x - plx) * ix, (et.x - plx) * ix);
            const float ty = fmaxf((-et.y - ply) * iy, (et.y - ply) * iy);
            const float tz = fmaxf((-et.z - plz) * iz, (et.z - plz) * iz);
            const float t = fminf(fminf(tx, ty), tz);
            if (t > 0.0f && t < 3.402823e38f) {
                dx = (Px + Rx * t) - pr.x;
                dy = (Py + Ry * t) - pr.y;
                dz = (Pz + Rz * t) - pr.z;
            }
        } else {
            const float ox = Px - pr.x, oy = Py - pr.y, oz = Pz - pr.z;
            const float bb = ox * Rx + oy * Ry + oz * Rz;
            const float cc = (ox * ox + oy * oy + oz * oz) - pr.w * pr.w;
            const float disc = bb * bb - cc;
            if (disc >= 0.0f) {
                const float t = -bb + sqrtf(disc);
                if (t > 0.0f) {
                    dx = (Px + Rx * t) - pr.x;
                    dy = (Py + Ry * t) - pr.y;
                    dz = (Pz + Rz * t) - pr.z;
                }
            }
        }
        float sr, sg, sb;
        cube_sample(e, dx, dy, dz, uint32_t(layer), level, sr, sg, sb);
        const float contrib = w * (1.0f - acc);
        ar += sr * brightness * contrib;
        ag += sg * brightness * contrib;
        ab += sb * brightness * contrib;
        acc += contrib;
    }
    if (acc < 0.999f) {  // layer 0 as the skylight, along R
        float sr, sg, sb;
        cube_sample(e, Rx, Ry, Rz, 0u, level, sr, sg, sb);
        ar += sr * (1.0f - acc);
        ag += sg * (1.0f - acc);
        ab += sb * (1.0f - acc);
    }
    return make_float3(ar, ag, ab);
}

__device__ __forceinline__ float smoothstep_(float lo, float hi, float x) {
    const float t = fminf(fmaxf((x - lo) / (hi - lo), 0.0f), 1.0f);
    return t * t * (3.0f - 2.0f * t);
}

// Every load a pixel needs (G-buffer texel, hit images, lightmap UV, target texel) is
// issued before the first branch on its values, so a thread has them all in flight at
// once; the pass is bound by that latency, not by bandwidth.
template <uint32_t LAYOUT, uint32_t TARGET>
__global__ void __launch_bounds__(kRefThreadsX* kRefThreadsY, 3)
    reflect_kernel(const __grid_constant__ ReflectParams p) {
    const uint32_t x = blockIdx.x * kRefThreadsX + threadIdx.x, y = blockIdx.y * kRefThreadsY + threadIdx.y;
    if (x >= p.gb.width || y >= p.gb.height) return;
    const gbuf::Texel<LAYOUT> t = gbuf::load_texel<LAYOUT>(p.gb, x, y);
    const float4 ssr = p.ssr ? load_h4(p.ssr + p.ssr_pitch * y + 8ull * x) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 pl = p.planar ? load_h4(p.planar + p.planar_pitch * y + 8ull * x) : make_float4(0.f, 0.f, 0.f, 0.f);
    // no image: the G-buffer's (-1, -1) no-lightmap sentinel
    const float lmu =
        p.lmuv ? __half2float(__ldg(reinterpret_cast<const __half*>(p.lmuv + p.lmuv_pitch * y + 4ull * x))) : -1.0f;
    unsigned char* o = p.out.data + p.out.pitch * y + (TARGET == HL_TARGET_RGBA32F ? 16ull : 8ull) * x;
    const TargetTexel<TARGET> dst = load_target<TARGET>(o);
    const DeferredGlobals* glb = p.globals;
    const uint32_t dm = __ldg(&glb->debug_mode);
    const bool refl_on = __ldg(&glb->enable_reflections) != 0u;
    const bool rc_on = __ldg(&glb->has_rc_gi) > 0u;
    if (!(t.depth < 1.0f)) return;  // :1268
    if (dm == 30u || dm == 31u) {   // :1271-1276, the replacement pipeline
        const float one = 1.0f;
        if (dm == 30u)
            store_target<TARGET>(o, dst, ssr.w, ssr.w, ssr.w, &one);
        else
            store_target<TARGET>(o, dst, ssr.x, ssr.y, ssr.z, &one);
        return;
    }
    if (dm == 1u || dm == 2u || dm == 4u || dm == 5u || dm == 10u || dm == 11u || dm == 20u || dm == 21u) return;
    const float rough = t.rough;
    const bool want_rc = rc_on && rough > 0.6f;
    const bool use_ssr = refl_on && ssr.w > 0.0f, use_pl = refl_on && pl.w > 0.0f;
    const bool use_env = p.env.caps != nullptr && refl_on && __ldg(&glb->enable_env_reflections) != 0u;
    if (!use_ssr && !use_pl && !want_rc && !use_env) return;  // nothing to add: the target keeps its bits

    // N, F0 (:1287-1295); lightmap sentinel (:1300-1303)
    const float nn = sqrtf(t.nx * t.nx + t.ny * t.ny + t.nz * t.nz);
    const float Nx = t.nx / nn, Ny = t.ny / nn, Nz = t.nz / nn;
    const float f0[3] = {fminf(fmaxf(t.f0r, 0.0f), 0.999f), fminf(fmaxf(t.f0g, 0.0f), 0.999f),
                         fminf(fmaxf(t.f0b, 0.0f), 0.999f)};
    const bool has_lightmap = !(lmu < -1.5f) && lmu >= 0.0f;

    // World position (:1305-1307) as a double-float without the row renormalisation
    // (~4e-10 relative at far depth); V (:1308) from camera - P with the low word folded
    // in, normalised in f32: F_ibl and R need V to f32 accuracy only.
    const GpuCamera* cam = p.camera;
    float Px, Py, Pz, Plx, Ply, Plz;
    reconstruct<true, false>(cam->inv_view_proj, x, y, float(p.gb.width), float(p.gb.height), t.depth, Px, Py, Pz,
                             Plx, Ply, Plz);
    float Vx = (cam->position_near[0] - Px) - Plx, Vy = (cam->position_near[1] - Py) - Ply,
          Vz = (cam->position_near[2] - Pz) - Plz;
    const float vn = sqrtf(Vx * Vx + Vy * Vy + Vz * Vz);
    Vx /= vn;
    Vy /= vn;
    Vz /= vn;
    const float nv = Nx * Vx + Ny * Vy + Nz * Vz;
    const float ndv = fmaxf(nv, 0.0f);
    const float c = fminf(fmaxf(1.0f - ndv, 0.0f), 1.0f);
    const float p5 = c * c * c * c * c;
    float F[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) F[k] = f0[k] + (fmaxf(1.0f - rough, f0[k]) - f0[k]) * p5;  // pbr_eval.wgsl:63-66

    float spec[3] = {0.0f, 0.0f, 0.0f};  // the environment term under the black fallback cube
    if (use_env) {
        // R = reflect(-V, N) (:1311); spec = env (F0 env_brdf.x + env_brdf.y) (:1313-1318)
        const float Rx = 2.0f * nv * Nx - Vx, Ry = 2.0f * nv * Ny - Vy, Rz = 2.0f * nv * Nz - Vz;
        const float3 env = reflection_environment(p.env, __ldg(&glb->reflection_capture_count), Px + Plx, Py + Ply,
                                                  Pz + Plz, Rx, Ry, Rz, rough * 8.0f, p.status);
        // env_brdf_approx (pbr_eval.wgsl:70-76)
        const float r0 = rough * -1.0f + 1.0f, r1 = rough * -0.0275f + 0.0425f, r2 = rough * -0.572f + 1.04f,
                    r3 = rough * 0.022f - 0.04f;
        const float a004 = fminf(r0 * r0, exp2f(-9.28f * ndv)) * r0 + r1;
        const float bx = -1.04f * a004 + r2, by = 1.04f * a004 + r3;
        spec[0] = env.x * (f0[0] * bx + by);
        spec[1] = env.y * (f0[1] * bx + by);
        spec[2] = env.z * (f0[2] * bx + by);
    }
    if (use_ssr) {
        const float s[3] = {ssr.x, ssr.y, ssr.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) spec[k] = spec[k] * (1.0f - ssr.w) + s[k] * F[k] * ssr.w;
    }
    if (use_pl) {
        const float s[3] = {pl.x, pl.y, pl.z};
#pragma unroll
        for (int k = 0; k < 3; ++k) spec[k] = spec[k] * (1.0f - pl.w) + s[k] * F[k] * pl.w;
    }
    if (want_rc) {
        if (!p.rc.rc) {
            raise_status(p.status, HL_ERR_NOT_SUPPORTED);
            return;
        }
        // R = reflect(-V, N); lookup = normalize(mix(R, N, 0.5 roughness)) (:1311, :946)
        const float Rx = 2.0f * nv * Nx - Vx, Ry = 2.0f * nv * Ny - Vy, Rz = 2.0f * nv * Nz - Vz;
        const float h = rough * 0.5f;
        float lx = Rx * (1.0f - h) + Nx * h, ly = Ry * (1.0f - h) + Ny * h, lz = Rz * (1.0f - h) + Nz * h;
        const float ll = sqrtf(lx * lx + ly * ly + lz * lz);
        lx /= ll;
        ly /= ll;
        lz /= ll;
        float ir, ig, ib;
        rc::irradiance(p.rc, glb, Px + Plx, Py + Ply, Pz + Plz, lx, ly, lz, ir, ig, ib);
        const float w = smoothstep_(0.6f, 0.9f, rough) * 0.4f;
        spec[0] = spec[0] * (1.0f - w) + ir * w;
        spec[1] = spec[1] * (1.0f - w) + ig * w;
        spec[2] = spec[2] * (1.0f - w) + ib * w;
    }
    const float ao = has_lightmap ? 1.0f : t.ao;  // orm.r times the white SSAO fallback (:1297)
    store_target<TARGET>(o, dst, dst.v.x + spec[0] * ao, dst.v.y + spec[1] * ao, dst.v.z + spec[2] * ao, nullptr);
}

template <uint32_t LAYOUT>
cudaError_t launch_layout(uint32_t target, const ReflectParams& p, cudaStream_t stream) {
    const dim3 block(kRefThreadsX, kRefThreadsY);
    const dim3 grid((p.gb.width + kRefThreadsX - 1) / kRefThreadsX, (p.gb.height + kRefThreadsY - 1) / kRefThreadsY);
    if (target == HL_TARGET_RGBA32F)
        reflect_kernel<LAYOUT, HL_TARGET_RGBA32F><<<grid, block, 0, stream>>>(p);
    else
        reflect_kernel<LAYOUT, HL_TARGET_RGBA16F><<<grid, block, 0, stream>>>(p);
    return cudaGetLastError();
}

}  // namespace
}  // namespace hl

using namespace hl_host;

extern "C" hl_status hl_shade_reflections(hl_ctx* ctx, const void* camera, const void* globals,
                                          const hl_gbuffer* gbuffer, const hl_reflection_inputs* inputs,
                                          const hl_target* radiance, void* stream) {
    hl_status s = check_common(ctx, camera, nullptr, 0);
    if (s != HL_OK) return s;
    if (!globals || !aligned(globals, 16)) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "globals is NULL or misaligned");
    hl::ReflectParams p;
    std::memset(&p, 0, sizeof p);
    if ((s = check_gbuffer(ctx, gbuffer, p.gb)) != HL_OK) return s;
    if ((s = check_target(ctx, radiance, gbuffer->width, p.out)) != HL_OK) return s;
    const uint32_t W = gbuffer->width;
    if (inputs) {
        struct Img {
            const void* data;
            uint64_t pitch;
            uint32_t bpp;
            const char* name;
        } imgs[3] = {{inputs->ssr, inputs->ssr_pitch, 8, "ssr"},
                     {inputs->planar, inputs->planar_pitch, 8, "planar"},
                     {inputs->lightmap_uv, inputs->lightmap_uv_pitch, 4, "lightmap_uv"}};
        for (const Img& im : imgs) {
            if (!im.data) continue;
            if (!aligned(im.data, im.bpp) || im.pitch % im.bpp != 0)
                return fail(ctx, HL_ERR_LAYOUT, "%s image pointer/pitch not %u-byte aligned", im.name, im.bpp);
            if (im.pitch < uint64_t(W) * im.bpp)
                return fail(ctx, HL_ERR_LAYOUT, "%s image pitch %llu < %u x %u bytes", im.name,
                            (unsigned long long)im.pitch, W, im.bpp);
        }
        p.ssr = static_cast<const unsigned char*>(inputs->ssr);
        p.ssr_pitch = inputs->ssr_pitch;
        p.planar = static_cast<const unsigned char*>(inputs->planar);
        p.planar_pitch = inputs->planar_pitch;
        p.lmuv = static_cast<const unsigned char*>(inputs->lightmap_uv);
        p.lmuv_pitch = inputs->lightmap_uv_pitch;
        if (const hl_rc_cascade* rc = inputs->rc) {
            const uint32_t need_w = HL_RC_PROBE_DIM * HL_RC_DIR_DIM,
                           need_h = HL_RC_PROBE_DIM * HL_RC_PROBE_DIM * HL_RC_DIR_DIM;
            if (!rc->texels) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "rc cascade texels are NULL");
            if (!aligned(rc->texels, 16) || rc->pitch % 16 != 0)
                return fail(ctx, HL_ERR_LAYOUT, "rc cascade pointer/pitch not 16-byte aligned");
            if (rc->width < need_w || rc->height < need_h || rc->pitch < uint64_t(rc->width) * 8)
                return fail(ctx, HL_ERR_SIZE, "rc cascade is %ux%u (pitch %llu), needs at least %ux%u", rc->width,
                            rc->height, (unsigned long long)rc->pitch, need_w, need_h);
            p.rc.rc = static_cast<const unsigned char*>(rc->texels);
            p.rc.rc_pitch = rc->pitch;
        }
        if (const hl_reflection_env* env = inputs->env) {
            if (!env->captures || !env->texels)
                return fail(ctx, HL_ERR_INVALID_ARGUMENT, "reflection env: captures or texels NULL");
            if (!aligned(env->captures, 16) || !aligned(env->texels, 8))
                return fail(ctx, HL_ERR_LAYOUT, "reflection env: captures need 16-byte, texels 8-byte alignment");
            if (env->face_size == 0 || env->face_size > 16384 || env->mip_levels == 0 || env->mip_levels > 15 ||
                env->layers == 0 || env->layers > 65536)
                return fail(ctx, HL_ERR_SIZE, "reflection env: face %u, %u levels, %u layers", env->face_size,
                            env->mip_levels, env->layers);
            uint64_t chain = 0;
            for (uint32_t m = 0; m < env->mip_levels; ++m) {
                const uint64_t n = std::max<uint64_t>(1, env->face_size >> m);
                chain += n * n;
            }
            p.env.caps = static_cast<const unsigned char*>(env->captures);
            p.env.texels = static_cast<const unsigned char*>(env->texels);
            p.env.count = env->count;
            p.env.size = env->face_size;
            p.env.levels = env->mip_levels;
            p.env.layers = env->layers;
            p.env.chain = chain;
        }
    }
    p.camera = static_cast<const hl::GpuCamera*>(camera);
    p.globals = static_cast<const hl::DeferredGlobals*>(globals);
    p.status = ctx->d_status;
    p.rc.status = ctx->d_status;

    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    cudaError_t e;
    switch (gbuffer->layout) {
        case HL_GBUF_REFERENCE: e = hl::launch_layout<HL_GBUF_REFERENCE>(radiance->format, p, as_stream(stream)); break;
        case HL_GBUF_F32: e = hl::launch_layout<HL_GBUF_F32>(radiance->format, p, as_stream(stream)); break;
        default: e = hl::launch_layout<HL_GBUF_F16>(radiance->format, p, as_stream(stream)); break;
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "reflection launch");
    return HL_OK;
}
