// hl_shade.cu — deferred lighting (fs_main under fallback bindings) for sm_103a.
//
// One thread per pixel, 16x16-pixel CTAs (one reference light-cull tile per CTA).
// Each thread decodes its G-buffer texel, reconstructs the world position, walks its
// tile or froxel light list in list order and accumulates pbr_direct_light in f32
// with Kahan compensation, then adds hemisphere ambient and emissive.
#include "hl_common.cuh"
#include "hl_internal.h"
#include "hl_shade_math.cuh"

namespace hl {

namespace {

using namespace sm;

constexpr int kShadeTile = 16;

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

__device__ __forceinline__ ShadeLight load_light(const GpuLight* __restrict__ lights, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(lights + i);
    const float4 a = __ldg(p + 0), b = __ldg(p + 1), c = __ldg(p + 2);
    const uint4 d = __ldg(reinterpret_cast<const uint4*>(p + 3));
    ShadeLight l;
    l.px = a.x;
    l.py = a.y;
    l.pz = a.z;
    l.range = a.w;
    l.dx = b.x;
    l.dy = b.y;
    l.dz = b.z;
    l.cos_outer = b.w;
    l.cr = c.x;
    l.cg = c.y;
    l.cb = c.z;
    l.intensity = c.w;
    l.type = d.y;
    l.cos_inner = __uint_as_float(d.z);
    return l;
}

template <uint32_t LAYOUT, uint32_t GRID, uint32_t TARGET, bool STATS>
__global__ void __launch_bounds__(kShadeTile* kShadeTile) shade_kernel(
    const GpuCamera* __restrict__ cam, const DeferredGlobals* __restrict__ glb, const GBufView gb,
    const GpuLight* __restrict__ lights, uint32_t n_lights, const GridView grid, const __grid_constant__ SliceTable tab,
    const TargetView out, uint32_t* __restrict__ stats, int* __restrict__ status) {
    constexpr bool PRECISE = (LAYOUT != HL_GBUF_F16);
    __shared__ float s_tab[kMaxSlices + 1];
    if (GRID == HL_GRID_FROXELS) {
        for (uint32_t i = threadIdx.y * kShadeTile + threadIdx.x; i <= grid.fp.grid_z; i += kShadeTile * kShadeTile)
            s_tab[i] = tab.z[i];
        __syncthreads();
    }
    const uint32_t x = blockIdx.x * kShadeTile + threadIdx.x;
    const uint32_t y = blockIdx.y * kShadeTile + threadIdx.y;
    if (x >= gb.width || y >= gb.height) return;

    const Texel<LAYOUT> t = load_texel<LAYOUT>(gb, x, y);
    if (!(t.depth < 1.0f)) {  // sky: the reference discards (deferred_lighting.wgsl:996-997)
        if (STATS) {
            uint32_t* s = stats + (size_t(y) * gb.width + x) * 3;
            s[0] = s[1] = s[2] = 0;
        }
        return;
    }
    const uint32_t debug_mode = glb->debug_mode;
    if (glb->has_rc_gi != 0u || debug_mode == 10u || debug_mode == 11u) raise_status(status, HL_ERR_NOT_SUPPORTED);

    Pixel p;
    reconstruct<PRECISE>(cam->inv_view_proj, x, y, float(gb.width), float(gb.height), t.depth, p.Px, p.Py, p.Pz, p.Plx,
                         p.Ply, p.Plz);
    finish_pixel(p, t.nx, t.ny, t.nz, t.ar, t.ag, t.ab, t.rough, t.metal, t.f0r, t.f0g, t.f0b, cam->position_near[0],
                 cam->position_near[1], cam->position_near[2]);
    const PixelBrdf brdf = pixel_brdf(p);

    // Light list of the pixel.
    const uint32_t* list = nullptr;
    uint32_t count = 0;
    if (GRID == HL_GRID_TILES) {
        const uint32_t tile = (y / kTile) * glb->num_tiles_x + x / kTile;
        if (tile < grid.tiles) {
            count = grid.counts[tile];
            if (count > kMaxPerTile) {
                raise_status(status, HL_ERR_DEVICE_BOUNDS);
                count = kMaxPerTile;
            }
            list = grid.lists + size_t(tile) * kMaxPerTile;
        } else {
            raise_status(status, HL_ERR_DEVICE_BOUNDS);
        }
    } else {
        const float nr = cam->position_near[3], fr = cam->forward_far[3];
        const float d = div_(nr * fr, fma_(-t.depth, fr - nr, fr));
        const hl_froxel_params& fp = grid.fp;
        uint32_t s = 0;
        for (uint32_t step = 64; step > 0; step >>= 1)
            if (s + step < fp.grid_z && s_tab[s + step] <= d) s += step;
        const uint32_t fx = uint32_t((uint64_t(x) * fp.grid_x) / fp.width);
        const uint32_t fy = uint32_t((uint64_t(y) * fp.grid_y) / fp.height);
        const uint32_t f = (fy * fp.grid_x + fx) * fp.grid_z + s;
        const uint32_t b = grid.counts[f], e = grid.counts[f + 1];
        if (b <= e && e <= grid.lists_capacity) {
            list = grid.lists + b;
            count = e - b;
        } else {
            raise_status(status, HL_ERR_DEVICE_BOUNDS);
        }
    }

    float sr = 0.0f, sg = 0.0f, sb = 0.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f;
    uint32_t n_range = 0, n_full = 0;
    for (uint32_t j = 0; j < count; ++j) {
        const uint32_t idx = __ldg(list + j);
        if (idx >= n_lights) {
            raise_status(status, HL_ERR_DEVICE_BOUNDS);
            continue;
        }
        const ShadeLight l = load_light(lights, idx);
        if (STATS && in_range(p, l)) ++n_range;
        float r, g, b;
        if (eval<PRECISE>(p, brdf, l, r, g, b)) {
            kahan_add(sr, cr, r);
            kahan_add(sg, cg, g);
            kahan_add(sb, cb, b);
            ++n_full;
        }
    }
    if (STATS) {
        uint32_t* s = stats + (size_t(y) * gb.width + x) * 3;
        s[0] = count;
        s[1] = n_range;
        s[2] = n_full;
        return;
    }

    // Hemisphere ambient (deferred_lighting.wgsl:1196-1199) times ao (x white SSAO).
    const float amb = glb->ambient_intensity;
    const float skr = glb->ambient_color[0] * amb, skg = glb->ambient_color[1] * amb, skb = glb->ambient_color[2] * amb;
    const float ht = fma_(p.Ny, 0.5f, 0.5f);
    const float hr = fma_(skr, ht, skr * 0.15f * (1.0f - ht)) * t.ar;
    const float hg = fma_(skg, ht, skg * 0.15f * (1.0f - ht)) * t.ag;
    const float hb = fma_(skb, ht, skb * 0.15f * (1.0f - ht)) * t.ab;
    float4 c;
    c.x = (sr + fma_(hr, t.ao, 0.0f)) + t.er;
    c.y = (sg + fma_(hg, t.ao, 0.0f)) + t.eg;
    c.z = (sb + fma_(hb, t.ao, 0.0f)) + t.eb;
    c.w = t.alpha;
    if (debug_mode == 1u || debug_mode == 2u || debug_mode == 4u || debug_mode == 20u || debug_mode == 21u) {
        c = make_float4(t.ar, t.ag, t.ab, t.alpha);
    } else if (debug_mode == 5u) {
        c = make_float4(fma_(p.Nx, 0.5f, 0.5f), fma_(p.Ny, 0.5f, 0.5f), fma_(p.Nz, 0.5f, 0.5f), 1.0f);
    }
    unsigned char* row = out.data + out.pitch * y;
    if (TARGET == HL_TARGET_RGBA32F) {
        reinterpret_cast<float4*>(row)[x] = c;
    } else {
        const __half2 lo = __floats2half2_rn(c.x, c.y), hi = __floats2half2_rn(c.z, c.w);
        uint2 v;
        v.x = *reinterpret_cast<const uint32_t*>(&lo);
        v.y = *reinterpret_cast<const uint32_t*>(&hi);
        reinterpret_cast<uint2*>(row)[x] = v;
    }
}

template <uint32_t LAYOUT, uint32_t GRID, uint32_t TARGET, bool STATS>
cudaError_t launch_one(const void* camera, const void* globals, const GBufView& gb, const void* lights, uint32_t n,
                       const GridView& grid, const SliceTable& tab, const TargetView& out, uint32_t* stats, int* status,
                       cudaStream_t stream) {
    const dim3 block(kShadeTile, kShadeTile);
    const dim3 g((gb.width + kShadeTile - 1) / kShadeTile, (gb.height + kShadeTile - 1) / kShadeTile);
    shade_kernel<LAYOUT, GRID, TARGET, STATS><<<g, block, 0, stream>>>(
        static_cast<const GpuCamera*>(camera), static_cast<const DeferredGlobals*>(globals), gb,
        static_cast<const GpuLight*>(lights), n, grid, tab, out, stats, status);
    return cudaGetLastError();
}

template <uint32_t LAYOUT, uint32_t GRID>
cudaError_t dispatch_target(uint32_t target, const void* camera, const void* globals, const GBufView& gb,
                            const void* lights, uint32_t n, const GridView& grid, const SliceTable& tab,
                            const TargetView& out, uint32_t* stats, int* status, cudaStream_t stream) {
    if (stats) return launch_one<LAYOUT, GRID, HL_TARGET_RGBA32F, true>(camera, globals, gb, lights, n, grid, tab, out, stats, status, stream);
    if (target == HL_TARGET_RGBA16F)
        return launch_one<LAYOUT, GRID, HL_TARGET_RGBA16F, false>(camera, globals, gb, lights, n, grid, tab, out, stats, status, stream);
    return launch_one<LAYOUT, GRID, HL_TARGET_RGBA32F, false>(camera, globals, gb, lights, n, grid, tab, out, stats, status, stream);
}

template <uint32_t LAYOUT>
cudaError_t dispatch_grid(uint32_t grid_kind, uint32_t target, const void* camera, const void* globals,
                          const GBufView& gb, const void* lights, uint32_t n, const GridView& grid,
                          const SliceTable& tab, const TargetView& out, uint32_t* stats, int* status,
                          cudaStream_t stream) {
    if (grid_kind == HL_GRID_FROXELS)
        return dispatch_target<LAYOUT, HL_GRID_FROXELS>(target, camera, globals, gb, lights, n, grid, tab, out, stats, status, stream);
    return dispatch_target<LAYOUT, HL_GRID_TILES>(target, camera, globals, gb, lights, n, grid, tab, out, stats, status, stream);
}

}  // namespace

cudaError_t launch_shade(uint32_t layout, uint32_t grid_kind, uint32_t target_format, const void* camera,
                         const void* globals, const GBufView& gb, const void* lights, uint32_t n_lights,
                         const GridView& grid, const SliceTable& tab, const TargetView& out, uint32_t* stats,
                         int* status, cudaStream_t stream) {
    switch (layout) {
        case HL_GBUF_REFERENCE:
            return dispatch_grid<HL_GBUF_REFERENCE>(grid_kind, target_format, camera, globals, gb, lights, n_lights, grid, tab, out, stats, status, stream);
        case HL_GBUF_F32:
            return dispatch_grid<HL_GBUF_F32>(grid_kind, target_format, camera, globals, gb, lights, n_lights, grid, tab, out, stats, status, stream);
        default:
            return dispatch_grid<HL_GBUF_F16>(grid_kind, target_format, camera, globals, gb, lights, n_lights, grid, tab, out, stats, status, stream);
    }
}

}  // namespace hl
