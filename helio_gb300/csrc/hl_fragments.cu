// hl_fragments.cu — light loops of the fragment shaders that read the same light
// lists as the deferred pass: Forward+ (forward_lit.wgsl:443-494) and transparent
// surfaces (transparent_base.wgsl:181-220), for fragments given as hl_fragment records.
//
//  * prep_frag_lights: one thread per light builds its shading record; in the forward
//    mode with entity indices, position and direction come from the scene's Transform
//    of that entity (direction = Euler Y X Z rotation applied to -Z,
//    forward_lit.wgsl:333-383), as the Forward+ shader reads them.
//  * shade_fragments: one thread per fragment, set up on the precise path (world
//    position, compensated NdV), walks its tile or froxel list in list order and sums
//    pbr_direct_light with compensated (Kahan) sums. Fragments arrive in raster order,
//    so the lanes of a warp mostly share a list.
#include "hl_common.cuh"
#include "hl_internal.h"
#include "hl_shade_math.cuh"

namespace hl {

namespace {

using namespace sm;

struct alignas(16) FragLight {
    float px, py, pz, range;
    float dx, dy, dz, cos_outer;
    float cr, cg, cb, intensity;
    uint32_t type;
    float cos_inner;
    uint32_t usable;
    uint32_t pad;
};
static_assert(sizeof(FragLight) == 64, "FragLight is 64 bytes");

struct Quat {
    float x, y, z, w;
};

__device__ __forceinline__ Quat qmul(Quat a, Quat b) {
    return Quat{a.w * b.x + a.x * b.w + a.y * b.z - a.z * b.y, a.w * b.y - a.x * b.z + a.y * b.w + a.z * b.x,
                a.w * b.z + a.x * b.y - a.y * b.x + a.z * b.w, a.w * b.w - a.x * b.x - a.y * b.y - a.z * b.z};
}

// Direction of a Transform rotation (degrees: pitch x, yaw y, roll z): q = qy qx qz
// applied to (0, 0, -1), as v + w t + q.xyz x t with t = 2 q.xyz x v.
__device__ __forceinline__ void light_dir_from_rotation(const float* rot_deg, float& x, float& y, float& z) {
    const float k = 0.5f * 0.017453292519943295f;
    float sp, cp, sy, cy, sr, cr;
    sincosf(rot_deg[0] * k, &sp, &cp);
    sincosf(rot_deg[1] * k, &sy, &cy);
    sincosf(rot_deg[2] * k, &sr, &cr);
    const Quat q = qmul(qmul(Quat{0.0f, sy, 0.0f, cy}, Quat{sp, 0.0f, 0.0f, cp}), Quat{0.0f, 0.0f, sr, cr});
    // t = 2 (q.xyz x (0,0,-1)) = 2 (-q.y, q.x, 0)
    const float tx = -2.0f * q.y, ty = 2.0f * q.x, tz = 0.0f;
    // v + w t + q.xyz x t
    const float vx = q.w * tx + (q.y * tz - q.z * ty);
    const float vy = q.w * ty + (q.z * tx - q.x * tz);
    const float vz = -1.0f + q.w * tz + (q.x * ty - q.y * tx);
    const float inv = rsqrt_(vx * vx + vy * vy + vz * vz);
    x = vx * inv;
    y = vy * inv;
    z = vz * inv;
}

__global__ void __launch_bounds__(256) prep_frag_lights_kernel(const GpuLight* __restrict__ lights, uint32_t n,
                                                               const uint32_t* __restrict__ entity,
                                                               const float* __restrict__ transforms, uint32_t n_xf,
                                                               FragLight* __restrict__ out, int* __restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const GpuLight& g = lights[i];
    FragLight l;
    l.px = g.position_range[0];
    l.py = g.position_range[1];
    l.pz = g.position_range[2];
    l.range = g.position_range[3];
    l.dx = g.direction_outer[0];
    l.dy = g.direction_outer[1];
    l.dz = g.direction_outer[2];
    l.cos_outer = g.direction_outer[3];
    l.cr = g.color_intensity[0];
    l.cg = g.color_intensity[1];
    l.cb = g.color_intensity[2];
    l.intensity = g.color_intensity[3];
    l.type = g.light_type;
    l.cos_inner = g.inner_angle;
    l.usable = 1u;
    l.pad = 0u;
    if (entity) {
        const uint32_t e = entity[i];
        if (e >= n_xf) {
            l.usable = 0u;
            raise_status(status, HL_ERR_DEVICE_BOUNDS);
        } else {
            const float* t = transforms + size_t(e) * 9;
            l.px = t[0];
            l.py = t[1];
            l.pz = t[2];
            light_dir_from_rotation(t + 3, l.dx, l.dy, l.dz);
        }
    }
    out[i] = l;
}

template <uint32_t MODE, uint32_t GRID>
__global__ void __launch_bounds__(256, 4) shade_fragments_kernel(
    const GpuCamera* __restrict__ cam, const hl_fragment_params prm, const float4* __restrict__ frags, uint32_t n,
    const FragLight* __restrict__ fl, uint32_t n_lights, const GridView grid, const __grid_constant__ SliceTable tab,
    float4* __restrict__ out, int* __restrict__ status) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 f0 = frags[5 * size_t(i) + 0], f1 = frags[5 * size_t(i) + 1], f2 = frags[5 * size_t(i) + 2],
                 f3 = frags[5 * size_t(i) + 3], f4 = frags[5 * size_t(i) + 4];
    const float alpha = f1.w;
    if (MODE == HL_FRAGMENTS_FORWARD && !(alpha > 0.001f)) return;  // discard
    const uint32_t pixel = __float_as_uint(f0.w);
    const uint32_t x = pixel & 0xFFFFu, y = pixel >> 16;
    const float camx = cam->position_near[0], camy = cam->position_near[1], camz = cam->position_near[2];
    Pixel p;
    p.Px = f0.x;
    p.Py = f0.y;
    p.Pz = f0.z;
    p.Plx = p.Ply = p.Plz = 0.0f;
    finish_pixel<true>(p, f1.x, f1.y, f1.z, f2.x, f2.y, f2.z, f2.w, f3.w, f3.x, f3.y, f3.z, camx, camy, camz);
    p.f0r = f3.x;  // the material's F0 as given, not clamped
    p.f0g = f3.y;
    p.f0b = f3.z;
    PixelBrdf b = pixel_brdf(p);
    df_view(p, b, camx, camy, camz);  // V as a double-float unit vector
    uint32_t base = 0, count = 0;
    if (GRID == HL_GRID_TILES) {
        const uint32_t tile = (y / kTile) * prm.num_tiles_x + x / kTile;
        if (tile < grid.tiles) {
            count = __ldg(grid.counts + tile);
            if (count > kMaxPerTile) {
                raise_status(status, HL_ERR_DEVICE_BOUNDS);
                count = kMaxPerTile;
            }
            base = tile * kMaxPerTile;
        } else {
            raise_status(status, HL_ERR_DEVICE_BOUNDS);
        }
    } else {
        const hl_froxel_params& fp = grid.fp;
        const float* v = cam->view;
        const float d = -fma_(v[10], p.Pz, fma_(v[6], p.Py, fma_(v[2], p.Px, v[14])));
        uint32_t sl = 0;
        for (uint32_t step = 64; step > 0; step >>= 1)
            if (sl + step < fp.grid_z && tab.z[sl + step] <= d) sl += step;
        if (x < fp.width && y < fp.height) {
            const uint32_t fx = uint32_t((uint64_t(x) * fp.grid_x) / fp.width);
            const uint32_t fy = uint32_t((uint64_t(y) * fp.grid_y) / fp.height);
            const uint32_t f = (fy * fp.grid_x + fx) * fp.grid_z + sl;
            base = __ldg(grid.counts + f);
            const uint32_t e = __ldg(grid.counts + f + 1);
            if (base <= e && e <= grid.lists_capacity) {
                count = e - base;
            } else {
                raise_status(status, HL_ERR_DEVICE_BOUNDS);
                base = 0;
            }
        } else {
            raise_status(status, HL_ERR_DEVICE_BOUNDS);
        }
    }
    const float cut = MODE == HL_FRAGMENTS_FORWARD ? 0.0f : kRadianceCut;
    float sr = 0.0f, sg = 0.0f, sb = 0.0f, cr = 0.0f, cg = 0.0f, cb = 0.0f;
    for (uint32_t j = 0; j < count; ++j) {
        const uint32_t li = __ldg(grid.lists + base + j);
        if (li >= n_lights) {
            raise_status(status, HL_ERR_DEVICE_BOUNDS);
            continue;
        }
        const float4* r = reinterpret_cast<const float4*>(fl + li);
        const float4 a = __ldg(r), bb = __ldg(r + 1), c = __ldg(r + 2);
        const uint4 t = __ldg(reinterpret_cast<const uint4*>(r + 3));
        if (t.z == 0u) continue;  // entity index out of range
        ShadeLight l;
        l.px = a.x; l.py = a.y; l.pz = a.z; l.range = a.w;
        l.dx = bb.x; l.dy = bb.y; l.dz = bb.z; l.cos_outer = bb.w;
        l.cr = c.x; l.cg = c.y; l.cb = c.z; l.intensity = c.w;
        l.type = t.x;
        l.cos_inner = __uint_as_float(t.y);
        if (!in_range(p, l)) continue;
        float orr, og, ob;
        if (eval<true>(p, b, l, orr, og, ob, 0.0f, cut) == kLit) {
            kahan_add(sr, cr, orr);
            kahan_add(sg, cg, og);
            kahan_add(sb, cb, ob);
        }
    }
    float4 o;
    if (MODE == HL_FRAGMENTS_FORWARD) {
        const float ar = prm.ambient_color[0] * prm.ambient_intensity, ag = prm.ambient_color[1] * prm.ambient_intensity,
                    ab = prm.ambient_color[2] * prm.ambient_intensity;
        o.x = (sr + ar * f2.x * f4.w) + f4.x;
        o.y = (sg + ag * f2.y * f4.w) + f4.y;
        o.z = (sb + ab * f2.z * f4.w) + f4.z;
    } else {
        o.x = f4.x + sr;
        o.y = f4.y + sg;
        o.z = f4.z + sb;
    }
    o.w = alpha;
    out[i] = o;
}

template <uint32_t MODE>
cudaError_t launch_mode(const void* camera, const hl_fragment_params& prm, const void* frags, uint32_t n,
                        const FragLight* fl, uint32_t n_lights, const GridView& grid, const SliceTable& tab,
                        float* out, int* status, uint32_t grid_kind, cudaStream_t stream) {
    const dim3 g((n + 255) / 256);
    const GpuCamera* cam = static_cast<const GpuCamera*>(camera);
    const float4* fr = static_cast<const float4*>(frags);
    float4* o = reinterpret_cast<float4*>(out);
    if (grid_kind == HL_GRID_FROXELS)
        shade_fragments_kernel<MODE, HL_GRID_FROXELS><<<g, 256, 0, stream>>>(cam, prm, fr, n, fl, n_lights, grid, tab, o,
                                                                            status);
    else
        shade_fragments_kernel<MODE, HL_GRID_TILES><<<g, 256, 0, stream>>>(cam, prm, fr, n, fl, n_lights, grid, tab, o,
                                                                          status);
    return cudaGetLastError();
}

}  // namespace

size_t frag_light_bytes() { return sizeof(FragLight); }

cudaError_t launch_shade_fragments(const void* camera, const hl_fragment_params& prm, const void* frags, uint32_t n,
                                   const void* lights, uint32_t n_lights, const uint32_t* entity,
                                   const void* transforms, uint32_t n_xf, uint32_t grid_kind, const GridView& grid,
                                   const SliceTable& tab, void* light_scratch, float* out, int* status,
                                   cudaStream_t stream) {
    FragLight* fl = static_cast<FragLight*>(light_scratch);
    if (n_lights > 0) {
        prep_frag_lights_kernel<<<(n_lights + 255) / 256, 256, 0, stream>>>(
            static_cast<const GpuLight*>(lights), n_lights, entity, static_cast<const float*>(transforms), n_xf, fl,
            status);
        const cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (n == 0) return cudaSuccess;
    if (prm.mode == HL_FRAGMENTS_FORWARD)
        return launch_mode<HL_FRAGMENTS_FORWARD>(camera, prm, frags, n, fl, n_lights, grid, tab, out, status, grid_kind,
                                                 stream);
    return launch_mode<HL_FRAGMENTS_TRANSPARENT>(camera, prm, frags, n, fl, n_lights, grid, tab, out, status,
                                                 grid_kind, stream);
}

}  // namespace hl
