// hl_adjoint.cu — adjoint of deferred lighting for sm_103a: the gradient of
// sum(w * radiance) with respect to the lights (position, intensity, colour) and to the
// per-pixel material (albedo, roughness, metallic), for the radiance hl_shade computes.
//
// Forward values are recomputed, nothing per pair is stored. The gradient is
// deterministic: every sum is taken in an order fixed by the launch shape alone.
//  * adjoint_kernel: a persistent grid; CTA g takes 16x8-pixel tiles g, g+G, g+2G, ...
//    Each warp owns an 8x4 block; its lanes set their pixels up (precise path) and walk
//    their own lights lists in a warp-wide merge: each step takes the smallest light
//    index at the head of any lane's list, the lanes holding it evaluate the pair's
//    adjoint, and the warp sums the seven light gradients by a fixed butterfly into the
//    warp's own shared-memory accumulator for that light. Pixel gradients stay in the
//    lane, in list order. Lights are taken in windows of 256 (shared-memory table and
//    accumulators); after a window the CTA adds its warps in order and stores one f32
//    partial per light.
//  * reduce_kernel: one warp per light sums the G partials in f64, lane k taking CTAs
//    k, k+32, ..., then a fixed shuffle tree.
#include "hl_common.cuh"
#include "hl_internal.h"
#include "hl_shade_math.cuh"
#include "hl_texel.cuh"

namespace hl {

namespace {

using namespace sm;
using gbuf::Texel;
using gbuf::load_texel;

constexpr int kThreads = 128;
constexpr int kWarps = kThreads / 32;
constexpr int kWin = 256;   // lights per window
constexpr int kTW = 16, kTH = 8;
constexpr int kComps = 8;   // 7 light gradient components, padded

struct AdjSmem {
    float acc[kWarps][kWin][kComps];
    ShadeLight light[kWin];
    float tab[kMaxSlices + 1];
};

// Sums v[0..7] over the warp. Returns, in every lane, the total of component
// ((lane >> 4) & 1) * 4 + ((lane >> 3) & 1) * 2 + ((lane >> 2) & 1): 9 shuffles.
__device__ __forceinline__ float warp_sum8(float (&v)[kComps], uint32_t lane) {
    const unsigned full = 0xffffffffu;
    const bool b4 = lane & 16u, b3 = lane & 8u, b2 = lane & 4u;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const float send = b4 ? v[i] : v[i + 4], keep = b4 ? v[i + 4] : v[i];
        v[i] = keep + __shfl_xor_sync(full, send, 16);
    }
#pragma unroll
    for (int i = 0; i < 2; ++i) {
        const float send = b3 ? v[i] : v[i + 2], keep = b3 ? v[i + 2] : v[i];
        v[i] = keep + __shfl_xor_sync(full, send, 8);
    }
    {
        const float send = b2 ? v[0] : v[1], keep = b2 ? v[1] : v[0];
        v[0] = keep + __shfl_xor_sync(full, send, 4);
    }
    v[0] += __shfl_xor_sync(full, v[0], 2);
    v[0] += __shfl_xor_sync(full, v[0], 1);
    return v[0];
}

__device__ __forceinline__ ShadeLight load_shade_light(const GpuLight* lights, uint32_t i) {
    const float4* g = reinterpret_cast<const float4*>(lights + i);
    const float4 a = __ldg(g + 0), b = __ldg(g + 1), c = __ldg(g + 2);
    const uint4 d = __ldg(reinterpret_cast<const uint4*>(g + 3));
    ShadeLight l;
    l.px = a.x; l.py = a.y; l.pz = a.z; l.range = a.w;
    l.dx = b.x; l.dy = b.y; l.dz = b.z; l.cos_outer = b.w;
    l.cr = c.x; l.cg = c.y; l.cb = c.z; l.intensity = c.w;
    l.type = d.y;
    l.cos_inner = __uint_as_float(d.z);
    return l;
}

// First position in list[lo, hi) whose entry is >= key (the list is ascending).
__device__ __forceinline__ uint32_t lower_bound(const uint32_t* list, uint32_t lo, uint32_t hi, uint32_t key) {
    while (lo < hi) {
        const uint32_t mid = lo + (hi - lo) / 2;
        if (__ldg(list + mid) < key) lo = mid + 1; else hi = mid;
    }
    return lo;
}

template <uint32_t LAYOUT, uint32_t GRID>
__global__ void __launch_bounds__(kThreads, 4) adjoint_kernel(
    const GpuCamera* __restrict__ cam, const DeferredGlobals* __restrict__ glb, const GBufView gb,
    const GpuLight* __restrict__ lights, uint32_t n_lights, const GridView grid, const __grid_constant__ SliceTable tab,
    const unsigned char* __restrict__ d_rad, uint64_t d_rad_pitch, float* __restrict__ part,
    float* __restrict__ d_pix, int* __restrict__ status) {
    constexpr bool FROXELS = (GRID == HL_GRID_FROXELS);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    AdjSmem& s = *reinterpret_cast<AdjSmem*>(smem_raw);
    const uint32_t t = threadIdx.x, lane = t & 31u, warp = t >> 5;
    const uint32_t tiles_x = (gb.width + kTW - 1) / kTW, tiles_y = (gb.height + kTH - 1) / kTH;
    const uint32_t n_tiles = tiles_x * tiles_y;
    const float W = float(gb.width), H = float(gb.height);
    const float camx = cam->position_near[0], camy = cam->position_near[1], camz = cam->position_near[2];
    const float nr = cam->position_near[3], fr = cam->forward_far[3];
    const float amb = glb->ambient_intensity;
    const float sky[3] = {glb->ambient_color[0] * amb, glb->ambient_color[1] * amb, glb->ambient_color[2] * amb};
    if (t == 0 && blockIdx.x == 0 && (glb->has_rc_gi != 0u || glb->debug_mode != 0u))
        raise_status(status, HL_ERR_NOT_SUPPORTED);
    if (FROXELS)
        for (uint32_t k = t; k <= grid.fp.grid_z; k += kThreads) s.tab[k] = tab.z[k];
    // the warp's 8x4 block inside the 16x8 tile
    const uint32_t px_in_tile_x = (warp & 1u) * 8u + (lane & 7u), px_in_tile_y = (warp >> 1) * 4u + (lane >> 3);

    // windows of kWin lights; one (empty) window when there are none, for the ambient term
#pragma unroll 1
    for (uint32_t wlo = 0;; wlo += kWin) {
        const uint32_t whi = min(n_lights, wlo + kWin);
        __syncthreads();  // the previous window's partials are read out
        for (uint32_t k = t; k < whi - wlo; k += kThreads) s.light[k] = load_shade_light(lights, wlo + k);
        float* accf = &s.acc[0][0][0];
        for (uint32_t k = t; k < uint32_t(kWarps * kWin * kComps); k += kThreads) accf[k] = 0.0f;
        __syncthreads();

#pragma unroll 1
        for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
            const uint32_t x = (tile % tiles_x) * kTW + px_in_tile_x, y = (tile / tiles_x) * kTH + px_in_tile_y;
            bool valid = false;
            Pixel p;
            PixelBrdf pb;
            float ao = 1.0f;
            float wr = 0.0f, wg = 0.0f, wb = 0.0f;
            uint32_t cur = 0, end = 0;
            const uint32_t* list = grid.lists;
            bool f0_from_albedo = true;
            if (x < gb.width && y < gb.height) {
                const Texel<LAYOUT> tx = load_texel<LAYOUT>(gb, x, y);
                valid = tx.depth < 1.0f;
                if (valid) {
                    reconstruct<true>(cam->inv_view_proj, x, y, W, H, tx.depth, p.Px, p.Py, p.Pz, p.Plx, p.Ply, p.Plz);
                    finish_pixel<true>(p, tx.nx, tx.ny, tx.nz, tx.ar, tx.ag, tx.ab, tx.rough, tx.metal, tx.f0r,
                                       tx.f0g, tx.f0b, camx, camy, camz);
                    pb = pixel_brdf(p);
                    ao = tx.ao;
                    f0_from_albedo = (LAYOUT != HL_GBUF_REFERENCE);
                    const float4 w = *reinterpret_cast<const float4*>(d_rad + d_rad_pitch * y + 16ull * x);
                    wr = w.x;
                    wg = w.y;
                    wb = w.z;
                    if (FROXELS) {
                        const float dv = div_(nr * fr, fma_(-tx.depth, fr - nr, fr));
                        const hl_froxel_params& fp = grid.fp;
                        uint32_t sl = 0;
                        for (uint32_t step = 64; step > 0; step >>= 1)
                            if (sl + step < fp.grid_z && s.tab[sl + step] <= dv) sl += step;
                        const uint32_t fx = (x * fp.grid_x) / fp.width, fy = (y * fp.grid_y) / fp.height;
                        const uint32_t f = (fy * fp.grid_x + fx) * fp.grid_z + sl;
                        cur = __ldg(grid.counts + f);
                        end = __ldg(grid.counts + f + 1);
                        if (!(cur <= end && end <= grid.lists_capacity)) {
                            raise_status(status, HL_ERR_DEVICE_BOUNDS);
                            cur = end = 0;
                        }
                    } else {
                        const uint32_t tl = (y / 16u) * glb->num_tiles_x + x / 16u;
                        if (tl < grid.tiles) {
                            uint32_t c = __ldg(grid.counts + tl);
                            if (c > kMaxPerTile) {
                                raise_status(status, HL_ERR_DEVICE_BOUNDS);
                                c = kMaxPerTile;
                            }
                            cur = tl * kMaxPerTile;
                            end = cur + c;
                        } else {
                            raise_status(status, HL_ERR_DEVICE_BOUNDS);
                        }
                    }
                    if (wlo > 0) cur = lower_bound(list, cur, end, wlo);
                }
            }
            float gp[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
            // a lane's walk of this window ends at its list's end or at an entry outside
            // [wlo, whi) (lists are ascending; the range check keeps unsorted input in bounds)
            uint32_t head = (cur < end) ? __ldg(list + cur) : 0xFFFFFFFFu;
            if (head < wlo || head >= whi) head = 0xFFFFFFFFu;
            float (*acc)[kComps] = s.acc[warp];
#pragma unroll 1
            while (true) {
                const uint32_t m = __reduce_min_sync(0xffffffffu, head);
                if (m == 0xFFFFFFFFu) break;
                float g[kComps] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
                bool lit = false;
                if (head == m) {
                    ++cur;
                    head = (cur < end) ? __ldg(list + cur) : 0xFFFFFFFFu;
                    if (head < wlo || head >= whi) head = 0xFFFFFFFFu;
                    const ShadeLight l = s.light[m - wlo];
                    lit = eval_adjoint<true>(p, pb, l, wr, wg, wb, f0_from_albedo, g, gp);
                }
                if (__any_sync(0xffffffffu, lit)) {
                    const float v = warp_sum8(g, lane);
                    const uint32_t c = ((lane >> 4) & 1u) * 4u + ((lane >> 3) & 1u) * 2u + ((lane >> 2) & 1u);
                    if ((lane & 3u) == 0u && c < 7u) acc[m - wlo][c] += v;
                }
            }
            if (valid) {
                float* o = d_pix + (size_t(y) * gb.width + x) * 5;
                if (wlo == 0) {
                    // hemisphere ambient times ao (deferred_lighting.wgsl:1196-1199) depends on albedo
                    const float ht = fma_(p.Ny, 0.5f, 0.5f);
                    const float wc[3] = {wr, wg, wb};
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        gp[c] += wc[c] * fma_(sky[c], ht, sky[c] * 0.15f * (1.0f - ht)) * ao;
#pragma unroll
                    for (int c = 0; c < 5; ++c) o[c] = gp[c];
                } else {
#pragma unroll
                    for (int c = 0; c < 5; ++c) o[c] += gp[c];
                }
            } else if (wlo == 0 && x < gb.width && y < gb.height) {
                float* o = d_pix + (size_t(y) * gb.width + x) * 5;
#pragma unroll
                for (int c = 0; c < 5; ++c) o[c] = 0.0f;
            }
        }
        __syncthreads();
        // the CTA's partial for this window: warps added in order
        for (uint32_t k = t; k < whi - wlo; k += kThreads) {
            float v[kComps];
#pragma unroll
            for (int c = 0; c < kComps; ++c) v[c] = ((s.acc[0][k][c] + s.acc[1][k][c]) + s.acc[2][k][c]) + s.acc[3][k][c];
            float4* dst = reinterpret_cast<float4*>(part + (size_t(blockIdx.x) * n_lights + wlo + k) * kComps);
            dst[0] = make_float4(v[0], v[1], v[2], v[3]);
            dst[1] = make_float4(v[4], v[5], v[6], 0.0f);
        }
        if (whi >= n_lights) break;
    }
}

// d_lights[l*7 + c] = sum over CTAs g = 0..G-1 of part[g][l][c], in f64.
__global__ void __launch_bounds__(256) reduce_kernel(const float* __restrict__ part, uint32_t G, uint32_t n,
                                                     double* __restrict__ d_lights) {
    const uint32_t lane = threadIdx.x & 31u;
    const uint32_t l = blockIdx.x * (blockDim.x / 32u) + threadIdx.x / 32u;
    if (l >= n) return;
    double acc[7] = {0, 0, 0, 0, 0, 0, 0};
    for (uint32_t g = lane; g < G; g += 32u) {
        const float4* src = reinterpret_cast<const float4*>(part + (size_t(g) * n + l) * kComps);
        const float4 a = __ldg(src), b = __ldg(src + 1);
        acc[0] += double(a.x);
        acc[1] += double(a.y);
        acc[2] += double(a.z);
        acc[3] += double(a.w);
        acc[4] += double(b.x);
        acc[5] += double(b.y);
        acc[6] += double(b.z);
    }
#pragma unroll
    for (int c = 0; c < 7; ++c)
        for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
    if (lane < 7u) {
        double v = acc[0];
#pragma unroll
        for (int c = 1; c < 7; ++c) v = (lane == uint32_t(c)) ? acc[c] : v;
        d_lights[size_t(l) * 7 + lane] = v;
    }
}

int g_grid_size[64] = {};  // persistent grid size per device (0 = not yet queried)

template <uint32_t LAYOUT, uint32_t GRID>
cudaError_t launch_adjoint_t(const void* camera, const void* globals, const GBufView& gb, const void* lights,
                             uint32_t n, const GridView& grid, const SliceTable& tab, const unsigned char* d_rad,
                             uint64_t d_rad_pitch, float* part, uint32_t G, double* d_lights, float* d_pix,
                             int* status, cudaStream_t stream) {
    auto k = adjoint_kernel<LAYOUT, GRID>;
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(AdjSmem)));
    if (e != cudaSuccess) return e;
    k<<<G, kThreads, sizeof(AdjSmem), stream>>>(static_cast<const GpuCamera*>(camera),
                                                static_cast<const DeferredGlobals*>(globals), gb,
                                                static_cast<const GpuLight*>(lights), n, grid, tab, d_rad,
                                                d_rad_pitch, part, d_pix, status);
    e = cudaGetLastError();
    if (e != cudaSuccess || n == 0) return e;
    reduce_kernel<<<(n + 7) / 8, 256, 0, stream>>>(part, G, n, d_lights);
    return cudaGetLastError();
}

template <uint32_t LAYOUT>
cudaError_t dispatch_adjoint(uint32_t grid_kind, const void* camera, const void* globals, const GBufView& gb,
                             const void* lights, uint32_t n, const GridView& grid, const SliceTable& tab,
                             const unsigned char* d_rad, uint64_t pitch, float* part, uint32_t G, double* d_lights,
                             float* d_pix, int* status, cudaStream_t stream) {
    if (grid_kind == HL_GRID_FROXELS)
        return launch_adjoint_t<LAYOUT, HL_GRID_FROXELS>(camera, globals, gb, lights, n, grid, tab, d_rad, pitch, part,
                                                         G, d_lights, d_pix, status, stream);
    return launch_adjoint_t<LAYOUT, HL_GRID_TILES>(camera, globals, gb, lights, n, grid, tab, d_rad, pitch, part, G,
                                                   d_lights, d_pix, status, stream);
}

}  // namespace

uint32_t adjoint_grid_size(int device, uint32_t width, uint32_t height) {
    const uint32_t tiles = ((width + kTW - 1) / kTW) * ((height + kTH - 1) / kTH);
    int g = (device >= 0 && device < 64) ? g_grid_size[device] : 0;
    if (g == 0) {
        int sms = 0, per_sm = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) sms = 1;
        auto k = adjoint_kernel<HL_GBUF_F32, HL_GRID_FROXELS>;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, int(sizeof(AdjSmem))) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, sizeof(AdjSmem)) != cudaSuccess ||
            per_sm < 1)
            per_sm = 1;
        cudaGetLastError();
        g = sms * per_sm;
        if (device >= 0 && device < 64) g_grid_size[device] = g;
    }
    return tiles < uint32_t(g) ? tiles : uint32_t(g);
}

cudaError_t launch_shade_adjoint(uint32_t layout, uint32_t grid_kind, const void* camera, const void* globals,
                                 const GBufView& gb, const void* lights, uint32_t n_lights, const GridView& grid,
                                 const SliceTable& tab, const void* d_radiance, uint64_t d_radiance_pitch,
                                 float* partials, uint32_t grid_size, double* d_lights, float* d_pixels, int* status,
                                 cudaStream_t stream) {
    const unsigned char* dr = static_cast<const unsigned char*>(d_radiance);
    switch (layout) {
        case HL_GBUF_REFERENCE:
            return dispatch_adjoint<HL_GBUF_REFERENCE>(grid_kind, camera, globals, gb, lights, n_lights, grid, tab, dr,
                                                       d_radiance_pitch, partials, grid_size, d_lights, d_pixels,
                                                       status, stream);
        case HL_GBUF_F32:
            return dispatch_adjoint<HL_GBUF_F32>(grid_kind, camera, globals, gb, lights, n_lights, grid, tab, dr,
                                                 d_radiance_pitch, partials, grid_size, d_lights, d_pixels, status,
                                                 stream);
        default:
            return dispatch_adjoint<HL_GBUF_F16>(grid_kind, camera, globals, gb, lights, n_lights, grid, tab, dr,
                                                 d_radiance_pitch, partials, grid_size, d_lights, d_pixels, status,
                                                 stream);
    }
}

}  // namespace hl
