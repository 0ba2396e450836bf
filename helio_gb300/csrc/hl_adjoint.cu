// hl_adjoint.cu — adjoint of deferred lighting for sm_103a: the gradient of
// sum(w * radiance) with respect to the lights (position, intensity, colour) and to the
// per-pixel material (albedo, roughness, metallic), for the radiance hl_shade computes.
//
// Forward values are recomputed, nothing per pair is stored. The gradient is
// deterministic: every sum is taken in an order fixed by the launch shape alone.
//  * adjoint_kernel: a persistent grid of 256-thread CTAs over 16x16-pixel tiles; warp w
//    of CTA g takes rows 2w and 2w+1 of tiles g, g+G, g+2G, ... Each lane sets its pixel
//    up (precise path) into a shared-memory record, walks its own light list (range and
//    NdL sign tests) and queues the passing (pixel, light) pairs in the warp's ring. The
//    ring is evaluated 32 pairs at a time, one per lane, so the adjoint of
//    pbr_direct_light runs with every lane busy whatever the list lengths. Per batch the
//    first lane holding a light sums that light's pairs in lane order into the warp's
//    accumulator for it, and the first lane holding a pixel does the same for the pixel's
//    gradient. Lights are taken in windows of 256 (shared-memory table and accumulators);
//    after a window the CTA adds its warps in order and stores one f32 partial per light.
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

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kWin = 256;   // lights per window
constexpr int kTW = 16, kTH = 16;
constexpr int kPx = kTW * kTH;
constexpr int kComps = 8;   // 7 light gradient components, padded in the partials
constexpr int kPipe = 2;    // list entries a lane loads ahead
constexpr int kQueue = 128; // per-warp pair ring: at most 31 + 32 kPipe pairs pending
static_assert(kPx == kThreads, "one pixel per thread");
static_assert(31 + 32 * kPipe <= kQueue, "ring too small");

// Pixel record (structure of arrays). N, V, F0 (metallic workflow) and the BRDF constants
// are recomputed from it with finish_pixel's own operations.
enum Field : int {
    F_PX, F_PY, F_PZ, F_PLX, F_PLY, F_PLZ, F_NDV, F_AR, F_AG, F_AB, F_ROUGH, F_METAL, F_NRX, F_NRY, F_NRZ,
    F_WR, F_WG, F_WB,     // dLoss / d radiance
    F_F0R, F_F0G, F_F0B,  // reference layout only
    F_COUNT
};

template <uint32_t LAYOUT>
__host__ __device__ constexpr int record_fields() { return LAYOUT == HL_GBUF_REFERENCE ? int(F_COUNT) : int(F_F0R); }

template <int NF>
struct AdjSmem {
    float acc[kWarps][kWin][7];     // each warp's light gradients of the current window
    ShadeLight light[kWin];
    float rec[NF][kPx];
    float gpx[5][kPx];              // pixel gradients of the current tile
    uint32_t queue[kWarps][kQueue]; // ring of (pixel << 23) | light index
    float gbuf[kWarps][32][12];     // one batch's gradients by lane: 7 light, 5 pixel
    float tab[kMaxSlices + 1];
};

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
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

// The pixel as finish_pixel<true> set it up, from its record.
template <uint32_t LAYOUT, int NF>
__device__ __forceinline__ void load_pixel(const AdjSmem<NF>& s, uint32_t i, Pixel& p, PixelBrdf& b, float camx,
                                           float camy, float camz) {
    p.Px = s.rec[F_PX][i]; p.Py = s.rec[F_PY][i]; p.Pz = s.rec[F_PZ][i];
    p.Plx = s.rec[F_PLX][i]; p.Ply = s.rec[F_PLY][i]; p.Plz = s.rec[F_PLZ][i];
    p.nrx = s.rec[F_NRX][i]; p.nry = s.rec[F_NRY][i]; p.nrz = s.rec[F_NRZ][i];
    p.inv_n = rsqrt_(fma_(p.nrz, p.nrz, fma_(p.nry, p.nry, p.nrx * p.nrx)));
    p.Nx = p.nrx * p.inv_n;
    p.Ny = p.nry * p.inv_n;
    p.Nz = p.nrz * p.inv_n;
    const DF ux = two_sum(camx, -p.Px), uy = two_sum(camy, -p.Py), uz = two_sum(camz, -p.Pz);
    const float vx = two_sum(ux.hi, ux.lo - p.Plx).hi, vy = two_sum(uy.hi, uy.lo - p.Ply).hi,
                vz = two_sum(uz.hi, uz.lo - p.Plz).hi;
    const float iv = rsqrt_(fma_(vz, vz, fma_(vy, vy, vx * vx)));
    p.Vx = vx * iv;
    p.Vy = vy * iv;
    p.Vz = vz * iv;
    p.NdV = s.rec[F_NDV][i];
    const float ar = s.rec[F_AR][i], ag = s.rec[F_AG][i], ab = s.rec[F_AB][i];
    p.dr = ar * kInvPi; p.dg = ag * kInvPi; p.db = ab * kInvPi;
    p.rough = s.rec[F_ROUGH][i]; p.metal = s.rec[F_METAL][i];
    if (NF > int(F_F0R)) {
        p.f0r = s.rec[F_F0R][i]; p.f0g = s.rec[F_F0G][i]; p.f0b = s.rec[F_F0B][i];
    } else {  // the metallic workflow's F0, clamped as finish_pixel clamps it
        p.f0r = fmin_(fmax_(metallic_f0(ar, p.metal), 0.0f), 0.999f);
        p.f0g = fmin_(fmax_(metallic_f0(ag, p.metal), 0.0f), 0.999f);
        p.f0b = fmin_(fmax_(metallic_f0(ab, p.metal), 0.0f), 0.999f);
    }
    b = pixel_brdf(p);
}

// Evaluates nb queued pairs of this warp, one per lane, and accumulates their gradients:
// the first lane holding a light (a pixel) sums that light's (pixel's) pairs of the batch
// in lane order and adds the sum to the warp's accumulator. Out of line: one copy of the
// adjoint code.
template <uint32_t LAYOUT, int NF>
__device__ __noinline__ void flush_batch(AdjSmem<NF>& s, uint32_t warp, uint32_t lane, uint32_t head, uint32_t nb,
                                         uint32_t wlo, float camx, float camy, float camz) {
    const bool act = lane < nb;
    const uint32_t e = act ? s.queue[warp][(head + lane) & (kQueue - 1)] : 0u;
    const uint32_t q = e >> 23, li = e & 0x7fffffu;
    float g[kComps] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    float gp[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    bool lit = false;
    if (act) {
        Pixel p;
        PixelBrdf pb;
        load_pixel<LAYOUT>(s, q, p, pb, camx, camy, camz);
        const ShadeLight l = s.light[li - wlo];
        lit = eval_adjoint<true>(p, pb, l, s.rec[F_WR][q], s.rec[F_WG][q], s.rec[F_WB][q],
                                 LAYOUT != HL_GBUF_REFERENCE, g, gp);
    }
    float* mine = s.gbuf[warp][lane];
#pragma unroll
    for (int c = 0; c < 7; ++c) mine[c] = g[c];
#pragma unroll
    for (int c = 0; c < 5; ++c) mine[7 + c] = gp[c];
    __syncwarp();
    const uint32_t lt = lanemask_lt();
    const uint32_t lpeers = __match_any_sync(0xffffffffu, lit ? li : (0x800000u | lane));
    const uint32_t ppeers = __match_any_sync(0xffffffffu, lit ? q : (0x10000u | lane));
    if (lit && (lpeers & lt) == 0u) {
        float sum[7] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        for (uint32_t m = lpeers; m; m &= m - 1u) {
            const float* o = s.gbuf[warp][__ffs(m) - 1];
#pragma unroll
            for (int c = 0; c < 7; ++c) sum[c] += o[c];
        }
        float* a = s.acc[warp][li - wlo];
#pragma unroll
        for (int c = 0; c < 7; ++c) a[c] += sum[c];
    }
    if (lit && (ppeers & lt) == 0u) {
        float sum[5] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
        for (uint32_t m = ppeers; m; m &= m - 1u) {
            const float* o = s.gbuf[warp][__ffs(m) - 1];
#pragma unroll
            for (int c = 0; c < 5; ++c) sum[c] += o[7 + c];
        }
#pragma unroll
        for (int c = 0; c < 5; ++c) s.gpx[c][q] += sum[c];
    }
    __syncwarp();
}

template <uint32_t LAYOUT, uint32_t GRID>
__global__ void __launch_bounds__(kThreads, 2) adjoint_kernel(
    const GpuCamera* __restrict__ cam, const DeferredGlobals* __restrict__ glb, const GBufView gb,
    const GpuLight* __restrict__ lights, uint32_t n_lights, const GridView grid, const __grid_constant__ SliceTable tab,
    const unsigned char* __restrict__ d_rad, uint64_t d_rad_pitch, float* __restrict__ part,
    float* __restrict__ d_pix, int* __restrict__ status) {
    constexpr bool FROXELS = (GRID == HL_GRID_FROXELS);
    constexpr int NF = record_fields<LAYOUT>();
    extern __shared__ __align__(16) unsigned char smem_raw[];
    AdjSmem<NF>& s = *reinterpret_cast<AdjSmem<NF>*>(smem_raw);
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
    uint32_t* queue = s.queue[warp];
    const uint32_t* list = grid.lists;

    // windows of kWin lights; one (empty) window when there are none, for the ambient term
#pragma unroll 1
    for (uint32_t wlo = 0;; wlo += kWin) {
        const uint32_t whi = min(n_lights, wlo + kWin);
        __syncthreads();  // the previous window's partials are read out
        for (uint32_t k = t; k < whi - wlo; k += kThreads) s.light[k] = load_shade_light(lights, wlo + k);
        float* accf = &s.acc[0][0][0];
        for (uint32_t k = t; k < uint32_t(kWarps * kWin * 7); k += kThreads) accf[k] = 0.0f;
        __syncthreads();

        // a warp only touches its own pixels' records and its own accumulators: no
        // CTA-wide barrier inside a window
#pragma unroll 1
        for (uint32_t tile = blockIdx.x; tile < n_tiles; tile += gridDim.x) {
            // ---- set-up of this lane's pixel ----
            const uint32_t x = (tile % tiles_x) * kTW + t % kTW, y = (tile / tiles_x) * kTH + t / kTW;
            bool valid = false;
            float px = 0, py = 0, pz = 0, plx = 0, ply = 0, plz = 0, ny = 0, nx = 0, nz = 0, slack = 0;
            float ao = 1.0f;
            uint32_t cur = 0, end = 0;
#pragma unroll
            for (int c = 0; c < 5; ++c) s.gpx[c][t] = 0.0f;
            if (x < gb.width && y < gb.height) {
                const Texel<LAYOUT> tx = load_texel<LAYOUT>(gb, x, y);
                valid = tx.depth < 1.0f;
                if (valid) {
                    Pixel p;
                    reconstruct<true>(cam->inv_view_proj, x, y, W, H, tx.depth, p.Px, p.Py, p.Pz, p.Plx, p.Ply, p.Plz);
                    finish_pixel<true>(p, tx.nx, tx.ny, tx.nz, tx.ar, tx.ag, tx.ab, tx.rough, tx.metal, tx.f0r,
                                       tx.f0g, tx.f0b, camx, camy, camz);
                    ao = tx.ao;
                    const float4 w = *reinterpret_cast<const float4*>(d_rad + d_rad_pitch * y + 16ull * x);
                    s.rec[F_PX][t] = p.Px; s.rec[F_PY][t] = p.Py; s.rec[F_PZ][t] = p.Pz;
                    s.rec[F_PLX][t] = p.Plx; s.rec[F_PLY][t] = p.Ply; s.rec[F_PLZ][t] = p.Plz;
                    s.rec[F_NDV][t] = p.NdV;
                    s.rec[F_AR][t] = tx.ar; s.rec[F_AG][t] = tx.ag; s.rec[F_AB][t] = tx.ab;
                    s.rec[F_ROUGH][t] = p.rough; s.rec[F_METAL][t] = p.metal;
                    s.rec[F_NRX][t] = p.nrx; s.rec[F_NRY][t] = p.nry; s.rec[F_NRZ][t] = p.nrz;
                    s.rec[F_WR][t] = w.x; s.rec[F_WG][t] = w.y; s.rec[F_WB][t] = w.z;
                    if (NF > int(F_F0R)) {
                        s.rec[F_F0R][t] = p.f0r; s.rec[F_F0G][t] = p.f0g; s.rec[F_F0B][t] = p.f0b;
                    }
                    px = p.Px; py = p.Py; pz = p.Pz; plx = p.Plx; ply = p.Ply; plz = p.Plz;
                    nx = p.Nx; ny = p.Ny; nz = p.Nz;
                    // |N.t| within |P| 2^-20 of zero is left to the exact NdL cut
                    slack = fma_(pz, pz, fma_(py, py, px * px)) * (1.0f / 1099511627776.0f);
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
                    // this window's part of the (ascending) list
                    if (wlo > 0) cur = lower_bound(list, cur, end, wlo);
                    if (whi < n_lights) end = lower_bound(list, cur, end, whi);
                }
            }
            __syncwarp();  // the warp's records are written

            // ---- walk: own list entries tested for range and NdL sign, passing pairs queued ----
            uint32_t head = 0, qlen = 0;
            const uint32_t ln = end - cur;
            const uint32_t maxlen = __reduce_max_sync(0xffffffffu, ln);
#pragma unroll 1
            for (uint32_t j0 = 0; j0 < maxlen; j0 += kPipe) {
                uint32_t li[kPipe];
#pragma unroll
                for (int u = 0; u < kPipe; ++u) li[u] = (j0 + u < ln) ? __ldg(list + cur + j0 + u) : 0xffffffffu;
#pragma unroll
                for (int u = 0; u < kPipe; ++u) {
                    // entries outside [wlo, whi) only come from an unsorted list; they are skipped
                    bool pass = false;
                    if (li[u] >= wlo && li[u] < whi) {
                        const ShadeLight& l = s.light[li[u] - wlo];
                        pass = l.type == 0u || candidate(px, py, pz, plx, ply, plz, nx, ny, nz, l.px, l.py, l.pz,
                                                         l.range * l.range * (1.0f + 1.0f / 512.0f), slack, true);
                    }
                    const uint32_t pm = __ballot_sync(0xffffffffu, pass);
                    if (pass) queue[(head + qlen + __popc(pm & lanemask_lt())) & (kQueue - 1)] = (t << 23) | li[u];
                    qlen += __popc(pm);
                }
                __syncwarp();
                while (qlen >= 32) {
                    flush_batch<LAYOUT>(s, warp, lane, head, 32, wlo, camx, camy, camz);
                    head += 32;
                    qlen -= 32;
                }
            }
            if (qlen > 0) flush_batch<LAYOUT>(s, warp, lane, head, qlen, wlo, camx, camy, camz);

            // ---- this lane's pixel gradients (all its pairs were the warp's own) ----
            if (x < gb.width && y < gb.height) {
                float* o = d_pix + (size_t(y) * gb.width + x) * 5;
                if (!valid) {
                    if (wlo == 0) {
#pragma unroll
                        for (int c = 0; c < 5; ++c) o[c] = 0.0f;
                    }
                } else if (wlo == 0) {
                    // hemisphere ambient times ao (deferred_lighting.wgsl:1196-1199) depends on albedo
                    const float ht = fma_(ny, 0.5f, 0.5f);
                    const float wc[3] = {s.rec[F_WR][t], s.rec[F_WG][t], s.rec[F_WB][t]};
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        o[c] = s.gpx[c][t] + wc[c] * fma_(sky[c], ht, sky[c] * 0.15f * (1.0f - ht)) * ao;
                    o[3] = s.gpx[3][t];
                    o[4] = s.gpx[4][t];
                } else {
#pragma unroll
                    for (int c = 0; c < 5; ++c) o[c] += s.gpx[c][t];
                }
            }
            __syncwarp();  // records and pixel gradients are reused by the next tile
        }
        __syncthreads();
        // the CTA's partial for this window: warps added in order
        for (uint32_t k = t; k < whi - wlo; k += kThreads) {
            float v[7];
#pragma unroll
            for (int c = 0; c < 7; ++c) {
                float a = s.acc[0][k][c];
#pragma unroll
                for (int w = 1; w < kWarps; ++w) a += s.acc[w][k][c];
                v[c] = a;
            }
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
    const int smem = int(sizeof(AdjSmem<record_fields<LAYOUT>()>));
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    k<<<G, kThreads, smem, stream>>>(static_cast<const GpuCamera*>(camera),
                                     static_cast<const DeferredGlobals*>(globals), gb,
                                     static_cast<const GpuLight*>(lights), n, grid, tab, d_rad, d_rad_pitch, part,
                                     d_pix, status);
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
        // the largest record (reference layout) bounds every layout's occupancy
        auto k = adjoint_kernel<HL_GBUF_REFERENCE, HL_GRID_FROXELS>;
        const int smem = int(sizeof(AdjSmem<record_fields<HL_GBUF_REFERENCE>()>));
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess ||
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kThreads, smem) != cudaSuccess || per_sm < 1)
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
