// hl_shade.cu — deferred lighting (fs_main under fallback bindings) for sm_103a.
//
// One CTA of 256 threads lights a 32x16-pixel tile (froxel grid) or one 16x16 reference
// light-cull tile (tile grid):
//  1. threads decode the tile's G-buffer texels (coalesced along x) and set each pixel
//     up (world position, N, V, NdV, albedo, F0, Schlick-GGX of the view) into shared
//     memory, with its light list (its froxel's list, or the tile's reference list);
//  2. pixels are counting-sorted by froxel (slice, column), so a group of 32 pixels
//     mostly shares one list; each warp takes a light and a heavy group;
//  3. each lane walks its own pixel's list in list order, three entries at a time (two
//     on the precise path) with their loads in flight together, and tests each light
//     for range and the NdL sign; passing (pixel, light) pairs go to a per-warp queue;
//  4. queued pairs are evaluated 32 at a time, one per lane, so the full BRDF of
//     pbr_direct_light runs with all lanes busy, and are added into per-pixel Kahan
//     accumulators in queue order, which is list order for every pixel, as the
//     reference's light loop adds them;
//  5. threads compose hemisphere ambient and emissive and store their pixels.
#include "hl_common.cuh"
#include "hl_internal.h"
#include "hl_shade_math.cuh"
#include "hl_indirect.cuh"
#include "hl_shadow.cuh"
#include "hl_texel.cuh"
#include "hl_precise.cuh"

namespace hl {

namespace {

using namespace sm;
using gbuf::Texel;
using gbuf::load_texel;

namespace sk {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kQueue = 128;      // per-warp pair ring (up to 31 + kPipe * 32 pending)
constexpr int kBins = 512;       // froxel keys of the pixel sort
constexpr int kPipe = 3;         // list entries in flight per lane (fast path; 2 on the precise path)
constexpr int kBoxMin = 8;       // shortest shared list worth a box cull

// Pixel record fields (structure of arrays). N, 1/|n|, V, F0 (except for the reference
// layout, which stores its own), the view's Schlick-GGX term and the fast path's guard
// are not stored: they are recomputed from these with the set-up's own operations, so a
// record of 16 fields (19 for the reference layout) keeps three CTAs on an SM.
enum Field : int {
    F_PX, F_PY, F_PZ, F_PLX, F_PLY, F_PLZ, F_NDV, F_AR, F_AG, F_AB, F_ROUGH, F_METAL,
    F_DEPTH,  // negative: the pixel was set up on the precise path (its guard is 0)
    F_NRX, F_NRY, F_NRZ,
    F_F0R, F_F0G, F_F0B,  // reference layout only
    F_COUNT
};

template <uint32_t LAYOUT>
__host__ __device__ constexpr int record_fields() { return LAYOUT == HL_GBUF_REFERENCE ? int(F_COUNT) : int(F_F0R); }

static_assert(31 + 32 * kPipe <= kQueue, "pair ring too small");

template <int NPX, int NF>
struct Smem {
    float px[NF][NPX];
    float acc[6][NPX];              // Kahan (sum, compensation) x RGB; statistics reuse it
    uint32_t base[NPX], len[NPX];   // each pixel's light list
    union {
        struct {                    // set-up and sort only
            uint32_t hist[kBins];
            float tab[kMaxSlices + 1];        // slice boundaries
            uint16_t col_of[32], row_of[16];  // froxel column / row of the tile's pixel columns / rows
        } sort;
        uint32_t queue[kWarps][kQueue];  // walk only: ring of (pixel << 23) | light index
    } u;
    uint16_t order[NPX];            // pixels sorted by froxel
    uint32_t warp_tot[kWarps];
    uint32_t n_valid;
    uint32_t next_group;            // next group of sorted pixels to hand to a warp
};
// Three CTAs of the FP16 / FP32 record fit in a 164 KB shared-memory carve-out, which
// leaves 92 KB of the SM's 256 KB to L1 for the light tables and lists.
static_assert(3 * (sizeof(Smem<512, int(F_F0R)>) + 1024) <= 164 * 1024, "shading CTA shared memory");

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <int NPX, int NF>
__device__ __forceinline__ void store_pixel(Smem<NPX, NF>& s, int i, const Pixel& p, bool precise, float depth,
                                            float ar, float ag, float ab) {
    s.px[F_PX][i] = p.Px; s.px[F_PY][i] = p.Py; s.px[F_PZ][i] = p.Pz;
    s.px[F_PLX][i] = p.Plx; s.px[F_PLY][i] = p.Ply; s.px[F_PLZ][i] = p.Plz;
    s.px[F_NDV][i] = p.NdV;
    s.px[F_AR][i] = ar; s.px[F_AG][i] = ag; s.px[F_AB][i] = ab;
    s.px[F_ROUGH][i] = p.rough; s.px[F_METAL][i] = p.metal;
    s.px[F_DEPTH][i] = precise ? -depth : depth;
    s.px[F_NRX][i] = p.nrx; s.px[F_NRY][i] = p.nry; s.px[F_NRZ][i] = p.nrz;
    if (NF > int(F_F0R)) {
        s.px[F_F0R][i] = p.f0r; s.px[F_F0G][i] = p.f0g; s.px[F_F0B][i] = p.f0b;
    }
}

// The unit normal finish_pixel computed, from the stored raw normal.
template <int NPX, int NF>
__device__ __forceinline__ void pixel_normal(const Smem<NPX, NF>& s, int i, float& nx, float& ny, float& nz,
                                             float& in) {
    const float rx = s.px[F_NRX][i], ry = s.px[F_NRY][i], rz = s.px[F_NRZ][i];
    in = rsqrt_(fma_(rz, rz, fma_(ry, ry, rx * rx)));
    nx = rx * in;
    ny = ry * in;
    nz = rz * in;
}

// V as finish_pixel computed it: from the camera-relative position on the fast path
// (camera at the origin; lo is 0 unless the pixel was set up precisely), from the
// double-float difference to the camera otherwise.
template <bool PRECISE>
__device__ __forceinline__ void pixel_view(Pixel& p, float camx, float camy, float camz) {
    float vx, vy, vz;
    if (PRECISE) {
        const DF ux = two_sum(camx, -p.Px), uy = two_sum(camy, -p.Py), uz = two_sum(camz, -p.Pz);
        vx = two_sum(ux.hi, ux.lo - p.Plx).hi;
        vy = two_sum(uy.hi, uy.lo - p.Ply).hi;
        vz = two_sum(uz.hi, uz.lo - p.Plz).hi;
    } else {
        vx = -p.Px - p.Plx;
        vy = -p.Py - p.Ply;
        vz = -p.Pz - p.Plz;
    }
    const float iv = rsqrt_(fma_(vz, vz, fma_(vy, vy, vx * vx)));
    p.Vx = vx * iv;
    p.Vy = vy * iv;
    p.Vz = vz * iv;
}

template <uint32_t LAYOUT, int NPX, int NF>
__device__ __forceinline__ void load_pixel(const Smem<NPX, NF>& s, int i, Pixel& p, PixelBrdf& b, float camx,
                                           float camy, float camz) {
    constexpr bool PRECISE = (LAYOUT != HL_GBUF_F16);
    p.Px = s.px[F_PX][i]; p.Py = s.px[F_PY][i]; p.Pz = s.px[F_PZ][i];
    p.Plx = s.px[F_PLX][i]; p.Ply = s.px[F_PLY][i]; p.Plz = s.px[F_PLZ][i];
    p.nrx = s.px[F_NRX][i]; p.nry = s.px[F_NRY][i]; p.nrz = s.px[F_NRZ][i];
    pixel_normal(s, i, p.Nx, p.Ny, p.Nz, p.inv_n);
    pixel_view<PRECISE>(p, camx, camy, camz);
    p.NdV = s.px[F_NDV][i];
    const float ar = s.px[F_AR][i], ag = s.px[F_AG][i], ab = s.px[F_AB][i];
    p.dr = ar * kInvPi; p.dg = ag * kInvPi; p.db = ab * kInvPi;
    p.rough = s.px[F_ROUGH][i]; p.metal = s.px[F_METAL][i];
    if (NF > int(F_F0R)) {
        p.f0r = s.px[F_F0R][i]; p.f0g = s.px[F_F0G][i]; p.f0b = s.px[F_F0B][i];
    } else {  // the metallic workflow's F0, clamped as finish_pixel clamps it
        p.f0r = fmin_(fmax_(metallic_f0(ar, p.metal), 0.0f), 0.999f);
        p.f0g = fmin_(fmax_(metallic_f0(ag, p.metal), 0.0f), 0.999f);
        p.f0b = fmin_(fmax_(metallic_f0(ab, p.metal), 0.0f), 0.999f);
    }
    b = pixel_brdf(p);
    if (PRECISE) df_view(p, b, camx, camy, camz);  // V as a double-float unit vector
}

}  // namespace sk

// Evaluates nb queued pairs (ring positions head..head+nb-1), one per lane, and adds
// them into the per-pixel Kahan accumulators in queue order. Out of line so that the
// BRDF code exists once in the kernel.
template <uint32_t LAYOUT, bool STATS, int TW, int NPX, bool EXT>
__device__ __noinline__ void flush_batch(sk::Smem<NPX, sk::record_fields<LAYOUT>()>& s, const uint32_t* queue, uint32_t head, uint32_t nb,
                                         uint32_t lane, const GpuCamera* cam, const GpuLight* lights, uint32_t x0,
                                         uint32_t y0, float W, float H, const ExtView* sv, const PairLog log) {
    using namespace sk;
    constexpr bool PRECISE = (LAYOUT != HL_GBUF_F16);
    uint32_t (*cnt)[NPX] = reinterpret_cast<uint32_t (*)[NPX]>(s.acc);
    const bool act = lane < nb;
    const uint32_t e = act ? queue[(head + lane) & (kQueue - 1)] : 0u;
    const uint32_t q = e >> 23, li = e & 0x7fffffu;
    int st = kCut;
    float cr = 0.0f, cg = 0.0f, cb = 0.0f;
    bool rng = false;
    if (act) {
        Pixel p;
        PixelBrdf pb;
        load_pixel<LAYOUT>(s, q, p, pb, cam->position_near[0], cam->position_near[1], cam->position_near[2]);
        const float4* gl = reinterpret_cast<const float4*>(lights + li);
        const float4 a = __ldg(gl + 0), b = __ldg(gl + 1), c = __ldg(gl + 2);
        const uint4 d = __ldg(reinterpret_cast<const uint4*>(gl + 3));
        ShadeLight l;
        l.range = a.w;
        l.dx = b.x; l.dy = b.y; l.dz = b.z; l.cos_outer = b.w;
        l.cr = c.x; l.cg = c.y; l.cb = c.z; l.intensity = c.w;
        l.type = d.y;
        l.cos_inner = __uint_as_float(d.z);
        DF ux{a.x, 0.0f}, uy{a.y, 0.0f}, uz{a.z, 0.0f};
        if (!PRECISE) {  // camera-relative light position and its exact rounding residual
            ux = two_sum(a.x, -cam->position_near[0]);
            uy = two_sum(a.y, -cam->position_near[1]);
            uz = two_sum(a.z, -cam->position_near[2]);
        }
        l.px = ux.hi; l.py = uy.hi; l.pz = uz.hi;
        if (STATS) rng = in_range(p, l);
        const float dq = s.px[F_DEPTH][q];
        st = eval<PRECISE>(p, pb, l, cr, cg, cb, (PRECISE || dq < 0.0f) ? 0.0f : fast_guard(p));
        if (!PRECISE && st == kNeedsPrecise)
            st = precise_pair(cam, x0 + q % TW, y0 + q / TW, W, H, dq, p, s.px[F_AR][q], s.px[F_AG][q],
                              s.px[F_AB][q], l, ux.lo, uy.lo, uz.lo, cr, cg, cb);
        if (EXT && sv->dyn && st == kLit && li < sv->max_lights && d.x != HL_NO_SHADOW) {
            // the pair's shadow factor (deferred_lighting.wgsl:1136-1141) at the pixel's world
            // position rounded to f32: on the fast path from a precise reconstruction, since
            // the camera-relative f32 position can be ~1e-5 off, enough to move a receiver
            // across a shadow texel's depth
            const float camx = cam->position_near[0], camy = cam->position_near[1], camz = cam->position_near[2];
            float wx = p.Px + p.Plx, wy = p.Py + p.Ply, wz = p.Pz + p.Plz;
            if (!PRECISE) {
                float hx, hy, hz, lx, ly, lz;
                reconstruct<true, false>(cam->inv_view_proj, x0 + q % TW, y0 + q / TW, W, H, fabsf(dq), hx, hy, hz,
                                         lx, ly, lz);
                wx = hx + lx;
                wy = hy + ly;
                wz = hz + lz;
            }
            const float4 csm = __ldg(reinterpret_cast<const float4*>(sv->csm));
            const float sf = shadow_factor(*sv, li, a, b, d.x, d.y, wx, wy, wz, p.Nx, p.Ny, p.Nz,
                                           float(x0 + q % TW) + 0.5f, float(y0 + q / TW) + 0.5f, camx, camy, camz, csm);
            cr *= sf;
            cg *= sf;
            cb *= sf;
        }
    }
    const bool lit = act && st == kLit;
    if (!STATS && log.pairs) {  // record the pairs the kernel lit (branch decisions for verification)
        const uint32_t m = __ballot_sync(0xffffffffu, lit);
        if (m) {
            uint32_t base = 0;
            if (lane == 0) base = atomicAdd(log.count, uint32_t(__popc(m)));
            base = __shfl_sync(0xffffffffu, base, 0);
            const uint32_t slot = base + __popc(m & lanemask_lt());
            if (lit && slot < log.capacity)
                log.pairs[slot] = make_uint2((y0 + q / TW) * uint32_t(W) + x0 + q % TW, li);
        }
    }
    if (STATS) {
        if (act && rng) atomicAdd(&cnt[1][q], 1u);
        if (lit) atomicAdd(&cnt[2][q], 1u);
    } else {
        // rank of this pair among the batch's pairs of the same pixel (queue order)
        const uint32_t k2 = lit ? q : (0x10000u | lane);
        const uint32_t peers = __match_any_sync(0xffffffffu, k2);
        const uint32_t rank = __popc(peers & lanemask_lt());
        const uint32_t rounds = __reduce_max_sync(0xffffffffu, lit ? rank + 1 : 0u);
        for (uint32_t r = 0; r < rounds; ++r) {
            if (lit && rank == r) {
                kahan_add(s.acc[0][q], s.acc[3][q], cr);
                kahan_add(s.acc[1][q], s.acc[4][q], cg);
                kahan_add(s.acc[2][q], s.acc[5][q], cb);
            }
            __syncwarp();
        }
    }
    __syncwarp();
}

// Light-space projection view of shadow debug mode 11 (deferred_lighting.wgsl:1066-1080):
// the pixel's world position in f32 as the shader forms it (uv = frag / size, ndc,
// inv_view_proj v / w), projected by the first shadow matrix; orange inside its
// frustum (depth in red), dark blue outside. Correctly rounded operations in the
// shader's order.
__device__ __noinline__ float4 shadow_projection_view(const float* ivp, const float* m0, uint32_t x, uint32_t y,
                                                      float W, float H, float depth) {
    const float ux = xdiv(xadd(float(x), 0.5f), W), uy = xdiv(xadd(float(y), 0.5f), H);
    const float nx = xsub(xmul(ux, 2.0f), 1.0f), ny = xsub(1.0f, xmul(uy, 2.0f));
    const float hw = xmat_row(ivp, 3, nx, ny, depth, 1.0f);
    const float wx = xdiv(xmat_row(ivp, 0, nx, ny, depth, 1.0f), hw);
    const float wy = xdiv(xmat_row(ivp, 1, nx, ny, depth, 1.0f), hw);
    const float wz = xdiv(xmat_row(ivp, 2, nx, ny, depth, 1.0f), hw);
    float m[16];
#pragma unroll
    for (int k = 0; k < 16; ++k) m[k] = __ldg(m0 + k);
    const float lw = xmat_row(m, 3, wx, wy, wz, 1.0f);
    if (lw > 0.001f) {
        const float n0 = xdiv(xmat_row(m, 0, wx, wy, wz, 1.0f), lw);
        const float n1 = xdiv(xmat_row(m, 1, wx, wy, wz, 1.0f), lw);
        const float n2 = xdiv(xmat_row(m, 2, wx, wy, wz, 1.0f), lw);
        const float u = xadd(xmul(n0, 0.5f), 0.5f), v = xadd(xmul(-n1, 0.5f), 0.5f);
        if (u >= 0.0f && v >= 0.0f && u <= 1.0f && v <= 1.0f && n2 >= 0.0f && n2 <= 1.0f)
            return make_float4(n2, xmul(n2, 0.3f), 0.0f, 1.0f);
    }
    return make_float4(0.0f, 0.0f, 0.2f, 1.0f);
}

// TW x TH = 512 (froxel grid) or 256 (tile grid) pixels, 256 threads.
// One tile (bx, by) of one view; tabz: the view's slice boundaries (froxel grid).
// PREFETCH: the kernel's grid is this view's tiles (bx, by); before the walk the CTA asks
// L2 for the G-buffer of the tile three CTAs per SM further on, the one likely to start
// on an SM as the current wave drains, so its set-up loads hit L2.
template <uint32_t LAYOUT, uint32_t GRID, uint32_t TARGET, bool STATS, int TW, int TH, bool PREFETCH = false,
          bool EXT = false>
__device__ __forceinline__ void shade_tile(
    const GpuCamera* __restrict__ cam, const DeferredGlobals* __restrict__ glb, const GBufView& gb,
    const GpuLight* __restrict__ lights, const float4* __restrict__ cand, uint32_t n_lights, const GridView& grid,
    const float* __restrict__ tabz, const TargetView& out, uint32_t* __restrict__ stats, int* __restrict__ status,
    uint32_t bx, uint32_t by, const ExtView* sv, const PairLog& log) {
    using namespace sk;
    constexpr bool FROXELS = (GRID == HL_GRID_FROXELS);
    constexpr int NPX = TW * TH;
    constexpr int PPT = NPX / kThreads;  // pixels per thread in set-up and output
    constexpr int NG = NPX / 32;         // groups of 32 sorted pixels
    static_assert(NPX % kThreads == 0 && (NG == kWarps || NG == 2 * kWarps), "256 or 512 pixels per tile");
    static_assert(TW <= 32 && TH <= 16 && TW + TH <= kThreads, "column / row tables of the tile");
    constexpr bool PRECISE = (LAYOUT != HL_GBUF_F16);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    constexpr int NF = record_fields<LAYOUT>();
    Smem<NPX, NF>& s = *reinterpret_cast<Smem<NPX, NF>*>(smem_raw);
    uint32_t (*cnt)[NPX] = reinterpret_cast<uint32_t (*)[NPX]>(s.acc);  // statistics view
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t x0 = bx * TW, y0 = by * TH;
    const float W = float(gb.width), H = float(gb.height);
    const float camx = cam->position_near[0], camy = cam->position_near[1], camz = cam->position_near[2];

    // the tile's G-buffer texels, loaded before the first barrier so that their latency
    // overlaps the set-up of shared memory; decoded in the set-up loop
    gbuf::RawTexel raw[PPT];
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const uint32_t i = t + k * kThreads;
        const uint32_t x = x0 + i % TW, y = y0 + i / TW;
        raw[k] = gbuf::RawTexel{};
        raw[k].depth = 1.0f;
        if (x < gb.width && y < gb.height) raw[k] = gbuf::load_raw<LAYOUT>(gb, x, y);
    }

    for (uint32_t b = t; b < uint32_t(kBins); b += kThreads) s.u.sort.hist[b] = 0;
    if (FROXELS) {
        for (uint32_t k = t; k <= grid.fp.grid_z; k += kThreads) s.u.sort.tab[k] = tabz[k];
        // froxel column of each pixel column and row of the tile (one division each)
        if (t < uint32_t(TW))
            s.u.sort.col_of[t] = uint16_t((uint64_t(x0 + t) * grid.fp.grid_x) / grid.fp.width);
        else if (t < uint32_t(TW + TH))
            s.u.sort.row_of[t - TW] = uint16_t((uint64_t(y0 + t - TW) * grid.fp.grid_y) / grid.fp.height);
    }
#pragma unroll
    for (int k = 0; k < PPT; ++k)
        for (int c = 0; c < 6; ++c) s.acc[c][t + k * kThreads] = 0.0f;

    // the tile's froxel columns, and the tile grid's list
    uint32_t fx0 = 0, fy0 = 0, ncx = 1, ncols = 1, tile_base = 0, tile_len = 0;
    bool key_by_column = false;
    if (FROXELS) {
        const hl_froxel_params& fp = grid.fp;
        const uint32_t xe = min(x0 + TW, gb.width) - 1, ye = min(y0 + TH, gb.height) - 1;
        fx0 = (x0 * fp.grid_x) / fp.width;
        fy0 = (y0 * fp.grid_y) / fp.height;
        ncx = (xe * fp.grid_x) / fp.width - fx0 + 1;
        ncols = ncx * ((ye * fp.grid_y) / fp.height - fy0 + 1);
        key_by_column = ncols * fp.grid_z <= uint32_t(kBins);
    } else {
        const uint32_t tile = by * glb->num_tiles_x + bx;
        pdl_wait();  // the lists are written
        if (tile < grid.tiles) {
            tile_len = __ldg(grid.counts + tile);
            if (tile_len > kMaxPerTile) {
                if (t == 0) raise_status(status, HL_ERR_DEVICE_BOUNDS);
                tile_len = kMaxPerTile;
            }
            tile_base = tile * kMaxPerTile;
        } else if (t == 0) {
            raise_status(status, HL_ERR_DEVICE_BOUNDS);
        }
    }
    __syncthreads();

    // slices are exponential from slice_near to tab[grid_z]: slice ~ log2(d / near) * scale
    const float slice_inv_near = FROXELS ? rcp_(grid.fp.slice_near) : 0.0f;
    const float slice_scale =
        FROXELS ? float(grid.fp.grid_z) * rcp_(__log2f(fmaxf(s.u.sort.tab[grid.fp.grid_z] * slice_inv_near, 2.0f))) : 0.0f;

    // ---- 1. pixel set-up -------------------------------------------------------
    float rel[12], wrow[4];
    if (!PRECISE) camera_relative_rows(cam->inv_view_proj, camx, camy, camz, rel, wrow);
    const float iW = rcp_(W), iH = rcp_(H);
    bool valid[PPT];
    uint32_t key[PPT], slot[PPT];
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const uint32_t i = t + k * kThreads;
        const uint32_t x = x0 + i % TW, y = y0 + i / TW;
        valid[k] = false;
        key[k] = 0;
        slot[k] = 0;
        if (x < gb.width && y < gb.height) {
            const Texel<LAYOUT> tx = gbuf::decode_texel<LAYOUT>(raw[k]);
            valid[k] = tx.depth < 1.0f;
            if (valid[k]) {
                Pixel p;
                bool precise_setup = PRECISE;
                if (PRECISE) {
                    reconstruct<true>(cam->inv_view_proj, x, y, W, H, tx.depth, p.Px, p.Py, p.Pz, p.Plx, p.Ply, p.Plz);
                    finish_pixel<true>(p, tx.nx, tx.ny, tx.nz, tx.ar, tx.ag, tx.ab, tx.rough, tx.metal, tx.f0r, tx.f0g,
                                       tx.f0b, camx, camy, camz);
                } else {
                    const float ndx = fma_(float(2u * x + 1u), iW, -1.0f);
                    const float ndy = fma_(float(2u * y + 1u), -iH, 1.0f);
                    reconstruct_relative(rel, wrow, ndx, ndy, tx.depth, p.Px, p.Py, p.Pz);
                    p.Plx = p.Ply = p.Plz = 0.0f;
                    finish_pixel<false>(p, tx.nx, tx.ny, tx.nz, tx.ar, tx.ag, tx.ab, tx.rough, tx.metal, tx.f0r,
                                        tx.f0g, tx.f0b, 0.0f, 0.0f, 0.0f);
                    if (p.NdV < kFastMinNdV) {
                        // grazing view: precise set-up, camera-relative double-float position
                        reconstruct<true, false>(cam->inv_view_proj, x, y, W, H, tx.depth, p.Px, p.Py, p.Pz, p.Plx,
                                                 p.Ply, p.Plz);
                        const DF ax = two_sum(p.Px, -camx), ay = two_sum(p.Py, -camy), az = two_sum(p.Pz, -camz);
                        const DF bx = two_sum(ax.hi, ax.lo + p.Plx), by = two_sum(ay.hi, ay.lo + p.Ply),
                                 bz = two_sum(az.hi, az.lo + p.Plz);
                        p.Px = bx.hi; p.Plx = bx.lo; p.Py = by.hi; p.Ply = by.lo; p.Pz = bz.hi; p.Plz = bz.lo;
                        finish_pixel<true>(p, tx.nx, tx.ny, tx.nz, tx.ar, tx.ag, tx.ab, tx.rough, tx.metal, tx.f0r,
                                           tx.f0g, tx.f0b, 0.0f, 0.0f, 0.0f);
                        precise_setup = true;
                    }
                }
                store_pixel(s, i, p, precise_setup, tx.depth, tx.ar, tx.ag, tx.ab);
                uint32_t b = tile_base, n = tile_len;
                if (FROXELS) {
                    // own froxel: column of (x, y), slice of the linear view depth
                    const float nr = cam->position_near[3], fr = cam->forward_far[3];
                    const float dv = div_(nr * fr, fma_(-tx.depth, fr - nr, fr));
                    const hl_froxel_params& fp = grid.fp;
                    // largest sl < grid_z with tab[sl] <= dv: a guess from the exponential
                    // slice spacing, then exact steps against the table
                    const int guess = int(__log2f(dv * slice_inv_near) * slice_scale);
                    uint32_t sl = uint32_t(min(max(guess, 0), int(fp.grid_z) - 1));
                    while (sl + 1 < fp.grid_z && s.u.sort.tab[sl + 1] <= dv) ++sl;
                    while (sl > 0 && s.u.sort.tab[sl] > dv) --sl;
                    const uint32_t fx = s.u.sort.col_of[x - x0];
                    const uint32_t fy = s.u.sort.row_of[y - y0];
                    const uint32_t f = (fy * fp.grid_x + fx) * fp.grid_z + sl;
                    pdl_wait();  // the lists are written (the texel loads above overlap the binning)
                    b = __ldg(grid.counts + f);
                    const uint32_t e = __ldg(grid.counts + f + 1);
                    if (b <= e && e <= grid.lists_capacity) {
                        n = e - b;
                    } else {
                        raise_status(status, HL_ERR_DEVICE_BOUNDS);
                        n = 0;
                    }
                    key[k] = key_by_column ? sl * ncols + (fy - fy0) * ncx + (fx - fx0) : sl;
                }
                s.base[i] = b;
                s.len[i] = n;
                if (STATS) cnt[3][i] = n;
                slot[k] = atomicAdd(&s.u.sort.hist[key[k]], 1u);
            }
        }
    }
    pdl_wait();  // every thread: the walk reads the lists and the light table
    __syncthreads();
    {   // exclusive scan of the froxel-key histogram, two bins per thread
        const uint32_t a = s.u.sort.hist[2 * t], b = s.u.sort.hist[2 * t + 1];
        uint32_t v = a + b;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t n = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= uint32_t(o)) v += n;
        }
        if (lane == 31) s.warp_tot[warp] = v;
        __syncthreads();
        uint32_t before = 0, total = 0;
#pragma unroll
        for (int w = 0; w < kWarps; ++w) {
            const uint32_t wt = s.warp_tot[w];
            before += (uint32_t(w) < warp) ? wt : 0u;
            total += wt;
        }
        const uint32_t excl = before + v - (a + b);
        __syncthreads();
        s.u.sort.hist[2 * t] = excl;
        s.u.sort.hist[2 * t + 1] = excl + a;
        if (t == 0) {
            s.n_valid = total;
            s.next_group = 0;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < PPT; ++k)
        if (valid[k]) s.order[s.u.sort.hist[key[k]] + slot[k]] = uint16_t(t + k * kThreads);
    __syncthreads();

    if (PREFETCH) {
        uint32_t nsm;
        asm("mov.u32 %0, %%nsmid;" : "=r"(nsm));
        const uint32_t next = by * gridDim.x + bx + 3u * nsm;
        if (next < gridDim.x * gridDim.y)
            gbuf::prefetch_tile<LAYOUT>(gb, (next % gridDim.x) * TW, (next / gridDim.x) * TH, TW, TH, t, kThreads);
    }

    // ---- 2-4. groups of 32 sorted pixels walk their lists --------------------------
    const uint32_t n_valid = s.n_valid;
    uint32_t qlen = 0;
    uint32_t* queue = s.u.queue[warp];

    uint32_t head = 0;  // ring position of the oldest pending pair

#pragma unroll 1
    for (;;) {
        // warps take groups as they finish, last group first: the far slices sort last
        // and hold the longest lists, so the long work starts early
        uint32_t g = 0;
        if (lane == 0) g = atomicAdd(&s.next_group, 1u);
        g = __shfl_sync(0xffffffffu, g, 0);
        if (g >= uint32_t(NG)) break;
        g = uint32_t(NG - 1) - g;
        if (g * 32u >= n_valid) continue;  // empty group
        const uint32_t gs = g * 32 + lane;
        const bool own = gs < n_valid;
        const uint32_t i = own ? s.order[gs] : 0u;
        float px = 0, py = 0, pz = 0, plx = 0, ply = 0, plz = 0, nx = 0, ny = 0, nz = 0, slack = 0;
        uint32_t lb = 0, ln = 0;
        if (own) {
            px = s.px[F_PX][i]; py = s.px[F_PY][i]; pz = s.px[F_PZ][i];
            plx = s.px[F_PLX][i]; ply = s.px[F_PLY][i]; plz = s.px[F_PLZ][i];
            float in_;
            pixel_normal(s, i, nx, ny, nz, in_);
            // |N.t| within |P| 2^-20 of zero is left to the exact NdL cut
            slack = fma_(pz, pz, fma_(py, py, px * px)) * (1.0f / 1099511627776.0f);
            lb = s.base[i];
            ln = s.len[i];
        }
        // A group whose lanes all hold one list (common where depth is coherent) first
        // culls that list against the box around its pixels, 32 lights at a time; only
        // the survivors are tested per pixel. The box test is looser than the per-pixel
        // test, so the queued pairs, and their order per pixel, are unchanged.
        const uint32_t lb0 = __shfl_sync(0xffffffffu, lb, 0), ln0 = __shfl_sync(0xffffffffu, ln, 0);
        const bool shared = ln0 >= uint32_t(kBoxMin) && __all_sync(0xffffffffu, !own || (lb == lb0 && ln == ln0));
        const uint32_t maxlen = shared ? 0u : __reduce_max_sync(0xffffffffu, ln);
        if (shared) {
            float b0x = own ? px : 3.0e38f, b0y = own ? py : 3.0e38f, b0z = own ? pz : 3.0e38f;
            float b1x = own ? px : -3.0e38f, b1y = own ? py : -3.0e38f, b1z = own ? pz : -3.0e38f;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                b0x = fminf(b0x, __shfl_xor_sync(0xffffffffu, b0x, o));
                b0y = fminf(b0y, __shfl_xor_sync(0xffffffffu, b0y, o));
                b0z = fminf(b0z, __shfl_xor_sync(0xffffffffu, b0z, o));
                b1x = fmaxf(b1x, __shfl_xor_sync(0xffffffffu, b1x, o));
                b1y = fmaxf(b1y, __shfl_xor_sync(0xffffffffu, b1y, o));
                b1z = fmaxf(b1z, __shfl_xor_sync(0xffffffffu, b1z, o));
            }
            // rounding of positions and differences: widen by 2^-18 of the magnitudes
            const float mag = fmaxf(fmaxf(fmaxf(fabsf(b0x), fabsf(b1x)), fmaxf(fabsf(b0y), fabsf(b1y))),
                                    fmaxf(fabsf(b0z), fabsf(b1z)));
#pragma unroll 1
            for (uint32_t j0 = 0; j0 < ln0; j0 += 32) {
                const uint32_t j = j0 + lane;
                const uint32_t lj = j < ln0 ? __ldg(grid.lists + lb0 + j) : 0xffffffffu;
                const bool ok = lj < n_lights;
                if (j < ln0 && !ok) raise_status(status, HL_ERR_DEVICE_BOUNDS);
                const float4 c = ok ? __ldg(cand + lj) : make_float4(0, 0, 0, -1.0f);
                bool keep = ok && c.w < 0.0f;
                if (ok && c.w >= 0.0f) {
                    const float e = (mag + fabsf(c.x) + fabsf(c.y) + fabsf(c.z)) * (1.0f / 262144.0f);
                    const float dx = fmaxf(fmaxf(b0x - c.x, c.x - b1x) - e, 0.0f);
                    const float dy = fmaxf(fmaxf(b0y - c.y, c.y - b1y) - e, 0.0f);
                    const float dz = fmaxf(fmaxf(b0z - c.z, c.z - b1z) - e, 0.0f);
                    keep = fma_(dz, dz, fma_(dy, dy, dx * dx)) <= c.w * (1.0f + 1.0f / 256.0f);
                }
                uint32_t m = __ballot_sync(0xffffffffu, keep);
                while (m) {
                    const int bl = __ffs(m) - 1;
                    m &= m - 1;
                    const uint32_t li = __shfl_sync(0xffffffffu, lj, bl);
                    const float ax = __shfl_sync(0xffffffffu, c.x, bl), ay = __shfl_sync(0xffffffffu, c.y, bl),
                                az = __shfl_sync(0xffffffffu, c.z, bl), aw = __shfl_sync(0xffffffffu, c.w, bl);
                    const bool pass = own && (aw < 0.0f || candidate(px, py, pz, plx, ply, plz, nx, ny, nz, ax, ay, az,
                                                                     aw, slack, !STATS));
                    const uint32_t pm = __ballot_sync(0xffffffffu, pass);
                    if (pass) queue[(head + qlen + __popc(pm & lanemask_lt())) & (kQueue - 1)] = (i << 23) | li;
                    qlen += __popc(pm);
                    __syncwarp();
                    if (qlen >= 32) {
                        flush_batch<LAYOUT, STATS, TW, NPX, EXT>(s, queue, head, 32, lane, cam, lights, x0, y0, W, H, sv, log);
                        head += 32;
                        qlen -= 32;
                    }
                }
            }
        }
        constexpr int PIPE = PRECISE ? 2 : kPipe;  // the precise path keeps fewer loads in flight (registers)
        for (uint32_t j0 = 0; j0 < maxlen; j0 += PIPE) {
            uint32_t li[PIPE];
            float4 a[PIPE];
#pragma unroll
            for (int u = 0; u < PIPE; ++u) li[u] = (j0 + u < ln) ? __ldg(grid.lists + lb + j0 + u) : 0xffffffffu;
#pragma unroll
            for (int u = 0; u < PIPE; ++u) a[u] = li[u] < n_lights ? __ldg(cand + li[u]) : make_float4(0, 0, 0, 0);
#pragma unroll
            for (int u = 0; u < PIPE; ++u) {
                if (j0 + u >= maxlen) break;  // warp-uniform
                bool pass = false;
                if (j0 + u < ln) {
                    if (li[u] >= n_lights) {
                        raise_status(status, HL_ERR_DEVICE_BOUNDS);
                    } else if (a[u].w < 0.0f) {
                        pass = true;  // directional
                    } else {
                        pass = candidate(px, py, pz, plx, ply, plz, nx, ny, nz, a[u].x, a[u].y, a[u].z, a[u].w, slack,
                                         !STATS);
                    }
                }
                const uint32_t pm = __ballot_sync(0xffffffffu, pass);
                if (pass) queue[(head + qlen + __popc(pm & lanemask_lt())) & (kQueue - 1)] = (i << 23) | li[u];
                qlen += __popc(pm);
            }
            __syncwarp();
            while (qlen >= 32) {
                flush_batch<LAYOUT, STATS, TW, NPX, EXT>(s, queue, head, 32, lane, cam, lights, x0, y0, W, H, sv, log);
                head += 32;
                qlen -= 32;
            }
        }
    }
    if (qlen > 0) flush_batch<LAYOUT, STATS, TW, NPX, EXT>(s, queue, head, qlen, lane, cam, lights, x0, y0, W, H, sv, log);

    // ---- 5. output -----------------------------------------------------------------
    __syncthreads();
    const uint32_t debug_mode = glb->debug_mode;
    bool rc_ok = false;  // radiance-cascade GI bound and enabled
    if (EXT) rc_ok = sv->rc != nullptr && glb->has_rc_gi != 0u;
    const uint32_t lcount = glb->light_count;
    bool shadows_bound = false;
    if (EXT) shadows_bound = sv->dyn != nullptr;
    // the light-space projection view (mode 11) needs the shadow matrices
    if (!STATS && t == 0 && ((glb->has_rc_gi != 0u && !rc_ok) || (debug_mode == 11u && lcount > 0u && !shadows_bound)))
        raise_status(status, HL_ERR_NOT_SUPPORTED);
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const uint32_t i = t + k * kThreads;
        const uint32_t x = x0 + i % TW, y = y0 + i / TW;
        if (x >= gb.width || y >= gb.height) continue;
        if (STATS) {
            uint32_t* o = stats + (size_t(y) * gb.width + x) * 3;
            if (valid[k]) {
                o[0] = cnt[3][i];
                o[1] = cnt[1][i];
                o[2] = cnt[2][i];
            } else {
                o[0] = o[1] = o[2] = 0;
            }
            continue;
        }
        if (!valid[k]) continue;
        // albedo from the record; ao, emissive and alpha exist only in the reference layout
        Texel<LAYOUT> tx;
        if (LAYOUT == HL_GBUF_REFERENCE) {
            tx = load_texel<LAYOUT>(gb, x, y);
        } else {
            tx.ar = s.px[F_AR][i];
            tx.ag = s.px[F_AG][i];
            tx.ab = s.px[F_AB][i];
            tx.ao = 1.0f;
            tx.alpha = 1.0f;
            tx.er = tx.eg = tx.eb = 0.0f;
        }
        float nxo, ny, nzo;
        float in_;
        pixel_normal(s, i, nxo, ny, nzo, in_);
        const float amb = glb->ambient_intensity;
        const float skr = glb->ambient_color[0] * amb, skg = glb->ambient_color[1] * amb,
                    skb = glb->ambient_color[2] * amb;
        const float ht = fma_(ny, 0.5f, 0.5f);
        // hemisphere ambient (deferred_lighting.wgsl:1196-1199) times ao (x white SSAO)
        float hr = fma_(skr, ht, skr * 0.15f * (1.0f - ht)) * tx.ar;
        float hg = fma_(skg, ht, skg * 0.15f * (1.0f - ht)) * tx.ag;
        float hb = fma_(skb, ht, skb * 0.15f * (1.0f - ht)) * tx.ab;
        if (EXT && rc_ok) {
            // radiance-cascade indirect diffuse blended over the hemisphere ambient
            // (deferred_lighting.wgsl:1159-1163, 1197-1209)
            const float camx = cam->position_near[0], camy = cam->position_near[1], camz = cam->position_near[2];
            const float wx = PRECISE ? s.px[F_PX][i] + s.px[F_PLX][i] : camx + (s.px[F_PX][i] + s.px[F_PLX][i]);
            const float wy = PRECISE ? s.px[F_PY][i] + s.px[F_PLY][i] : camy + (s.px[F_PY][i] + s.px[F_PLY][i]);
            const float wz = PRECISE ? s.px[F_PZ][i] + s.px[F_PLZ][i] : camz + (s.px[F_PZ][i] + s.px[F_PLZ][i]);
            const float metal = s.px[F_METAL][i];
            float f0r, f0g, f0b;
            if (int(NF) > int(F_F0R)) {
                f0r = s.px[F_F0R][i]; f0g = s.px[F_F0G][i]; f0b = s.px[F_F0B][i];
            } else {
                f0r = metallic_f0(tx.ar, metal); f0g = metallic_f0(tx.ag, metal); f0b = metallic_f0(tx.ab, metal);
            }
            rc::ambient(*sv, glb, wx, wy, wz, nxo, ny, nzo, s.px[F_NDV][i], s.px[F_ROUGH][i], metal,
                        fmin_(fmax_(f0r, 0.0f), 0.999f), fmin_(fmax_(f0g, 0.0f), 0.999f), fmin_(fmax_(f0b, 0.0f), 0.999f),
                        tx.ar, tx.ag, tx.ab, hr, hg, hb);
        }
        float4 c;
        c.x = (s.acc[0][i] + fma_(hr, tx.ao, 0.0f)) + tx.er;
        c.y = (s.acc[1][i] + fma_(hg, tx.ao, 0.0f)) + tx.eg;
        c.z = (s.acc[2][i] + fma_(hb, tx.ao, 0.0f)) + tx.eb;
        c.w = tx.alpha;
        if (debug_mode == 1u || debug_mode == 2u || debug_mode == 4u || debug_mode == 20u || debug_mode == 21u) {
            c = make_float4(tx.ar, tx.ag, tx.ab, tx.alpha);
        } else if (debug_mode == 5u) {
            c = make_float4(fma_(nxo, 0.5f, 0.5f), fma_(ny, 0.5f, 0.5f), fma_(nzo, 0.5f, 0.5f),
                            1.0f);
        } else if (debug_mode == 10u) {
            // shadow factor heatmap (deferred_lighting.wgsl:1049-1064): the mean shadow
            // factor of the first light_count lights, 1 for a light without shadow maps
            const uint32_t nl = min(lcount, n_lights);
            float sum = 0.0f;
            if (EXT && shadows_bound) {
                // the pixel's world position rounded to f32, as the pair's shadow factor takes it
                float wx = s.px[F_PX][i] + s.px[F_PLX][i], wy = s.px[F_PY][i] + s.px[F_PLY][i],
                      wz = s.px[F_PZ][i] + s.px[F_PLZ][i];
                if (!PRECISE) {
                    float hx, hy, hz, lx, ly, lz;
                    reconstruct<true, false>(cam->inv_view_proj, x, y, W, H, fabsf(s.px[F_DEPTH][i]), hx, hy, hz, lx,
                                             ly, lz);
                    wx = hx + lx;
                    wy = hy + ly;
                    wz = hz + lz;
                }
                const float4 csm = __ldg(reinterpret_cast<const float4*>(sv->csm));
                for (uint32_t li = 0; li < nl; ++li) {
                    const float4* gl = reinterpret_cast<const float4*>(lights + li);
                    const float4 la = __ldg(gl + 0), lb = __ldg(gl + 1);
                    const uint4 ld = __ldg(reinterpret_cast<const uint4*>(gl + 3));
                    sum = xadd(sum, shadow_factor(*sv, li, la, lb, ld.x, ld.y, wx, wy, wz, nxo, ny, nzo,
                                                  float(x) + 0.5f, float(y) + 0.5f, camx, camy, camz, csm));
                }
            } else {
                for (uint32_t li = 0; li < nl; ++li) sum = xadd(sum, 1.0f);
            }
            sum = xadd(sum, float(lcount - nl));  // lights beyond the buffer: lit
            const float sf = xdiv(sum, xmax(float(lcount), 1.0f));
            c = make_float4(sf, sf, sf, 1.0f);
        } else if (EXT && debug_mode == 11u && lcount > 0u && shadows_bound) {
            c = shadow_projection_view(cam->inv_view_proj, sv->mats, x, y, W, H, fabsf(s.px[F_DEPTH][i]));
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
}

template <uint32_t LAYOUT, uint32_t GRID, uint32_t TARGET, bool STATS, int TW, int TH, bool EXT>
__global__ void __launch_bounds__(sk::kThreads, 3) shade_kernel(
    const GpuCamera* __restrict__ cam, const DeferredGlobals* __restrict__ glb, const GBufView gb,
    const GpuLight* __restrict__ lights, uint32_t n_lights, const GridView grid, const __grid_constant__ SliceTable tab,
    const TargetView out, uint32_t* __restrict__ stats, int* __restrict__ status, const float4* __restrict__ cand,
    const __grid_constant__ ExtView sv, const __grid_constant__ PairLog log) {
    shade_tile<LAYOUT, GRID, TARGET, STATS, TW, TH, true, EXT>(cam, glb, gb, lights, cand, n_lights, grid, tab.z,
                                                                  out, stats, status, blockIdx.x, blockIdx.y, &sv, log);
}

// Every tile of every view of a batch (froxel grids, 32x16 tiles): CTA b lights tile
// b - tile_start of the view whose [tile_start, next tile_start) holds b.
template <uint32_t LAYOUT, uint32_t TARGET>
__global__ void __launch_bounds__(sk::kThreads, 3) shade_batched_kernel(
    const ShadeViewDesc* __restrict__ d, uint32_t n_views, const DeferredGlobals* __restrict__ glb,
    const GpuLight* __restrict__ lights, uint32_t n_lights, int* __restrict__ status) {
    uint32_t lo = 0, hi = n_views;
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (__ldg(&d[mid].tile_start) <= blockIdx.x) lo = mid; else hi = mid;
    }
    const ShadeViewDesc& v = d[lo];
    const uint32_t local = blockIdx.x - v.tile_start;
    const GBufView gb = v.gb;
    const GridView grid = v.grid;
    const TargetView out = v.out;
    shade_tile<LAYOUT, HL_GRID_FROXELS, TARGET, false, 32, 16>(static_cast<const GpuCamera*>(v.camera), glb, gb, lights,
                                                               v.cand, n_lights, grid, v.tabz, out, nullptr, status,
                                                               local % v.tiles_x, local / v.tiles_x, nullptr,
                                                               PairLog{nullptr, nullptr, 0});
}

// The light table of the candidate tests: position (camera-relative on the FP16
// G-buffer's fast path, as the shading kernel computes it), and range^2 (1 + 2^-9), or
// -1 for a directional light.
__device__ __forceinline__ float4 cand_entry(const GpuCamera* __restrict__ cam, const GpuLight& l, bool relative) {
    const float4 a = *reinterpret_cast<const float4*>(l.position_range);
    float4 c;
    c.x = relative ? a.x - cam->position_near[0] : a.x;
    c.y = relative ? a.y - cam->position_near[1] : a.y;
    c.z = relative ? a.z - cam->position_near[2] : a.z;
    c.w = l.light_type == 0u ? -1.0f : a.w * a.w * (1.0f + 1.0f / 512.0f);
    return c;
}

// The light's largest colour channel times its intensity: with the attenuation it bounds
// the radiance that pbr_direct_light compares with its 0.002 cut.
__device__ __forceinline__ float cand_peak(const GpuLight& l) {
    const float4 c = *reinterpret_cast<const float4*>(l.color_intensity);
    return fmaxf(fmaxf(c.x, c.y), c.z) * c.w;
}

// Launched as a dependent of whatever precedes it (the binning, in a frame): it reads
// only the camera and the lights, and waits for its predecessor before it ends, so the
// shading kernel that waits for it also waits for the lists.
__global__ void __launch_bounds__(256) prep_cand_kernel(const GpuCamera* __restrict__ cam,
                                                        const GpuLight* __restrict__ lights, uint32_t n,
                                                        uint32_t relative, float4* __restrict__ out) {
    pdl_launch_dependents();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) {
        out[i] = cand_entry(cam, lights[i], relative != 0u);
        reinterpret_cast<float*>(out + n)[i] = cand_peak(lights[i]);
    }
    pdl_wait();
}

__global__ void __launch_bounds__(256) prep_cand_batched_kernel(const ShadeViewDesc* __restrict__ d,
                                                                const GpuLight* __restrict__ lights, uint32_t n,
                                                                uint32_t relative) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    const ShadeViewDesc& v = d[blockIdx.y];
    if (i < n) {
        v.cand[i] = cand_entry(static_cast<const GpuCamera*>(v.camera), lights[i], relative != 0u);
        reinterpret_cast<float*>(v.cand + n)[i] = cand_peak(lights[i]);
    }
}

template <uint32_t LAYOUT, uint32_t TARGET>
cudaError_t launch_batched(const ShadeViewDesc* descs, uint32_t n_views, uint32_t total_tiles, const void* globals,
                           const void* lights, uint32_t n, int* status, cudaStream_t stream) {
    auto kern = shade_batched_kernel<LAYOUT, TARGET>;
    const int smem = int(sizeof(sk::Smem<32 * 16, sk::record_fields<LAYOUT>()>));
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return e;
    if (n > 0) {
        prep_cand_batched_kernel<<<dim3((n + 255) / 256, n_views), 256, 0, stream>>>(
            descs, static_cast<const GpuLight*>(lights), n, LAYOUT == HL_GBUF_F16 ? 1u : 0u);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (LAYOUT == HL_GBUF_F16)  // the single-view FP16 path's tile code, so that every view matches it
        return launch_shade_f16_batched(TARGET, descs, n_views, total_tiles, globals, lights, n, status, stream);
    kern<<<total_tiles, sk::kThreads, smem, stream>>>(descs, n_views, static_cast<const DeferredGlobals*>(globals),
                                                      static_cast<const GpuLight*>(lights), n, status);
    return cudaGetLastError();
}

template <uint32_t LAYOUT, uint32_t GRID, uint32_t TARGET, bool STATS, bool EXT = false>
cudaError_t launch_one(const void* camera, const void* globals, const GBufView& gb, const void* lights, uint32_t n,
                       const GridView& grid, const SliceTable& tab, const TargetView& out, uint32_t* stats, int* status, float4* cand,
                       const PairLog& log, cudaStream_t stream, const ExtView* sv = nullptr) {
    constexpr bool FROXELS = (GRID == HL_GRID_FROXELS);
    constexpr int TW = FROXELS ? 32 : 16, TH = 16;
    auto kern = shade_kernel<LAYOUT, GRID, TARGET, STATS, TW, TH, EXT>;
    const int smem = int(sizeof(sk::Smem<TW * TH, sk::record_fields<LAYOUT>()>));
    static unsigned long long attr_devices = 0;  // devices on which the smem limit is raised
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !(attr_devices & (1ull << dev))) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr_devices |= 1ull << dev;
    }
    if (n > 0) {
        cudaError_t e = launch_pdl(prep_cand_kernel, dim3((n + 255) / 256), dim3(256), 0, stream,
                                   static_cast<const GpuCamera*>(camera), static_cast<const GpuLight*>(lights), n,
                                   LAYOUT == HL_GBUF_F16 ? 1u : 0u, cand);
        if (e != cudaSuccess) return e;
    }
    const dim3 g((gb.width + TW - 1) / TW, (gb.height + TH - 1) / TH);
    ExtView svv{};
    if (sv) svv = *sv;
    return launch_pdl(kern, g, dim3(sk::kThreads), smem, stream, static_cast<const GpuCamera*>(camera),
                      static_cast<const DeferredGlobals*>(globals), gb, static_cast<const GpuLight*>(lights), n, grid,
                      tab, out, stats, status, static_cast<const float4*>(cand), svv, log);
}

template <uint32_t LAYOUT, uint32_t GRID>
cudaError_t dispatch_target(uint32_t target, const void* camera, const void* globals, const GBufView& gb,
                            const void* lights, uint32_t n, const GridView& grid, const SliceTable& tab,
                            const TargetView& out, uint32_t* stats, int* status, float4* cand, const PairLog& log,
                            cudaStream_t stream, const ExtView* sv) {
    if (sv && !stats) {
        if (target == HL_TARGET_RGBA16F)
            return launch_one<LAYOUT, GRID, HL_TARGET_RGBA16F, false, true>(camera, globals, gb, lights, n, grid, tab,
                                                                            out, stats, status, cand, log, stream, sv);
        return launch_one<LAYOUT, GRID, HL_TARGET_RGBA32F, false, true>(camera, globals, gb, lights, n, grid, tab, out,
                                                                        stats, status, cand, log, stream, sv);
    }
    if (stats)
        return launch_one<LAYOUT, GRID, HL_TARGET_RGBA32F, true>(camera, globals, gb, lights, n, grid, tab, out, stats,
                                                                 status, cand, log, stream);
    if (target == HL_TARGET_RGBA16F)
        return launch_one<LAYOUT, GRID, HL_TARGET_RGBA16F, false>(camera, globals, gb, lights, n, grid, tab, out,
                                                                  stats, status, cand, log, stream);
    return launch_one<LAYOUT, GRID, HL_TARGET_RGBA32F, false>(camera, globals, gb, lights, n, grid, tab, out, stats,
                                                              status, cand, log, stream);
}

template <uint32_t LAYOUT>
cudaError_t dispatch_grid(uint32_t grid_kind, uint32_t target, const void* camera, const void* globals,
                          const GBufView& gb, const void* lights, uint32_t n, const GridView& grid,
                          const SliceTable& tab, const TargetView& out, uint32_t* stats, int* status, float4* cand,
                          const PairLog& log, cudaStream_t stream, const ExtView* sv) {
    if (grid_kind == HL_GRID_FROXELS)
        return dispatch_target<LAYOUT, HL_GRID_FROXELS>(target, camera, globals, gb, lights, n, grid, tab, out, stats,
                                                        status, cand, log, stream, sv);
    return dispatch_target<LAYOUT, HL_GRID_TILES>(target, camera, globals, gb, lights, n, grid, tab, out, stats,
                                                  status, cand, log, stream, sv);
}

}  // namespace

cudaError_t launch_prep_cand_batched(const ShadeViewDesc* descs, uint32_t n_views, const void* lights, uint32_t n,
                                     bool relative, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    prep_cand_batched_kernel<<<dim3((n + 255) / 256, n_views), 256, 0, stream>>>(
        descs, static_cast<const GpuLight*>(lights), n, relative ? 1u : 0u);
    return cudaGetLastError();
}

cudaError_t launch_prep_cand(const void* camera, const void* lights, uint32_t n, bool relative, float4* cand,
                             cudaStream_t stream) {
    return launch_pdl(prep_cand_kernel, dim3((n + 255) / 256), dim3(256), 0, stream,
                      static_cast<const GpuCamera*>(camera), static_cast<const GpuLight*>(lights), n,
                      relative ? 1u : 0u, cand);
}

cudaError_t launch_shade(uint32_t layout, uint32_t grid_kind, uint32_t target_format, const void* camera,
                         const void* globals, const GBufView& gb, const void* lights, uint32_t n_lights,
                         const GridView& grid, const SliceTable& tab, const TargetView& out, uint32_t* stats,
                         int* status, float4* cand, const PairLog& log, cudaStream_t stream,
                         const ExtView* shadows) {
    if (layout == HL_GBUF_F16 && grid_kind == HL_GRID_FROXELS && !stats && !shadows)
        return launch_shade_f16(target_format, camera, globals, gb, lights, n_lights, grid, tab, out, status, cand, log,
                                stream);
    switch (layout) {
        case HL_GBUF_REFERENCE:
            return dispatch_grid<HL_GBUF_REFERENCE>(grid_kind, target_format, camera, globals, gb, lights, n_lights,
                                                    grid, tab, out, stats, status, cand, log, stream, shadows);
        case HL_GBUF_F32:
            return dispatch_grid<HL_GBUF_F32>(grid_kind, target_format, camera, globals, gb, lights, n_lights, grid,
                                              tab, out, stats, status, cand, log, stream, shadows);
        default:
            return dispatch_grid<HL_GBUF_F16>(grid_kind, target_format, camera, globals, gb, lights, n_lights, grid,
                                              tab, out, stats, status, cand, log, stream, shadows);
    }
}

cudaError_t launch_shade_batched(uint32_t layout, uint32_t target_format, const ShadeViewDesc* descs,
                                 uint32_t n_views, uint32_t total_tiles, const void* globals, const void* lights,
                                 uint32_t n_lights, int* status, cudaStream_t stream) {
    const bool h = target_format == HL_TARGET_RGBA16F;
    switch (layout) {
        case HL_GBUF_REFERENCE:
            return h ? launch_batched<HL_GBUF_REFERENCE, HL_TARGET_RGBA16F>(descs, n_views, total_tiles, globals, lights,
                                                                           n_lights, status, stream)
                     : launch_batched<HL_GBUF_REFERENCE, HL_TARGET_RGBA32F>(descs, n_views, total_tiles, globals, lights,
                                                                           n_lights, status, stream);
        case HL_GBUF_F32:
            return h ? launch_batched<HL_GBUF_F32, HL_TARGET_RGBA16F>(descs, n_views, total_tiles, globals, lights,
                                                                     n_lights, status, stream)
                     : launch_batched<HL_GBUF_F32, HL_TARGET_RGBA32F>(descs, n_views, total_tiles, globals, lights,
                                                                     n_lights, status, stream);
        default:
            return h ? launch_batched<HL_GBUF_F16, HL_TARGET_RGBA16F>(descs, n_views, total_tiles, globals, lights,
                                                                     n_lights, status, stream)
                     : launch_batched<HL_GBUF_F16, HL_TARGET_RGBA32F>(descs, n_views, total_tiles, globals, lights,
                                                                     n_lights, status, stream);
    }
}

}  // namespace hl
