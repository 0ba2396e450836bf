// hl_bin.cu — light binning kernels for sm_103a.
//
//  * prep_bin_lights   : one thread per light, view-space centre/axis (exact f32 order)
//  * bin_tiles_ref     : the reference's tile culling (light_cull.wgsl:123-180), one
//                        warp per 16x16 tile, lanes test 32 lights at a time and append
//                        in light-index order with ballot/popc, cap 64
//  * bin_froxels<FILL> : one CTA per froxel column; block-ordered compaction of the
//                        column's lights into shared memory, then one warp per slice
//                        tests the column list against the slice box (count pass, then
//                        fill pass after an exclusive scan of the counts)
//  * scan_counts       : single-CTA exclusive scan of the per-froxel counts
//
// All floating-point work here uses correctly rounded __f*_rn operations in the
// documented order, so the lists are bit-identical to the f32 CPU restatement.
#include "hl_common.cuh"
#include "hl_internal.h"

namespace hl {

namespace {

constexpr int kBinWarps = 8;
constexpr int kBinThreads = kBinWarps * 32;

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm volatile("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// make_plane_from_ndc_edge (light_cull.wgsl:85-100)
__device__ __forceinline__ f3 plane_from_ndc_edge(float p00, float p11, float p0x, float p0y, float p1x, float p1y) {
    f3 r0 = xnormalize(mk3(xdiv(p0x, p00), xdiv(p0y, p11), -1.0f));
    f3 r1 = xnormalize(mk3(xdiv(p1x, p00), xdiv(p1y, p11), -1.0f));
    return xnormalize(xcross(r0, r1));
}

struct Planes {
    f3 n[4];
};

// Left, right, top, bottom planes of an NDC rectangle (light_cull.wgsl:148-151).
__device__ __forceinline__ Planes rect_planes(float p00, float p11, float left, float right, float top, float bottom) {
    Planes p;
    p.n[0] = plane_from_ndc_edge(p00, p11, left, bottom, left, top);
    p.n[1] = plane_from_ndc_edge(p00, p11, right, top, right, bottom);
    p.n[2] = plane_from_ndc_edge(p00, p11, left, top, right, top);
    p.n[3] = plane_from_ndc_edge(p00, p11, right, bottom, left, bottom);
    return p;
}

// sphere_inside_tile_frustum (light_cull.wgsl:105-117); plane w = 0.
__device__ __forceinline__ bool sphere_in_planes(const Planes& p, float cx, float cy, float cz, float r) {
    const f3 c = mk3(cx, cy, cz);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        float dist = xadd(xdot(p.n[i], c), 0.0f);
        if (dist < -r) return false;
    }
    return true;
}

// One light in the camera's view space, with its culling radius (widened for froxels).
__device__ __forceinline__ BinLight prep_light(const GpuCamera* __restrict__ cam, const GpuLight& l,
                                               uint32_t froxel_margin) {
    const float* v = cam->view;
    const float px = l.position_range[0], py = l.position_range[1], pz = l.position_range[2];
    BinLight b;
    b.cx = xmat_row(v, 0, px, py, pz, 1.0f);
    b.cy = xmat_row(v, 1, px, py, pz, 1.0f);
    b.cz = xmat_row(v, 2, px, py, pz, 1.0f);
    const float r = l.position_range[3];
    b.r = froxel_margin ? xadd(r, xmul(xadd(r, 1.0f), 1.0f / 1024.0f)) : r;
    const float dx = l.direction_outer[0], dy = l.direction_outer[1], dz = l.direction_outer[2];
    f3 a = xnormalize(mk3(xmat_row(v, 0, dx, dy, dz, 0.0f), xmat_row(v, 1, dx, dy, dz, 0.0f),
                          xmat_row(v, 2, dx, dy, dz, 0.0f)));
    b.ax = a.x;
    b.ay = a.y;
    b.az = a.z;
    b.cos_o = l.direction_outer[3];
    b.sin_o = xsqrt(xmax(xsub(1.0f, xmul(b.cos_o, b.cos_o)), 0.0f));
    b.type = l.light_type;
    b.cone = (l.light_type == 2u) && (0.0f < b.cos_o) && (b.cos_o < l.inner_angle);
    b.pad = 0;
    return b;
}

__global__ void __launch_bounds__(256) prep_bin_lights_kernel(const GpuCamera* __restrict__ cam,
                                                              const GpuLight* __restrict__ lights, uint32_t n,
                                                              uint32_t froxel_margin, BinLight* __restrict__ out) {
    pdl_launch_dependents();  // the binning kernel sets its column up meanwhile
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[i] = prep_light(cam, lights[i], froxel_margin);
}

// ----------------------------------------------------------------------------------
// Reference tile culling
// ----------------------------------------------------------------------------------
constexpr int kTileChunk = 1024;

__global__ void __launch_bounds__(kBinThreads) bin_tiles_ref_kernel(const GpuCamera* __restrict__ cam,
                                                                     const BinLight* __restrict__ bl, uint32_t n,
                                                                     uint32_t W, uint32_t H, uint32_t tiles_x,
                                                                     uint32_t tiles, uint32_t* __restrict__ lists,
                                                                     uint32_t* __restrict__ counts) {
    __shared__ float4 s_sph[kTileChunk];
    __shared__ uint32_t s_dir[kTileChunk];
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t tile = blockIdx.x * kBinWarps + warp;
    const bool active = tile < tiles;

    Planes planes;
    if (active) {
        const uint32_t tx = tile % tiles_x, ty = tile / tiles_x;
        const float fw = float(W), fh = float(H), ts = float(kTile);
        // light_cull.wgsl:136-143
        const float left = xsub(xmul(xdiv(xmul(float(tx), ts), fw), 2.0f), 1.0f);
        const float right = xmin(xsub(xmul(xdiv(xmul(float(tx + 1), ts), fw), 2.0f), 1.0f), 1.0f);
        const float top = xsub(1.0f, xmul(xdiv(xmul(float(ty), ts), fh), 2.0f));
        const float bottom = xmax(xsub(1.0f, xmul(xdiv(xmul(float(ty + 1), ts), fh), 2.0f)), -1.0f);
        planes = rect_planes(cam->proj[0], cam->proj[5], left, right, top, bottom);
    }
    uint32_t count = 0;
    bool done = !active;
    uint32_t* out = lists + size_t(tile) * kMaxPerTile;
    for (uint32_t base = 0; base < n; base += kTileChunk) {
        const uint32_t len = min(uint32_t(kTileChunk), n - base);
        __syncthreads();
        for (uint32_t j = threadIdx.x; j < len; j += blockDim.x) {
            const BinLight b = bl[base + j];
            s_sph[j] = make_float4(b.cx, b.cy, b.cz, b.r);
            s_dir[j] = (b.type == 0u);
        }
        __syncthreads();
        if (done) continue;
        for (uint32_t j0 = 0; j0 < len; j0 += 32) {
            const uint32_t j = j0 + lane;
            bool pass = false;
            if (j < len) {
                if (s_dir[j]) {
                    pass = true;
                } else {
                    const float4 s = s_sph[j];
                    pass = sphere_in_planes(planes, s.x, s.y, s.z, s.w);
                }
            }
            const uint32_t mask = __ballot_sync(0xffffffffu, pass);
            const uint32_t slot = count + __popc(mask & lanemask_lt());
            if (pass && slot < kMaxPerTile) out[slot] = base + j;
            count += __popc(mask);
            if (count >= kMaxPerTile) {
                count = kMaxPerTile;
                done = true;
                break;
            }
        }
    }
    if (active && lane == 0) counts[tile] = count;
}

// ----------------------------------------------------------------------------------
// Froxel clustering
// ----------------------------------------------------------------------------------
constexpr int kColCap = 4096;  // column-list entries held in shared memory per round
constexpr uint32_t kGatherU = 4;  // 256-light sub-rounds per gather step

struct ColumnGeom {
    Planes planes;
    float kx0, kx1, ky_bot, ky_top;
};

__device__ __forceinline__ uint32_t ceil_div_u64(uint64_t a, uint64_t b) { return uint32_t((a + b - 1) / b); }

__device__ __forceinline__ ColumnGeom column_geom(const GpuCamera* cam, const hl_froxel_params& p, uint32_t fx,
                                                  uint32_t fy) {
    const uint32_t px0 = ceil_div_u64(uint64_t(fx) * p.width, p.grid_x);
    const uint32_t px1 = ceil_div_u64(uint64_t(fx + 1) * p.width, p.grid_x);
    const uint32_t py0 = ceil_div_u64(uint64_t(fy) * p.height, p.grid_y);
    const uint32_t py1 = ceil_div_u64(uint64_t(fy + 1) * p.height, p.grid_y);
    const float fw = float(p.width), fh = float(p.height);
    const float left = xsub(xmul(xdiv(float(px0), fw), 2.0f), 1.0f);
    const float right = xsub(xmul(xdiv(float(px1), fw), 2.0f), 1.0f);
    const float top = xsub(1.0f, xmul(xdiv(float(py0), fh), 2.0f));
    const float bottom = xsub(1.0f, xmul(xdiv(float(py1), fh), 2.0f));
    const float p00 = cam->proj[0], p11 = cam->proj[5];
    ColumnGeom g;
    g.planes = rect_planes(p00, p11, left, right, top, bottom);
    g.kx0 = xdiv(left, p00);
    g.kx1 = xdiv(right, p00);
    g.ky_bot = xdiv(bottom, p11);
    g.ky_top = xdiv(top, p11);
    return g;
}

struct Box {
    float lox, loy, loz, hix, hiy, hiz;
    float cx, cy, cz, radius;
};

__device__ __forceinline__ Box froxel_box(const ColumnGeom& g, float z0, float z1) {
    Box b;
    const float m = xadd(xmul(z1, 1.0f / 1024.0f), 1.0f / 4096.0f);
    b.lox = xsub(xmin(xmul(g.kx0, z0), xmul(g.kx0, z1)), m);
    b.hix = xadd(xmax(xmul(g.kx1, z0), xmul(g.kx1, z1)), m);
    b.loy = xsub(xmin(xmul(g.ky_bot, z0), xmul(g.ky_bot, z1)), m);
    b.hiy = xadd(xmax(xmul(g.ky_top, z0), xmul(g.ky_top, z1)), m);
    b.loz = xsub(-z1, m);
    b.hiz = xadd(-z0, m);
    b.cx = xmul(xadd(b.lox, b.hix), 0.5f);
    b.cy = xmul(xadd(b.loy, b.hiy), 0.5f);
    b.cz = xmul(xadd(b.loz, b.hiz), 0.5f);
    const f3 e = mk3(xsub(b.hix, b.lox), xsub(b.hiy, b.loy), xsub(b.hiz, b.loz));
    b.radius = xmul(xsqrt(xdot(e, e)), 0.5f);
    return b;
}

__device__ __forceinline__ float axis_gap(float c, float lo, float hi) {
    return c < lo ? xsub(lo, c) : (hi < c ? xsub(c, hi) : 0.0f);
}

__device__ __forceinline__ bool light_meets_froxel(const BinLight& l, const Box& b) {
    if (l.type == 0u) return true;
    const float dx = axis_gap(l.cx, b.lox, b.hix);
    const float dy = axis_gap(l.cy, b.loy, b.hiy);
    const float dz = axis_gap(l.cz, b.loz, b.hiz);
    const float d2 = xadd(xadd(xmul(dx, dx), xmul(dy, dy)), xmul(dz, dz));
    if (!(d2 <= xmul(l.r, l.r))) return false;
    if (l.cone) {
        const f3 v = mk3(xsub(b.cx, l.cx), xsub(b.cy, l.cy), xsub(b.cz, l.cz));
        const float vlen2 = xdot(v, v);
        const float v1 = xdot(v, mk3(l.ax, l.ay, l.az));
        const float closest = xsub(xmul(l.cos_o, xsqrt(xmax(xsub(vlen2, xmul(v1, v1)), 0.0f))), xmul(v1, l.sin_o));
        if (closest > b.radius) return false;
        if (v1 > xadd(b.radius, l.r)) return false;
        if (v1 < -b.radius) return false;
    }
    return true;
}

struct BinSmem {
    uint32_t col[kColCap];
    uint32_t warp_tot[kGatherU * kBinWarps];
    uint32_t slice_run[kMaxSlices];
};

// One froxel column (col_id) of one view: count (FILL = false) or fill its slices.
template <bool FILL>
__device__ __forceinline__ void bin_column(BinSmem& sm, const GpuCamera* __restrict__ cam,
                                           const BinLight* __restrict__ bl, uint32_t n, const hl_froxel_params& p,
                                           const float* __restrict__ tabz, uint32_t col_id,
                                           uint32_t* __restrict__ counts, const uint32_t* __restrict__ offsets,
                                           uint32_t* __restrict__ indices, uint32_t capacity, int* __restrict__ status) {
    uint32_t* s_col = sm.col;
    uint32_t* s_warp_tot = sm.warp_tot;
    uint32_t* s_slice_run = sm.slice_run;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t fx = col_id % p.grid_x, fy = col_id / p.grid_x;
    const ColumnGeom g = column_geom(cam, p, fx, fy);
    const float zlast = xmax(tabz[p.grid_z], cam->forward_far[3]);
    for (uint32_t s = threadIdx.x; s < p.grid_z; s += blockDim.x) s_slice_run[s] = 0;

    uint32_t col_len = 0;
    uint32_t base = 0;
    while (true) {
        // ---- gather the next round of the column list (light-index order) ----
        __syncthreads();
        col_len = 0;
        while (base < n && col_len + kBinThreads <= kColCap) {
            const uint32_t i = base + threadIdx.x;
            bool pass = false;
            if (i < n) {
                const BinLight l = bl[i];
                pass = (l.type == 0u) || sphere_in_planes(g.planes, l.cx, l.cy, l.cz, l.r);
            }
            const uint32_t mask = __ballot_sync(0xffffffffu, pass);
            if (lane == 0) s_warp_tot[warp] = __popc(mask);
            __syncthreads();
            uint32_t before = 0, total = 0;
#pragma unroll
            for (int w = 0; w < kBinWarps; ++w) {
                const uint32_t t = s_warp_tot[w];
                before += (uint32_t(w) < warp) ? t : 0u;
                total += t;
            }
            if (pass) s_col[col_len + before + __popc(mask & lanemask_lt())] = i;
            col_len += total;
            base += kBinThreads;
            __syncthreads();
        }
        // ---- one warp per slice: test the column list against the slice box ----
        for (uint32_t s = warp; s < p.grid_z; s += kBinWarps) {
            const float z0 = tabz[s];
            const float z1 = (s + 1 == p.grid_z) ? zlast : tabz[s + 1];
            const Box b = froxel_box(g, z0, z1);
            const uint32_t f = col_id * p.grid_z + s;
            uint32_t run = s_slice_run[s];
            const uint32_t dst0 = FILL ? offsets[f] : 0u;
            for (uint32_t j0 = 0; j0 < col_len; j0 += 32) {
                const uint32_t j = j0 + lane;
                bool pass = false;
                uint32_t li = 0;
                if (j < col_len) {
                    li = s_col[j];
                    pass = light_meets_froxel(bl[li], b);
                }
                const uint32_t mask = __ballot_sync(0xffffffffu, pass);
                if (FILL && pass) {
                    const uint64_t dst = uint64_t(dst0) + run + __popc(mask & lanemask_lt());
                    if (dst < capacity) indices[dst] = li;
                }
                run += __popc(mask);
            }
            if (lane == 0) s_slice_run[s] = run;
        }
        if (base >= n) break;
    }
    __syncthreads();
    if (!FILL) {
        for (uint32_t s = threadIdx.x; s < p.grid_z; s += blockDim.x) counts[col_id * p.grid_z + s] = s_slice_run[s];
    } else if (threadIdx.x == 0 && status) {
        const uint32_t f_last = col_id * p.grid_z + p.grid_z - 1;
        if (uint64_t(offsets[f_last]) + s_slice_run[p.grid_z - 1] > capacity) raise_status(status, HL_ERR_CAPACITY);
    }
}

template <bool FILL>
__global__ void __launch_bounds__(kBinThreads) bin_froxels_kernel(const GpuCamera* __restrict__ cam,
                                                                   const BinLight* __restrict__ bl, uint32_t n,
                                                                   hl_froxel_params p, const __grid_constant__ SliceTable tab,
                                                                   uint32_t* __restrict__ counts,
                                                                   const uint32_t* __restrict__ offsets,
                                                                   uint32_t* __restrict__ indices, uint32_t capacity,
                                                                   int* __restrict__ status) {
    __shared__ BinSmem sm;
    bin_column<FILL>(sm, cam, bl, n, p, tab.z, blockIdx.x, counts, offsets, indices, capacity, status);
}

// ---- single pass: count, chained scan across columns, fill — one launch ----------
//
// Each CTA takes a column by ticket (a device counter, so CTA k waits only for columns
// that started before it), counts its slices, publishes its total, finds the entries
// of all earlier columns by looking back along the chain of published totals
// (decoupled look-back: a predecessor's inclusive prefix ends the walk, its bare total
// is added and the walk goes on), publishes its own inclusive prefix, writes its
// offsets and fills its lists. Chain words hold epoch << 32 | state << 30 | value; a
// word of another launch's epoch reads as "not yet published". The ticket base and the
// epoch live on the device and the last CTA of a launch advances them, so a launch
// recorded in a CUDA graph can be replayed.
constexpr uint32_t kFlagAggregate = 1u, kFlagPrefix = 2u;
constexpr uint32_t kChainValueMax = (1u << 30) - 1u;
constexpr uint32_t kLookbackSpins = 1u << 20;  // ~0.1 s of polling before HL_ERR_TIMEOUT

constexpr uint32_t kMaskCap = 4096;  // (slice, 32-light chunk) results kept from the count for the fill

struct FusedSmem {
    BinSmem b;
    uint32_t slice_dst[kMaxSlices];  // first entry of each slice of this column
    uint32_t mask[kMaskCap];         // ballot of chunk c of slice s at [s * chunks + c]
    uint32_t col, excl, total;
};

__device__ __forceinline__ unsigned long long ld_chain(const unsigned long long* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}

__device__ __forceinline__ void st_chain(unsigned long long* p, uint32_t epoch, uint32_t state, uint32_t value) {
    __threadfence();
    *reinterpret_cast<volatile unsigned long long*>(p) =
        (static_cast<unsigned long long>(epoch) << 32) | (state << 30) | min(value, kChainValueMax);
}

// Appends to sm.col, in light-index order, the lights from `base` on that may touch the
// column (directional, or a sphere not outside its four planes), until the lights run out
// or the next step could overflow kColCap. A step tests kGatherU x 256 lights, their
// loads in flight together, with two barriers.
__device__ __forceinline__ uint32_t gather_round(BinSmem& sm, const ColumnGeom& g, const BinLight* __restrict__ bl,
                                                 uint32_t n, uint32_t& base) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t col_len = 0;
    __syncthreads();
    while (base < n && col_len + kGatherU * kBinThreads <= kColCap) {
        bool pass[kGatherU];
        uint32_t mask[kGatherU];
#pragma unroll
        for (uint32_t u = 0; u < kGatherU; ++u) {
            const uint32_t i = base + u * kBinThreads + threadIdx.x;
            pass[u] = false;
            if (i < n) {
                const BinLight l = bl[i];
                pass[u] = (l.type == 0u) || sphere_in_planes(g.planes, l.cx, l.cy, l.cz, l.r);
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < kGatherU; ++u) {
            mask[u] = __ballot_sync(0xffffffffu, pass[u]);
            if (lane == 0) sm.warp_tot[u * kBinWarps + warp] = __popc(mask[u]);
        }
        __syncthreads();
#pragma unroll
        for (uint32_t u = 0; u < kGatherU; ++u) {
            uint32_t before = 0, total = 0;
#pragma unroll
            for (int w = 0; w < kBinWarps; ++w) {
                const uint32_t t = sm.warp_tot[u * kBinWarps + w];
                before += (uint32_t(w) < warp) ? t : 0u;
                total += t;
            }
            if (pass[u]) sm.col[col_len + before + __popc(mask[u] & lanemask_lt())] = base + u * kBinThreads + threadIdx.x;
            col_len += total;
        }
        base += kGatherU * kBinThreads;
        __syncthreads();
    }
    return col_len;
}

// Tests a gathered round against every slice box of the column: counts into
// sm.slice_run, and with FILL writes the lists from sm.slice_dst. A warp takes a slice
// and four 32-light chunks at a time, their light loads in flight together. With MASKS
// the count keeps each chunk's ballot and the fill replays them instead of testing again.
template <bool FILL>
__device__ __forceinline__ void test_slices(FusedSmem& fs, const ColumnGeom& g, const BinLight* __restrict__ bl,
                                            const hl_froxel_params& p, const float* __restrict__ tabz, float zlast,
                                            uint32_t col_len, uint32_t* __restrict__ indices, uint32_t capacity,
                                            bool masks) {
    constexpr uint32_t kU = 4;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t chunks = (col_len + 31) / 32;
    for (uint32_t s = warp; s < p.grid_z; s += kBinWarps) {
        uint32_t run = fs.b.slice_run[s];
        const uint32_t dst0 = FILL ? fs.slice_dst[s] : 0u;
        uint32_t* sm_mask = fs.mask + s * chunks;
        if (FILL && masks) {
            for (uint32_t c = 0; c < chunks; ++c) {
                const uint32_t mask = sm_mask[c];
                if ((mask >> lane) & 1u) {
                    const uint64_t dst = uint64_t(dst0) + run + __popc(mask & lanemask_lt());
                    if (dst < capacity) indices[dst] = fs.b.col[c * 32 + lane];
                }
                run += __popc(mask);
            }
        } else {
            const float z0 = tabz[s];
            const float z1 = (s + 1 == p.grid_z) ? zlast : tabz[s + 1];
            const Box b = froxel_box(g, z0, z1);
            for (uint32_t c0 = 0; c0 < chunks; c0 += kU) {
                uint32_t li[kU];
                BinLight l[kU];
#pragma unroll
                for (uint32_t u = 0; u < kU; ++u) {
                    const uint32_t j = (c0 + u) * 32 + lane;
                    li[u] = j < col_len ? fs.b.col[j] : 0xffffffffu;
                    if (li[u] != 0xffffffffu) l[u] = bl[li[u]];
                }
#pragma unroll
                for (uint32_t u = 0; u < kU; ++u) {
                    if (c0 + u >= chunks) break;  // warp-uniform
                    const bool pass = li[u] != 0xffffffffu && light_meets_froxel(l[u], b);
                    const uint32_t mask = __ballot_sync(0xffffffffu, pass);
                    if (FILL && pass) {
                        const uint64_t dst = uint64_t(dst0) + run + __popc(mask & lanemask_lt());
                        if (dst < capacity) indices[dst] = li[u];
                    }
                    if (!FILL && masks && lane == 0) sm_mask[c0 + u] = mask;
                    run += __popc(mask);
                }
            }
        }
        if (lane == 0) fs.b.slice_run[s] = run;
    }
}

__global__ void __launch_bounds__(kBinThreads) bin_froxels_fused_kernel(
    const GpuCamera* __restrict__ cam, const BinLight* __restrict__ bl, uint32_t n, hl_froxel_params p,
    const __grid_constant__ SliceTable tab, uint32_t* __restrict__ offsets, uint32_t* __restrict__ indices,
    uint32_t capacity, int* __restrict__ status, unsigned long long* __restrict__ chain,
    BinChainState* __restrict__ state) {
    __shared__ FusedSmem fs;
    __shared__ uint32_t s_epoch;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t cols = p.grid_x * p.grid_y;
    if (threadIdx.x == 0) {
        // every CTA of the previous launch has finished before this one starts (stream
        // order), so base and epoch are that launch's final values
        const unsigned long long base = *reinterpret_cast<volatile unsigned long long*>(&state->base);
        s_epoch = *reinterpret_cast<volatile uint32_t*>(&state->epoch) + 1u;
        fs.col = uint32_t(atomicAdd(&state->ticket, 1ull) - base);
    }
    __syncthreads();
    const uint32_t col = fs.col, epoch = s_epoch;
    if (col >= cols) {  // launches overlapping on one context: refused
        if (threadIdx.x == 0) raise_status(status, HL_ERR_DEVICE_BOUNDS);
        return;
    }
    const ColumnGeom g = column_geom(cam, p, col % p.grid_x, col / p.grid_x);
    const float zlast = xmax(tab.z[p.grid_z], cam->forward_far[3]);
    for (uint32_t s = threadIdx.x; s < p.grid_z; s += blockDim.x) fs.b.slice_run[s] = 0;
    pdl_launch_dependents();  // the shading launch's light table and pixel set-up may start
    pdl_wait();               // the view-space lights are written

    // ---- 1. count ----
    uint32_t base = 0, col_len = 0;
    bool one_round = true, masks = false;
    for (bool first = true;; first = false) {
        col_len = gather_round(fs.b, g, bl, n, base);
        if (!first) one_round = false;
        // a column gathered in one round keeps its chunk ballots when they fit
        masks = one_round && base >= n && p.grid_z * ((col_len + 31) / 32) <= kMaskCap;
        test_slices<false>(fs, g, bl, p, tab.z, zlast, col_len, indices, capacity, masks);
        if (base >= n) break;
    }
    __syncthreads();

    // ---- 2. chained scan over columns ----
    if (warp == 0) {
        if (lane == 0) {
            uint32_t acc = 0;
            for (uint32_t s = 0; s < p.grid_z; ++s) {
                fs.slice_dst[s] = acc;
                acc += fs.b.slice_run[s];
            }
            fs.total = acc;
            st_chain(chain + col, epoch, col == 0 ? kFlagPrefix : kFlagAggregate, acc);
        }
        __syncwarp();
        uint32_t excl = 0;
        int32_t pred = int32_t(col) - 1;
        uint32_t spins = 0;
        while (pred >= 0) {
            const int32_t c = pred - int32_t(lane);
            uint32_t st = kFlagPrefix, val = 0;  // before column 0: a prefix of 0
            if (c >= 0) {
                const unsigned long long w = ld_chain(chain + c);
                st = uint32_t(w >> 32) == epoch ? (uint32_t(w) >> 30) : 0u;
                val = uint32_t(w) & kChainValueMax;
            }
            const uint32_t pm = __ballot_sync(0xffffffffu, st == kFlagPrefix);
            const int stop = pm ? __ffs(pm) - 1 : 31;  // lanes 0..stop are summed
            const uint32_t upto = stop == 31 ? 0xffffffffu : ((2u << stop) - 1u);
            if (__ballot_sync(0xffffffffu, st == 0u) & upto) {
                if (++spins > kLookbackSpins) {
                    if (lane == 0) raise_status(status, HL_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(64);
                continue;
            }
            excl += __reduce_add_sync(0xffffffffu, uint32_t(lane) <= uint32_t(stop) ? val : 0u);
            if (pm) break;
            pred -= 32;
        }
        if (lane == 0) {
            if (col > 0) st_chain(chain + col, epoch, kFlagPrefix, excl + fs.total);
            fs.excl = excl;
            if (uint64_t(excl) + fs.total > capacity) raise_status(status, HL_ERR_CAPACITY);
            if (uint64_t(excl) + fs.total > kChainValueMax) raise_status(status, HL_ERR_SIZE);
        }
    }
    __syncthreads();
    const uint32_t excl = fs.excl;
    for (uint32_t s = threadIdx.x; s < p.grid_z; s += blockDim.x) {
        fs.slice_dst[s] += excl;
        offsets[col * p.grid_z + s] = fs.slice_dst[s];
        fs.b.slice_run[s] = 0;
    }
    if (col == cols - 1 && threadIdx.x == 0) offsets[cols * p.grid_z] = excl + fs.total;
    __syncthreads();

    // ---- 3. fill (from the round still in shared memory when there was only one) ----
    if (one_round) {
        test_slices<true>(fs, g, bl, p, tab.z, zlast, col_len, indices, capacity, masks);
    } else {
        base = 0;
        for (;;) {
            col_len = gather_round(fs.b, g, bl, n, base);
            test_slices<true>(fs, g, bl, p, tab.z, zlast, col_len, indices, capacity, false);
            if (base >= n) break;
        }
    }
    // the last CTA to finish advances the ticket base and the epoch for the next launch
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&state->done, 1u) == cols - 1u) {
            state->done = 0u;
            state->base += cols;
            state->epoch = epoch;
            __threadfence();
        }
    }
}

// Exclusive scan of counts[F] into offsets[F+1] by one CTA of 1024 threads.
__device__ __forceinline__ void scan_counts(const uint32_t* __restrict__ counts, uint32_t F,
                                            uint32_t* __restrict__ offsets, uint32_t* s_warp) {
    const uint32_t t = threadIdx.x;
    const uint32_t per = (F + 1023) / 1024;
    const uint32_t b = min(F, t * per), e = min(F, b + per);
    uint32_t sum = 0;
    for (uint32_t i = b; i < e; ++i) sum += counts[i];
    // block exclusive scan of per-thread sums
    uint32_t x = sum;
    const uint32_t lane = t & 31, warp = t >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= uint32_t(o)) x += y;
    }
    if (lane == 31) s_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        uint32_t w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= uint32_t(o)) w += y;
        }
        s_warp[lane] = w;
    }
    __syncthreads();
    uint32_t run = x - sum + (warp ? s_warp[warp - 1] : 0u);
    for (uint32_t i = b; i < e; ++i) {
        offsets[i] = run;
        run += counts[i];
    }
    if (t == 1023) offsets[F] = run;
}

__global__ void __launch_bounds__(1024) scan_counts_kernel(const uint32_t* __restrict__ counts, uint32_t F,
                                                           uint32_t* __restrict__ offsets) {
    __shared__ uint32_t s_warp[32];
    scan_counts(counts, F, offsets, s_warp);
}

// ---- batched views: the same passes over every view of a batch in one launch each ----

__device__ __forceinline__ uint32_t find_view(const BinViewDesc* __restrict__ d, uint32_t n_views, uint32_t col) {
    uint32_t lo = 0, hi = n_views;  // largest v with d[v].col_start <= col
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) / 2;
        if (__ldg(&d[mid].col_start) <= col) lo = mid; else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(256) prep_bin_lights_batched_kernel(const BinViewDesc* __restrict__ d,
                                                                      const GpuLight* __restrict__ lights, uint32_t n) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const BinViewDesc& v = d[blockIdx.y];
    v.bl[i] = prep_light(static_cast<const GpuCamera*>(v.camera), lights[i], 1u);
}

template <bool FILL>
__global__ void __launch_bounds__(kBinThreads) bin_froxels_batched_kernel(const BinViewDesc* __restrict__ d,
                                                                           uint32_t n_views, uint32_t n,
                                                                           int* __restrict__ status) {
    __shared__ BinSmem sm;
    const uint32_t v = find_view(d, n_views, blockIdx.x);
    const BinViewDesc& vd = d[v];
    const hl_froxel_params p = vd.p;
    bin_column<FILL>(sm, static_cast<const GpuCamera*>(vd.camera), vd.bl, n, p, vd.tab.z, blockIdx.x - vd.col_start,
                     vd.counts, vd.offsets, vd.indices, vd.capacity, status);
}

__global__ void __launch_bounds__(1024) scan_counts_batched_kernel(const BinViewDesc* __restrict__ d) {
    __shared__ uint32_t s_warp[32];
    const BinViewDesc& v = d[blockIdx.x];
    scan_counts(v.counts, v.p.grid_x * v.p.grid_y * v.p.grid_z, v.offsets, s_warp);
}

}  // namespace

// ----------------------------------------------------------------------------------
// Launchers
// ----------------------------------------------------------------------------------
cudaError_t launch_prep_bin_lights(const void* camera, const void* lights, uint32_t n, bool froxel_margin,
                                   BinLight* out, cudaStream_t stream) {
    if (n == 0) return cudaSuccess;
    prep_bin_lights_kernel<<<(n + 255) / 256, 256, 0, stream>>>(static_cast<const GpuCamera*>(camera),
                                                                 static_cast<const GpuLight*>(lights), n,
                                                                 froxel_margin ? 1u : 0u, out);
    return cudaGetLastError();
}

cudaError_t launch_bin_tiles_ref(const void* camera, const BinLight* bl, uint32_t n, uint32_t W, uint32_t H,
                                 uint32_t* lists, uint32_t* counts, cudaStream_t stream) {
    const uint32_t tiles_x = (W + kTile - 1) / kTile, tiles_y = (H + kTile - 1) / kTile;
    const uint32_t tiles = tiles_x * tiles_y;
    const uint32_t grid = (tiles + kBinWarps - 1) / kBinWarps;
    bin_tiles_ref_kernel<<<grid, kBinThreads, 0, stream>>>(static_cast<const GpuCamera*>(camera), bl, n, W, H, tiles_x,
                                                           tiles, lists, counts);
    return cudaGetLastError();
}

cudaError_t launch_bin_froxels(const void* camera, const BinLight* bl, uint32_t n, const hl_froxel_params& p,
                               const SliceTable& tab, uint32_t* counts_scratch, uint32_t* offsets,
                               uint32_t* indices, uint32_t capacity, int* status, cudaStream_t stream) {
    const uint32_t cols = p.grid_x * p.grid_y;
    const uint32_t F = cols * p.grid_z;
    const GpuCamera* cam = static_cast<const GpuCamera*>(camera);
    bin_froxels_kernel<false><<<cols, kBinThreads, 0, stream>>>(cam, bl, n, p, tab, counts_scratch, nullptr, nullptr,
                                                                0, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    scan_counts_kernel<<<1, 1024, 0, stream>>>(counts_scratch, F, offsets);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    bin_froxels_kernel<true><<<cols, kBinThreads, 0, stream>>>(cam, bl, n, p, tab, nullptr, offsets, indices, capacity,
                                                               status);
    return cudaGetLastError();
}

cudaError_t launch_bin_froxels_batched(const BinViewDesc* descs, uint32_t n_views, uint32_t total_columns,
                                       const void* lights, uint32_t n, int* status, cudaStream_t stream) {
    if (n > 0) {
        prep_bin_lights_batched_kernel<<<dim3((n + 255) / 256, n_views), 256, 0, stream>>>(
            descs, static_cast<const GpuLight*>(lights), n);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    bin_froxels_batched_kernel<false><<<total_columns, kBinThreads, 0, stream>>>(descs, n_views, n, status);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    scan_counts_batched_kernel<<<n_views, 1024, 0, stream>>>(descs);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    bin_froxels_batched_kernel<true><<<total_columns, kBinThreads, 0, stream>>>(descs, n_views, n, status);
    return cudaGetLastError();
}

cudaError_t launch_bin_froxels_fused(const void* camera, const BinLight* bl, uint32_t n, const hl_froxel_params& p,
                                     const SliceTable& tab, uint32_t* offsets, uint32_t* indices, uint32_t capacity,
                                     int* status, unsigned long long* chain, BinChainState* state,
                                     cudaStream_t stream) {
    const uint32_t cols = p.grid_x * p.grid_y;
    // as a dependent launch only right after this call's light preparation: two binning
    // launches of one context must never overlap (ticket and epoch)
    if (n > 0)
        return launch_pdl(bin_froxels_fused_kernel, dim3(cols), dim3(kBinThreads), 0, stream,
                          static_cast<const GpuCamera*>(camera), bl, n, p, tab, offsets, indices, capacity, status,
                          chain, state);
    bin_froxels_fused_kernel<<<cols, kBinThreads, 0, stream>>>(static_cast<const GpuCamera*>(camera), bl, n, p, tab,
                                                               offsets, indices, capacity, status, chain, state);
    return cudaGetLastError();
}

}  // namespace hl
