// hl_bin_item.cuh — froxel binning of one work item (a froxel column, or a group of
// its slices) as device code shared by the single-launch binning of hl_bin_froxels and
// the persistent batched launch, plus the light-culling geometry both binning paths
// use: the reference's tile planes (light_cull.wgsl:85-117), the view-space light
// record and the froxel box tests. All floating-point work uses correctly rounded
// __f*_rn operations in the documented order, so the lists are bit-identical to the
// f32 CPU restatement.
#pragma once

#include "hl_common.cuh"

namespace hl {
namespace bin {

constexpr int kWarps = 8;
constexpr int kThreads = kWarps * 32;

// Asks for the 128-byte line at p in this SM's L1 (no register written, no fault on
// any address the caller may read).
__device__ __forceinline__ void prefetch_l1(const void* p) {
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

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

// The three rows of the camera's view matrix that map a point to view space, held in
// registers by code that transforms many lights (column-major: element (r, c) at
// m[4 c + r]; row r is m[r], m[4 + r], m[8 + r], m[12 + r]).
struct ViewRows {
    float m[3][4];
};

__device__ __forceinline__ ViewRows load_view_rows(const GpuCamera* __restrict__ cam) {
    ViewRows v;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) v.m[r][c] = __ldg(&cam->view[4 * c + r]);
    return v;
}

// xmat_row over ViewRows: the same operations in the same order.
__device__ __forceinline__ float view_row(const ViewRows& v, int r, float x, float y, float z, float w) {
    return xadd(xadd(xadd(xmul(v.m[r][0], x), xmul(v.m[r][1], y)), xmul(v.m[r][2], z)), xmul(v.m[r][3], w));
}

// The centre, culling radius and type of a light's BinLight (prep_light's first half):
// all a column test needs.
__device__ __forceinline__ void prep_light_centre(const ViewRows& v, float4 pr, uint32_t type, BinLight& b) {
    b.cx = view_row(v, 0, pr.x, pr.y, pr.z, 1.0f);
    b.cy = view_row(v, 1, pr.x, pr.y, pr.z, 1.0f);
    b.cz = view_row(v, 2, pr.x, pr.y, pr.z, 1.0f);
    b.r = xadd(pr.w, xmul(xadd(pr.w, 1.0f), 1.0f / 1024.0f));  // froxel margin
    b.type = type;
}

// The cone fields (prep_light's second half) of a light whose centre is set: the axis
// and sine only where the cone test applies (light_meets_froxel reads them only then).
__device__ __forceinline__ void prep_light_cone(const ViewRows& v, float4 dir, float inner, BinLight& b) {
    b.cos_o = dir.w;
    b.cone = (b.type == 2u) && (0.0f < dir.w) && (dir.w < inner);
    b.pad = 0;
    if (b.cone) {
        const f3 a = xnormalize(mk3(view_row(v, 0, dir.x, dir.y, dir.z, 0.0f), view_row(v, 1, dir.x, dir.y, dir.z, 0.0f),
                                    view_row(v, 2, dir.x, dir.y, dir.z, 0.0f)));
        b.ax = a.x;
        b.ay = a.y;
        b.az = a.z;
        b.sin_o = xsqrt(xmax(xsub(1.0f, xmul(dir.w, dir.w)), 0.0f));
    }
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

struct ColumnGeom {
    Planes planes;
    float kx0, kx1, ky_bot, ky_top;
};

__device__ __forceinline__ uint32_t ceil_div_u64(uint64_t a, uint64_t b) { return uint32_t((a + b - 1) / b); }

// The NDC rectangle of froxel column (fx, fy): its pixel edges, as the reference forms
// a tile's (light_cull.wgsl:140-147).
struct ColumnRect {
    float left, right, top, bottom;
};

__device__ __forceinline__ ColumnRect column_rect(const hl_froxel_params& p, uint32_t fx, uint32_t fy) {
    const uint32_t px0 = ceil_div_u64(uint64_t(fx) * p.width, p.grid_x);
    const uint32_t px1 = ceil_div_u64(uint64_t(fx + 1) * p.width, p.grid_x);
    const uint32_t py0 = ceil_div_u64(uint64_t(fy) * p.height, p.grid_y);
    const uint32_t py1 = ceil_div_u64(uint64_t(fy + 1) * p.height, p.grid_y);
    const float fw = float(p.width), fh = float(p.height);
    ColumnRect r;
    r.left = xsub(xmul(xdiv(float(px0), fw), 2.0f), 1.0f);
    r.right = xsub(xmul(xdiv(float(px1), fw), 2.0f), 1.0f);
    r.top = xsub(1.0f, xmul(xdiv(float(py0), fh), 2.0f));
    r.bottom = xsub(1.0f, xmul(xdiv(float(py1), fh), 2.0f));
    return r;
}

__device__ __forceinline__ ColumnGeom column_geom(const GpuCamera* cam, const hl_froxel_params& p, uint32_t fx,
                                                  uint32_t fy) {
    const ColumnRect c = column_rect(p, fx, fy);
    const float p00 = cam->proj[0], p11 = cam->proj[5];
    ColumnGeom g;
    g.planes = rect_planes(p00, p11, c.left, c.right, c.top, c.bottom);
    g.kx0 = xdiv(c.left, p00);
    g.kx1 = xdiv(c.right, p00);
    g.ky_bot = xdiv(c.bottom, p11);
    g.ky_top = xdiv(c.top, p11);
    return g;
}

// One fifth of column_geom, by the same operations: part 0-3 the plane rect_planes puts
// at that index, part 4 the slopes. Five lanes build a column's geometry side by side.
__device__ __forceinline__ void column_geom_part(const GpuCamera* cam, const hl_froxel_params& p, uint32_t fx,
                                                 uint32_t fy, uint32_t part, ColumnGeom& g) {
    const ColumnRect c = column_rect(p, fx, fy);
    const float p00 = __ldg(&cam->proj[0]), p11 = __ldg(&cam->proj[5]);
    switch (part) {
        case 0: g.planes.n[0] = plane_from_ndc_edge(p00, p11, c.left, c.bottom, c.left, c.top); break;
        case 1: g.planes.n[1] = plane_from_ndc_edge(p00, p11, c.right, c.top, c.right, c.bottom); break;
        case 2: g.planes.n[2] = plane_from_ndc_edge(p00, p11, c.left, c.top, c.right, c.top); break;
        case 3: g.planes.n[3] = plane_from_ndc_edge(p00, p11, c.right, c.bottom, c.left, c.bottom); break;
        default:
            g.kx0 = xdiv(c.left, p00);
            g.kx1 = xdiv(c.right, p00);
            g.ky_bot = xdiv(c.bottom, p11);
            g.ky_top = xdiv(c.top, p11);
            break;
    }
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


// ---- one work item: the slices [s0, s1) of one froxel column ---------------------
//
// The item gathers, in light-index order, the lights that may touch its column (each
// light transformed to view space here, from the GpuLight), tests them against the
// box of each of its slices (one warp per slice, the chunk ballots kept for the fill),
// publishes its total on a chain of per-item words, finds the entries of all earlier
// items by decoupled look-back (a predecessor's inclusive prefix ends the walk, its
// bare total is added and the walk goes on), publishes its own inclusive prefix, writes
// its offsets and fills its lists. Chain words hold epoch << 32 | state << 30 | value; a
// word of another epoch reads as "not yet published". An item waits only for items
// with smaller tickets, which were handed out to CTAs already running.
constexpr uint32_t kItemCap = 512;      // column-list entries per gather round
constexpr uint32_t kGatherU = 2;        // 256-light sub-rounds per gather step
constexpr uint32_t kItemMaskCap = 1024; // (slice, 32-light chunk) ballots kept from the count
constexpr uint32_t kFlagAggregate = 1u, kFlagPrefix = 2u;
constexpr uint32_t kChainValueMax = (1u << 30) - 1u;
constexpr uint32_t kLookbackSpins = 1u << 20;  // ~0.1 s of polling before HL_ERR_TIMEOUT
constexpr uint32_t kLookbackWords = 4;         // chain words per lane in one look-back read

template <int NW>
struct ItemSmemT {
    uint32_t idx[kItemCap];           // the round's column list: light indices
    BinLight bl[kItemCap];            // and their view-space records
    uint32_t mask[kItemMaskCap];      // ballot of chunk c of slice s0 + k at [k * chunks + c]
    uint32_t warp_tot[kGatherU * NW];
    uint32_t slice_run[kMaxSlices];   // entries per slice of the item
    uint32_t slice_dst[kMaxSlices];   // first entry of each slice
    uint32_t stop[2];                 // first light index not kept by a full round (by step parity)
    uint32_t excl, total;
    ColumnGeom geom;                  // the item's column
};
using ItemSmem = ItemSmemT<kWarps>;  // the 256-thread CTAs of the persistent batched launch

// Parameters of a failure-injection test: item `stall` never publishes its chain word,
// and the look-back gives up after `spins` polls. stall = ~0u: none.
struct StallTest {
    uint32_t stall, spins;
};

__device__ __forceinline__ unsigned long long ld_chain(const unsigned long long* p) {
    return *reinterpret_cast<const volatile unsigned long long*>(p);
}

// A chain word carries its whole message (state and value) in one 8-byte store, and
// the items that read it read nothing else this item wrote: no fence is needed.
__device__ __forceinline__ void st_chain(unsigned long long* p, uint32_t epoch, uint32_t state, uint32_t value) {
    *reinterpret_cast<volatile unsigned long long*>(p) =
        (static_cast<unsigned long long>(epoch) << 32) | (state << 30) | min(value, kChainValueMax);
}

// Appends to sm.idx / sm.bl, in light-index order, the lights from `base` on that may
// touch the column (directional, or a sphere not outside its four planes), until the
// lights run out or the round is full. A step tests kGatherU x NT lights on their
// view-space centres alone, their loads in flight together; when a step overflows the
// round, the round ends at the first light that did not fit and `base` resumes there.
// The kept lights' cone fields are computed at the end of the round, once per kept
// light (most lights miss a given column).
template <int NW>
__device__ __forceinline__ uint32_t gather_item_round(ItemSmemT<NW>& sm, const ViewRows& vr,
                                                      const GpuLight* __restrict__ lights, const ColumnGeom& g,
                                                      uint32_t n, uint32_t& base) {
    constexpr uint32_t NT = NW * 32;
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    uint32_t len = 0, step = 0;
    if (threadIdx.x == 0) sm.stop[0] = 0xffffffffu;
    __syncthreads();
    while (base < n) {
        bool pass[kGatherU];
        BinLight rec[kGatherU];
        uint32_t mask[kGatherU];
#pragma unroll
        for (uint32_t u = 0; u < kGatherU; ++u) {
            const uint32_t i = base + u * NT + threadIdx.x;
            pass[u] = false;
            if (i < n) {
                const float4 pr = __ldg(reinterpret_cast<const float4*>(lights[i].position_range));
                prep_light_centre(vr, pr, __ldg(&lights[i].light_type), rec[u]);
                pass[u] = (rec[u].type == 0u) || sphere_in_planes(g.planes, rec[u].cx, rec[u].cy, rec[u].cz, rec[u].r);
            }
        }
#pragma unroll
        for (uint32_t u = 0; u < kGatherU; ++u) {
            mask[u] = __ballot_sync(0xffffffffu, pass[u]);
            if (lane == 0) sm.warp_tot[u * NW + warp] = __popc(mask[u]);
        }
        __syncthreads();
        if (threadIdx.x == 0) sm.stop[(step + 1) & 1u] = 0xffffffffu;  // read by the last step before this barrier
        uint32_t run = len;
#pragma unroll
        for (uint32_t u = 0; u < kGatherU; ++u) {
            uint32_t before = 0, total = 0;
#pragma unroll
            for (int w = 0; w < NW; ++w) {
                const uint32_t t = sm.warp_tot[u * NW + w];
                before += (uint32_t(w) < warp) ? t : 0u;
                total += t;
            }
            if (pass[u]) {
                const uint32_t pos = run + before + __popc(mask[u] & lanemask_lt());
                if (pos < kItemCap) {
                    sm.idx[pos] = base + u * NT + threadIdx.x;
                    BinLight& d = sm.bl[pos];
                    d.cx = rec[u].cx;
                    d.cy = rec[u].cy;
                    d.cz = rec[u].cz;
                    d.r = rec[u].r;
                    d.type = rec[u].type;
                } else {
                    atomicMin(&sm.stop[step & 1u], base + u * NT + threadIdx.x);
                }
            }
            run += total;
        }
        __syncthreads();
        const uint32_t stop = sm.stop[step & 1u];
        if (stop != 0xffffffffu) {  // the round is full: the next one starts at `stop`
            base = stop;
            len = kItemCap;
            break;
        }
        len = run;
        base += kGatherU * NT;
        ++step;
    }
    for (uint32_t j = threadIdx.x; j < len; j += NT) {
        BinLight& d = sm.bl[j];
        if (d.type == 2u) {
            const GpuLight& l = lights[sm.idx[j]];
            prep_light_cone(vr, __ldg(reinterpret_cast<const float4*>(l.direction_outer)), __ldg(&l.inner_angle), d);
        } else {
            d.cone = 0u;
        }
    }
    __syncthreads();
    return len;
}

// Tests a gathered round against the item's slice boxes: counts into sm.slice_run, and
// with FILL writes the lists from sm.slice_dst. With MASKS the count keeps each chunk's
// ballot and the fill replays them instead of testing again.
template <int NW, bool FILL>
__device__ __forceinline__ void test_item_slices(ItemSmemT<NW>& sm, const ColumnGeom& g, const float* __restrict__ tabz,
                                                 uint32_t gz, float zlast, uint32_t s0, uint32_t s1, uint32_t len,
                                                 uint32_t* __restrict__ indices, uint32_t capacity, bool masks) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t chunks = (len + 31) / 32;
    for (uint32_t s = s0 + warp; s < s1; s += NW) {
        const uint32_t k = s - s0;
        uint32_t run = sm.slice_run[k];
        const uint32_t dst0 = FILL ? sm.slice_dst[k] : 0u;
        uint32_t* sm_mask = sm.mask + k * chunks;
        if (FILL && masks) {
            for (uint32_t c = 0; c < chunks; ++c) {
                const uint32_t mask = sm_mask[c];
                if ((mask >> lane) & 1u) {
                    const uint64_t dst = uint64_t(dst0) + run + __popc(mask & lanemask_lt());
                    if (dst < capacity) indices[dst] = sm.idx[c * 32 + lane];
                }
                run += __popc(mask);
            }
        } else {
            const float z0 = tabz[s];
            const float z1 = (s + 1 == gz) ? zlast : tabz[s + 1];
            const Box b = froxel_box(g, z0, z1);
            for (uint32_t c = 0; c < chunks; ++c) {
                const uint32_t j = c * 32 + lane;
                const bool pass = j < len && light_meets_froxel(sm.bl[j], b);
                const uint32_t mask = __ballot_sync(0xffffffffu, pass);
                if (FILL && pass) {
                    const uint64_t dst = uint64_t(dst0) + run + __popc(mask & lanemask_lt());
                    if (dst < capacity) indices[dst] = sm.idx[j];
                }
                if (!FILL && masks && lane == 0) sm_mask[c] = mask;
                run += __popc(mask);
            }
        }
        if (lane == 0) sm.slice_run[k] = run;
    }
}

// Bins item `item` of a view: froxel column item / groups, slices [s0, s1) of the
// group item % groups (groups of ceil(grid_z / groups) slices). Items of a view are in
// froxel order, so the item chain's prefix is the first entry of the item's froxels.
template <int NW>
__device__ __forceinline__ void bin_item(ItemSmemT<NW>& sm, const GpuCamera* __restrict__ cam,
                                         const GpuLight* __restrict__ lights, uint32_t n, const hl_froxel_params& p,
                                         const float* __restrict__ tabz, uint32_t item, uint32_t groups,
                                         uint32_t epoch, unsigned long long* __restrict__ chain,
                                         uint32_t* __restrict__ offsets, uint32_t* __restrict__ indices,
                                         uint32_t capacity, int* __restrict__ status, const StallTest& test) {
    const uint32_t warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t col = item / groups, grp = item % groups;
    const uint32_t spg = (p.grid_z + groups - 1) / groups;
    const uint32_t s0 = min(grp * spg, p.grid_z), s1 = min(s0 + spg, p.grid_z);
    const uint32_t ns = s1 - s0;
    const uint32_t items = p.grid_x * p.grid_y * groups;
    if (warp == 0 && lane < 5) column_geom_part(cam, p, col % p.grid_x, col / p.grid_x, lane, sm.geom);
    const ViewRows vr = load_view_rows(cam);
    const float zlast = xmax(tabz[p.grid_z], cam->forward_far[3]);
    for (uint32_t k = threadIdx.x; k < ns; k += blockDim.x) sm.slice_run[k] = 0;
    __syncthreads();
    const ColumnGeom g = sm.geom;

    // ---- 1. count ----
    uint32_t base = 0, len = 0;
    bool one_round = true, masks = false;
    for (bool first = true;; first = false) {
        len = gather_item_round<NW>(sm, vr, lights, g, n, base);
        if (!first) one_round = false;
        // an item gathered in one round keeps its chunk ballots when they fit
        masks = one_round && base >= n && ns * ((len + 31) / 32) <= kItemMaskCap;
        test_item_slices<NW, false>(sm, g, tabz, p.grid_z, zlast, s0, s1, len, indices, capacity, masks);
        if (base >= n) break;
    }
    __syncthreads();

    // ---- 2. chained scan over the items ----
    if (warp == 0) {
        const bool publish = item != test.stall;
        uint32_t acc = 0;  // exclusive scan of the slice counts, 32 slices at a time
        for (uint32_t k0 = 0; k0 < ns; k0 += 32) {
            const uint32_t k = k0 + lane;
            const uint32_t r = k < ns ? sm.slice_run[k] : 0u;
            uint32_t v = r;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t u = __shfl_up_sync(0xffffffffu, v, o);
                if (lane >= uint32_t(o)) v += u;
            }
            if (k < ns) sm.slice_dst[k] = acc + v - r;
            acc += __shfl_sync(0xffffffffu, v, 31);
        }
        if (lane == 0) {
            sm.total = acc;
            if (publish) st_chain(chain + item, epoch, item == 0 ? kFlagPrefix : kFlagAggregate, acc);
        }
        __syncwarp();
        // look-back: the warp reads kLookbackWords x 32 predecessors at once (item - 1
        // down), finds the nearest one holding an inclusive prefix (before item 0: a
        // prefix of 0) and sums that prefix and the bare totals after it; a window of
        // totals only is added whole and the walk goes on below it
        uint32_t excl = 0;
        int32_t hi = int32_t(item) - 1;
        uint32_t spins = 0;
        while (hi >= 0) {
            uint32_t st[kLookbackWords], val[kLookbackWords];
#pragma unroll
            for (uint32_t k = 0; k < kLookbackWords; ++k) {
                const int32_t c = hi - int32_t(lane + 32u * k);
                st[k] = kFlagPrefix;
                val[k] = 0;
                if (c >= 0) {
                    const unsigned long long w = ld_chain(chain + c);
                    st[k] = uint32_t(w >> 32) == epoch ? (uint32_t(w) >> 30) : 0u;
                    val[k] = uint32_t(w) & kChainValueMax;
                }
            }
            // offset (lane + 32 k) of the nearest prefix this lane holds
            uint32_t near = 0xffffffffu;
#pragma unroll
            for (int k = int(kLookbackWords) - 1; k >= 0; --k)
                if (st[k] == kFlagPrefix) near = lane + 32u * uint32_t(k);
            near = __reduce_min_sync(0xffffffffu, near);
            bool missing = false;
            uint32_t sum = 0;
#pragma unroll
            for (uint32_t k = 0; k < kLookbackWords; ++k) {
                if (lane + 32u * k <= near) {
                    missing |= st[k] == 0u;
                    sum += val[k];
                }
            }
            if (__any_sync(0xffffffffu, missing)) {  // a predecessor has not published yet
                if (++spins > test.spins) {
                    if (lane == 0) raise_status(status, HL_ERR_TIMEOUT);
                    break;
                }
                __nanosleep(64);
                continue;
            }
            excl += __reduce_add_sync(0xffffffffu, sum);
            if (near != 0xffffffffu) break;
            hi -= int32_t(32u * kLookbackWords);
        }
        if (lane == 0) {
            if (item > 0 && publish) st_chain(chain + item, epoch, kFlagPrefix, excl + sm.total);
            sm.excl = excl;
            if (uint64_t(excl) + sm.total > capacity) raise_status(status, HL_ERR_CAPACITY);
            if (uint64_t(excl) + sm.total > kChainValueMax) raise_status(status, HL_ERR_SIZE);
        }
    }
    __syncthreads();
    const uint32_t excl = sm.excl;
    for (uint32_t k = threadIdx.x; k < ns; k += blockDim.x) {
        sm.slice_dst[k] += excl;
        offsets[col * p.grid_z + s0 + k] = sm.slice_dst[k];
        sm.slice_run[k] = 0;
    }
    if (item == items - 1 && threadIdx.x == 0) offsets[p.grid_x * p.grid_y * p.grid_z] = excl + sm.total;
    __syncthreads();

    // ---- 3. fill (from the round still in shared memory when there was only one) ----
    if (one_round) {
        test_item_slices<NW, true>(sm, g, tabz, p.grid_z, zlast, s0, s1, len, indices, capacity, masks);
    } else {
        base = 0;
        for (;;) {
            len = gather_item_round<NW>(sm, vr, lights, g, n, base);
            test_item_slices<NW, true>(sm, g, tabz, p.grid_z, zlast, s0, s1, len, indices, capacity, false);
            if (base >= n) break;
        }
    }
    __syncthreads();
}

// Slice groups per column for a grid: enough items for `min_items`, at most one group
// per slice.
__host__ __device__ inline uint32_t item_groups(const hl_froxel_params& p, uint32_t min_items) {
    const uint32_t cols = p.grid_x * p.grid_y;
    uint32_t g = (min_items + cols - 1) / cols;
    if (g < 1) g = 1;
    if (g > p.grid_z) g = p.grid_z;
    return g;
}

}  // namespace bin
}  // namespace hl
