// hl_shade_f16.cu — deferred lighting (fs_main under fallback bindings) of an FP16
// G-buffer over froxel lists, the headline form of hl_shade.
//
// One CTA of 256 threads lights a 32x16-pixel tile:
//  1. threads load the tile's G-buffer texels (coalesced along x) first and set each pixel
//     up into a shared-memory record: camera-relative position, roughness, unit normal,
//     NdV, F0, albedo, metallic, with its froxel;
//  2. pixels are counting-sorted by froxel and, inside a froxel, by a depth sub-bin of
//     its slice, so that a group of 32 consecutive sorted pixels spans one froxel (or
//     a few of adjacent slices) and a narrow depth range;
//  3. a warp takes a group. For each froxel of the group it culls the froxel's list
//     against the bounding box of the group's pixels in that froxel (lanes test 32
//     lights at once; a chunk of at most four entries is kept whole), and each of those
//     pixels keeps the survivors as a bit mask. Then every lane walks its own mask,
//     testing its pixel against each surviving light for range, the NdL sign and a
//     conservative bound of the radiance against the 0.002 cut (walk_test). The box test
//     applies the per-pixel range test's own f32 operations to box-clamped differences,
//     so every pair the per-pixel test passes survives it: the queued pairs are exactly
//     those of walk_test over the pixel's whole list, in list order;
//  4. queued (pixel, light) pairs are evaluated 32 at a time, one per lane, and added
//     into per-pixel Kahan accumulators in queue order, which is list order for every
//     pixel, as the reference's light loop (deferred_lighting.wgsl:1119-1146) adds them;
//  5. when no group is left, a warp evaluates the pairs left in its queue and stores the
//     pixels of the groups it walked (hemisphere ambient added): every pair of a pixel
//     is queued, evaluated and accumulated by the warp that walked its group, so the
//     warps finish the tile without waiting for one another.
#include <algorithm>

#include "hl_bin_item.cuh"
#include "hl_common.cuh"
#include "hl_internal.h"
#include "hl_precise.cuh"
#include "hl_shade_math.cuh"
#include "hl_texel.cuh"

namespace hl {

namespace {

using namespace sm;

namespace f16k {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int TW = 32, TH = 16, NPX = TW * TH;
constexpr int PPT = NPX / kThreads;  // pixels per thread in set-up and output
constexpr int NG = NPX / 32;         // groups of 32 sorted pixels
constexpr int kQueue = 64;           // per-warp pair ring: at most 31 + 32 pending
constexpr int kBins = 512;           // keys of the pixel sort
static_assert(31 + 32 <= kQueue, "pair ring too small");

// Shared memory of a tile: 54.4 KB, so that three CTAs fit the 164 KB shared-memory
// configuration of an SM and leave 92 KB to L1 (the lists, the candidate table and the
// lights are read through it); 16 bytes more would need the 196 KB one.
// Pixel record: four arrays of 16-byte fields (consecutive pixels on consecutive banks),
// read by a lane evaluating a pair of a random pixel with four 16-byte loads; the view
// terms 1 / |P|, roughness^4, (r+1)^2/8 and Schlick-GGX are recomputed from them.
struct Smem {
    float4 P4[NPX];  // camera-relative position (f32), roughness
    float4 N4[NPX];  // unit normal, max(N.V, 0)
    float4 F4[NPX];  // F0 rgb, NDC depth (negative: seen at a grazing angle, every pair precise)
    float4 D4[NPX];  // albedo rgb, metallic
    float4 acc[2][NPX];  // Kahan sum and compensation (rgb)
    union {
        struct {
            uint32_t hist[kBins];
            uint16_t col_of[TW], row_of[TH];
        } sort;
        uint32_t queue[kWarps][kQueue];  // walk: ring of (pixel << 23) | light index
    } u;
    struct {
        uint32_t fidx[NPX];    // froxel of the pixel
        uint16_t order[NPX];   // pixels sorted by key
    } w;
    uint32_t n_valid, next_group;
    uint32_t fx0, fy0, ncx, ncols, kshift, by_column;
};
// three CTAs (with the 1 KB each that the driver reserves, in 128-byte steps) in 164 KB
static_assert(((sizeof(Smem) + 1024 + 127) / 128) * 128 * 3 <= 164 * 1024, "tile no longer fits 3 CTAs in 164 KB");

__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));  // not volatile: the compiler may keep it
    return m;
}

// Warp minimum / maximum of f32 values (redux.sync on f32, sm_100 and later); the values
// here are finite, and a lane outside the set passes +inf / -inf.
__device__ __forceinline__ float warp_min(float v) {
    float r;
    asm volatile("redux.sync.min.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}
__device__ __forceinline__ float warp_max(float v) {
    float r;
    asm volatile("redux.sync.max.f32 %0, %1, 0xffffffff;" : "=f"(r) : "f"(v));
    return r;
}

__device__ __forceinline__ float h2f(uint32_t bits16) { return __half2float(__ushort_as_half(uint16_t(bits16))); }

}  // namespace f16k

// The precise evaluation of the pair (pixel (x, y), light li), from the pixel's texel
// and the light buffer, so that only scalars cross the call. Returns (r, g, b, status).
__device__ __noinline__ float4 precise_f16(const GBufView& gb, uint32_t x, uint32_t y, const GpuCamera* cam,
                                           const GpuLight* lights, uint32_t li) {
    const gbuf::Texel<HL_GBUF_F16> tx = gbuf::load_texel<HL_GBUF_F16>(gb, x, y);
    Pixel p;
    p.nrx = tx.nx; p.nry = tx.ny; p.nrz = tx.nz;
    p.rough = tx.rough;
    p.metal = tx.metal;
    p.f0r = tx.f0r; p.f0g = tx.f0g; p.f0b = tx.f0b;
    const float4* gl = reinterpret_cast<const float4*>(lights + li);
    const float4 a = __ldg(gl + 0), b = __ldg(gl + 1), c = __ldg(gl + 2);
    const uint4 d = __ldg(reinterpret_cast<const uint4*>(gl + 3));
    const float camx = cam->position_near[0], camy = cam->position_near[1], camz = cam->position_near[2];
    const DF ux = two_sum(a.x, -camx), uy = two_sum(a.y, -camy), uz = two_sum(a.z, -camz);
    ShadeLight l;
    l.px = ux.hi; l.py = uy.hi; l.pz = uz.hi;
    l.range = a.w;
    l.dx = b.x; l.dy = b.y; l.dz = b.z; l.cos_outer = b.w;
    l.cr = c.x; l.cg = c.y; l.cb = c.z; l.intensity = c.w;
    l.type = d.y;
    l.cos_inner = __uint_as_float(d.z);
    float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const int st = precise_pair(cam, x, y, float(gb.width), float(gb.height), tx.depth, p, tx.ar, tx.ag, tx.ab, l,
                                ux.lo, uy.lo, uz.lo, o.x, o.y, o.z);
    o.w = __int_as_float(st);
    return o;
}

// pbr_direct_light of one queued pair (pixel q of the tile at x0, y0; light li) on the
// fast path, handed to precise_f16 when the guard flags it or the pixel is grazing.
// Returns (r, g, b) and the status in w.
__device__ __forceinline__ float4 eval_pair(const f16k::Smem& s, uint32_t q, uint32_t li, const GpuCamera* cam,
                                            const float3& camp, const GpuLight* lights, const GBufView& gb,
                                            uint32_t x0, uint32_t y0) {
    using namespace f16k;
    const float4 r0 = s.P4[q], r1 = s.N4[q], r2 = s.F4[q], r3 = s.D4[q];
    Pixel p;
    p.Px = r0.x; p.Py = r0.y; p.Pz = r0.z;
    p.Plx = p.Ply = p.Plz = 0.0f;
    p.Nx = r1.x; p.Ny = r1.y; p.Nz = r1.z;
    // V = -P / |P| (camera at the origin) and the BRDF's view terms, as the set-up forms them
    const float iv = rsqrt_(fma_(p.Pz, p.Pz, fma_(p.Py, p.Py, p.Px * p.Px)));
    p.Vx = -p.Px * iv;
    p.Vy = -p.Py * iv;
    p.Vz = -p.Pz * iv;
    p.NdV = r1.w;
    p.f0r = r2.x; p.f0g = r2.y; p.f0b = r2.z;
    p.dr = r3.x * kInvPi; p.dg = r3.y * kInvPi; p.db = r3.z * kInvPi;
    const float rough = r0.w, ra = rough * rough, r1k = rough + 1.0f;
    PixelBrdf pb;
    pb.a2 = ra * ra;
    pb.k = (r1k * r1k) * 0.125f;
    pb.omk = 1.0f - pb.k;
    pb.gv = divn_(p.NdV, fma_(p.NdV, 1.0f - pb.k, pb.k + 0.0001f));
    pb.one_m_metal = 1.0f - r3.w;
    pb.nv4 = 4.0f * p.NdV;
    pb.vlx = pb.vly = pb.vlz = 0.0f;
    const float4* gl = reinterpret_cast<const float4*>(lights + li);
    const float4 a = __ldg(gl + 0), b = __ldg(gl + 1), c = __ldg(gl + 2);
    const uint4 d = __ldg(reinterpret_cast<const uint4*>(gl + 3));
    ShadeLight l;
    l.px = a.x - camp.x;  // camera-relative light position (high word of its two-sum)
    l.py = a.y - camp.y;
    l.pz = a.z - camp.z;
    l.range = a.w;
    l.dx = b.x; l.dy = b.y; l.dz = b.z; l.cos_outer = b.w;
    l.cr = c.x; l.cg = c.y; l.cb = c.z; l.intensity = c.w;
    l.type = d.y;
    l.cos_inner = __uint_as_float(d.z);
    float4 o = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    int st = kNeedsPrecise;
    if (r2.w >= 0.0f) st = eval<false>(p, pb, l, o.x, o.y, o.z, fast_guard(p));
    if (st == kNeedsPrecise) return precise_f16(gb, x0 + q % TW, y0 + q / TW, cam, lights, li);
    o.w = __int_as_float(st);
    return o;
}

// The walk's test of a candidate pair (pixel at p, normal n; light record a, peak its
// largest colour channel times intensity): inside the widened range, in front of the
// surface (|N.t| within sqrt(slack) of zero is left to the exact NdL cut), and not surely
// below the radiance cut of pbr_direct_light. The radiance bound, peak falloff / (d^2 +
// 1e-4) compared as peak falloff < 0.002 (d^2 + 1e-4), takes the falloff with the
// widened range (no smaller than the true one) plus 2^-20 and 2^-8 to spare, so that no
// rounding of the fast or the precise evaluation reaches 0.002 on a pair it drops: those
// pairs would be evaluated only to be cut. Directional lights always pass.
__device__ __forceinline__ bool walk_test(float px, float py, float pz, float nx, float ny, float nz, const float4& a,
                                          float peak, float slack) {
    if (a.w < 0.0f) return true;
    const float tx = a.x - px, ty = a.y - py, tz = a.z - pz;
    const float d2 = fma_(tz, tz, fma_(ty, ty, tx * tx));
    const float ndl = fma_(nz, tz, fma_(ny, ty, nx * tx));
    if (!(d2 <= a.w) || !(ndl > 0.0f || ndl * ndl <= slack)) return false;
    float q;
    asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(q) : "f"(a.w));  // within 2 ulp: the 2^-20 covers it
    q *= d2;
    const float fall = fmax_(fma_(-q, q, 1.0f), 0.0f) + (1.0f / 1048576.0f);
    return !(peak * fall * (1.0f + 1.0f / 256.0f) < kRadianceCut * (d2 + 0.0001f));
}

// Records lit pairs for a verifier (hl_set_pair_log); a no-op without a log.
__device__ __forceinline__ void log_pair(const PairLog& log, bool lit, uint32_t lane, uint32_t x, uint32_t y,
                                         uint32_t W, uint32_t li) {
    if (!log.pairs) return;
    const uint32_t m = __ballot_sync(0xffffffffu, lit);
    if (!m) return;
    uint32_t base = 0;
    if (lane == 0) base = atomicAdd(log.count, uint32_t(__popc(m)));
    base = __shfl_sync(0xffffffffu, base, 0);
    const uint32_t slot = base + __popc(m & f16k::lanemask_lt());
    if (lit && slot < log.capacity) log.pairs[slot] = make_uint2(y * W + x, li);
}

// Adds each lane's contribution (when lit) to pixel q's accumulators, lanes in order
// where several hold the same pixel.
__device__ __forceinline__ void accumulate(f16k::Smem& s, bool lit, uint32_t q, float cr, float cg, float cb) {
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t peers = __match_any_sync(0xffffffffu, lit ? q : (0x10000u | lane));
    const uint32_t rank = __popc(peers & f16k::lanemask_lt());
    const uint32_t rounds = __reduce_max_sync(0xffffffffu, lit ? rank + 1 : 0u);
    for (uint32_t r = 0; r < rounds; ++r) {
        if (lit && rank == r) {
            float4 sum = s.acc[0][q], cmp = s.acc[1][q];
            kahan_add(sum.x, cmp.x, cr);
            kahan_add(sum.y, cmp.y, cg);
            kahan_add(sum.z, cmp.z, cb);
            s.acc[0][q] = sum;
            s.acc[1][q] = cmp;
        }
        __syncwarp();
    }
}

// Evaluates the 32 queued pairs at ring positions head..head+31 and accumulates them
// (inlined into the walk: a call there costs its live registers a trip through the stack).
__device__ __forceinline__ void flush32(f16k::Smem& s, const uint32_t* queue, uint32_t head, uint32_t lane,
                                     const GpuCamera* cam, const float3& camp, const GpuLight* lights,
                                     const GBufView& gb, uint32_t x0, uint32_t y0, const PairLog& log) {
    using namespace f16k;
    const uint32_t e = queue[(head + lane) & (kQueue - 1)];
    const uint32_t q = e >> 23, li = e & 0x7fffffu;
    const float4 o = eval_pair(s, q, li, cam, camp, lights, gb, x0, y0);
    const bool lit = __float_as_int(o.w) == kLit;
    log_pair(log, lit, lane, x0 + q % TW, y0 + q / TW, gb.width, li);
    accumulate(s, lit, q, o.x, o.y, o.z);
    __syncwarp();
}

// A load of the froxel lists: through the read-only path, or (COHERENT) by a plain
// L1-cached load (ld.global.ca) when the lists were written earlier in the same launch
// (the persistent batched launch). The read-only path may not be used for data written
// during the launch; a plain load may be, once ordered after the writes: a view's
// shading reads its lists only after thread 0 has seen every binning item of the view
// finish (the counter the items raise after a fence, read and followed by a fence) and
// the CTA barrier has passed that on, and no cache line holds two views' lists, so L1
// never holds a line of them from before they were written.
template <bool COHERENT>
__device__ __forceinline__ uint32_t list_ld(const uint32_t* p) {
    return COHERENT ? __ldca(p) : __ldg(p);
}

// Lights the 32x16 tile (bx, by) of one view. prefetch_next: the tile index (row-major
// over tiles_x tiles per row) whose G-buffer to ask L2 for, or ~0u.
template <uint32_t TARGET, bool COHERENT = false>
__device__ __forceinline__ void shade_tile_f16(f16k::Smem& s, const GpuCamera* __restrict__ cam,
                                               const DeferredGlobals* __restrict__ glb, const GBufView& gb,
                                               const GpuLight* __restrict__ lights, uint32_t n_lights,
                                               const GridView& grid, const float* __restrict__ tabz,
                                               const TargetView& out, int* __restrict__ status,
                                               const float4* __restrict__ cand, const PairLog& log, uint32_t bx,
                                               uint32_t by, uint32_t tiles_x, uint32_t prefetch_next) {
    using namespace f16k;
    const uint32_t t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const uint32_t x0 = bx * TW, y0 = by * TH;
    const hl_froxel_params& fp = grid.fp;

    // the tile's G-buffer texels, loaded before the first barrier so that their latency
    // overlaps the set-up of shared memory (outside the view: depth 1, sky)
    uint2 ga[PPT];
    uint32_t gn[PPT];
    uint16_t gm[PPT];
    float gd[PPT];
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        const uint32_t i = t + k * kThreads;
        const uint32_t x = x0 + i % TW, y = y0 + i / TW;
        ga[k] = make_uint2(0u, 0u);
        gn[k] = 0u;
        gm[k] = 0u;
        gd[k] = 1.0f;
        if (x < gb.width && y < gb.height) {
            ga[k] = *reinterpret_cast<const uint2*>(gb.plane[0] + gb.pitch[0] * y + 8ull * x);
            gn[k] = *reinterpret_cast<const uint32_t*>(gb.plane[1] + gb.pitch[1] * y + 4ull * x);
            gm[k] = *reinterpret_cast<const uint16_t*>(gb.plane[2] + gb.pitch[2] * y + 2ull * x);
            gd[k] = *reinterpret_cast<const float*>(gb.plane[3] + gb.pitch[3] * y + 4ull * x);
        }
    }
    for (uint32_t b = t; b < uint32_t(kBins); b += kThreads) s.u.sort.hist[b] = 0;
    // froxel column of each pixel column and row of the tile (x * grid_x < 2^32 for
    // viewports of at most 65536 pixels per side)
    if (t < uint32_t(TW)) {
        s.u.sort.col_of[t] = uint16_t(((x0 + t) * fp.grid_x) / fp.width);
    } else if (t < uint32_t(TW + TH)) {
        s.u.sort.row_of[t - TW] = uint16_t(((y0 + t - TW) * fp.grid_y) / fp.height);
    } else if (t == uint32_t(TW + TH)) {
        // the tile's froxel columns and the key layout: (slice, column) keys, slice-major,
        // each split into 2^kshift depth sub-bins, within the 512 bins
        const uint32_t xe = min(x0 + TW, gb.width) - 1, ye = min(y0 + TH, gb.height) - 1;
        const uint32_t fx0 = (x0 * fp.grid_x) / fp.width, fy0 = (y0 * fp.grid_y) / fp.height;
        const uint32_t ncx = (xe * fp.grid_x) / fp.width - fx0 + 1;
        const uint32_t ncols = ncx * ((ye * fp.grid_y) / fp.height - fy0 + 1);
        const bool by_column = ncols * fp.grid_z <= uint32_t(kBins);
        const uint32_t nk = by_column ? ncols * fp.grid_z : fp.grid_z;
        s.fx0 = fx0;
        s.fy0 = fy0;
        s.ncx = ncx;
        s.ncols = ncols;
        s.by_column = by_column;
        s.kshift = 31u - __clz(uint32_t(kBins) / nk);
    }
#pragma unroll
    for (int k = 0; k < PPT; ++k) {
        s.acc[0][t + k * kThreads] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        s.acc[1][t + k * kThreads] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    }
    __syncthreads();

    const float camx = cam->position_near[0], camy = cam->position_near[1], camz = cam->position_near[2];
    const float3 camp = make_float3(camx, camy, camz);  // kept in registers for the pair evaluations
    const float W = float(gb.width), H = float(gb.height);
    // slices are exponential from slice_near to tab[grid_z]: slice ~ log2(d / near) * scale
    const float slice_inv_near = rcpn_(fp.slice_near);
    const float slice_scale =
        float(fp.grid_z) * rcpn_(__log2f(fmaxf(__ldg(tabz + fp.grid_z) * slice_inv_near, 2.0f)));
    const float nr = cam->position_near[3], fr = cam->forward_far[3];
    const float nrfr = nr * fr, frmnr = fr - nr;
    const uint32_t fx0 = s.fx0, fy0 = s.fy0, ncx = s.ncx, ncols = s.ncols, kshift = s.kshift;
    const bool by_column = s.by_column != 0u;

    // ---- 1. pixel set-up -------------------------------------------------------------
    float rel[12], wrow[4];
    camera_relative_rows(cam->inv_view_proj, camx, camy, camz, rel, wrow);
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
        {
            const uint2 a = ga[k];
            const uint32_t on = gn[k];
            const uint16_t mt = gm[k];
            const float depth = gd[k];
            valid[k] = depth < 1.0f;
            if (valid[k]) {
                const float ndx = fma_(float(2u * x + 1u), iW, -1.0f);
                const float ndy = fma_(float(2u * y + 1u), -iH, 1.0f);
                float Px, Py, Pz;
                reconstruct_relative(rel, wrow, ndx, ndy, depth, Px, Py, Pz);
                float nx, ny, nz;
                oct_decode(f16k::h2f(on & 0xffffu), f16k::h2f(on >> 16), nx, ny, nz);
                const float in = rsqrt_(fma_(nz, nz, fma_(ny, ny, nx * nx)));
                // V = -P / |P| (camera at the origin), NdV as the fast path's set-up forms it
                const float iv = rsqrt_(fma_(Pz, Pz, fma_(Py, Py, Px * Px)));
                const float ndv = fmax_(fma_(nz, -Pz, fma_(ny, -Py, nx * -Px)) * in * iv, 0.0f);
                const float ar = f16k::h2f(a.x & 0xffffu), ag = f16k::h2f(a.x >> 16), ab = f16k::h2f(a.y & 0xffffu);
                const float rough = f16k::h2f(a.y >> 16), metal = f16k::h2f(mt);
                s.P4[i] = make_float4(Px, Py, Pz, rough);
                s.N4[i] = make_float4(nx * in, ny * in, nz * in, ndv);
                // grazing view: every pair of the pixel goes to the precise evaluation
                s.F4[i] = make_float4(fmin_(fmax_(metallic_f0(ar, metal), 0.0f), 0.999f),
                                      fmin_(fmax_(metallic_f0(ag, metal), 0.0f), 0.999f),
                                      fmin_(fmax_(metallic_f0(ab, metal), 0.0f), 0.999f),
                                      ndv < kFastMinNdV ? -depth : depth);
                s.D4[i] = make_float4(ar, ag, ab, metal);
                // own froxel: column of (x, y), slice of the linear view depth (the lists
                // are conservative by 2^-10 of the slice depth, so the slice only needs
                // the depth to a few ulp)
                const float dv = nrfr * rcpn_(fma_(-depth, frmnr, fr));
                const float sf = __log2f(dv * slice_inv_near) * slice_scale;
                // (near a slice boundary the rounding of this scale may give the
                // neighbouring slice: both lists hold every light that reaches the pixel,
                // a froxel's box being widened by 2^-10 of its far depth)
                const uint32_t sl = uint32_t(min(max(int(sf), 0), int(fp.grid_z) - 1));
                const uint32_t fx = s.u.sort.col_of[x - x0];
                const uint32_t fy = s.u.sort.row_of[y - y0];
                s.w.fidx[i] = (fy * fp.grid_x + fx) * fp.grid_z + sl;
                // depth sub-bin: the position inside the slice on its logarithmic scale
                const uint32_t nsub = 1u << kshift;
                const uint32_t sub = uint32_t(min(max(int((sf - float(sl)) * float(nsub)), 0), int(nsub) - 1));
                const uint32_t kb = by_column ? sl * ncols + (fy - fy0) * ncx + (fx - fx0) : sl;
                key[k] = (kb << kshift) | sub;
                slot[k] = atomicAdd(&s.u.sort.hist[key[k]], 1u);
            }
        }
    }
    __syncthreads();
    if (warp == 0) {
        // exclusive scan of the key histogram by one warp: 16 consecutive bins per lane
        uint4 h[4];
#pragma unroll
        for (int m = 0; m < 4; ++m) h[m] = reinterpret_cast<const uint4*>(s.u.sort.hist)[lane * 4 + m];
        uint32_t sum = 0;
#pragma unroll
        for (int m = 0; m < 4; ++m) sum += h[m].x + h[m].y + h[m].z + h[m].w;
        uint32_t inc = sum;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t n = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= uint32_t(o)) inc += n;
        }
        uint32_t run = inc - sum;
#pragma unroll
        for (int m = 0; m < 4; ++m) {
            uint4 e;
            e.x = run; run += h[m].x;
            e.y = run; run += h[m].y;
            e.z = run; run += h[m].z;
            e.w = run; run += h[m].w;
            reinterpret_cast<uint4*>(s.u.sort.hist)[lane * 4 + m] = e;
        }
        if (lane == 31) {
            s.n_valid = inc;
            s.next_group = 0;
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < PPT; ++k)
        if (valid[k]) s.w.order[s.u.sort.hist[key[k]] + slot[k]] = uint16_t(t + k * kThreads);

    if (prefetch_next != ~0u) {
        // ask L2 for the G-buffer rows of the tile the next wave will likely take:
        // 32 x 128 B of plane 0 (8 B/px), 16 x 128 B of planes 1 and 3, 16 x 64 B of plane 2
        const uint32_t next = prefetch_next;
        if (t < 80u) {
            const uint32_t nx0 = (next % tiles_x) * TW, ny0 = (next / tiles_x) * TH;
            const uint32_t pl = t < 32u ? 0u : t < 48u ? 1u : t < 64u ? 2u : 3u;
            const uint32_t row = t < 32u ? t >> 1 : (t - 16u) & 15u;
            const uint32_t bpp = pl == 0u ? 8u : pl == 2u ? 2u : 4u;
            const uint32_t yy = ny0 + row;
            if (yy < gb.height) {
                const uint32_t b0 = nx0 * bpp + (t < 32u ? (t & 1u) * 128u : 0u);
                const uint32_t bend = gb.width * bpp - 1u;
                gbuf::prefetch_l2(gb.plane[pl] + gb.pitch[pl] * yy + min(b0, bend));
            }
        }
    }
    pdl_wait();  // the lists and the candidate table are written
    __syncthreads();

    // ---- 2-4. groups of 32 sorted pixels -------------------------------------------------
    const uint32_t n_valid = s.n_valid;
    uint32_t* queue = s.u.queue[warp];
    uint32_t head = 0, qlen = 0;  // ring position of the oldest pending pair, pending pairs
    uint32_t mine = 0;            // the groups this warp walked
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
        mine |= 1u << g;
        const uint32_t gs = g * 32 + lane;
        const bool own = gs < n_valid;
        const uint32_t i = own ? s.w.order[gs] : 0u;
        float px = 0, py = 0, pz = 0, nx = 0, ny = 0, nz = 0;
        uint32_t f = 0xffffffffu, lb = 0, le = 0;
        if (own) {
            const float4 rp = s.P4[i], rn = s.N4[i];
            px = rp.x; py = rp.y; pz = rp.z;
            nx = rn.x; ny = rn.y; nz = rn.z;
            f = s.w.fidx[i];
            lb = list_ld<COHERENT>(grid.counts + f);
            le = list_ld<COHERENT>(grid.counts + f + 1);
            if (!(lb <= le && le <= grid.lists_capacity)) {
                raise_status(status, HL_ERR_DEVICE_BOUNDS);
                le = lb;
            }
        }
        // |N.t| within |P| 2^-20 of zero is left to the exact NdL cut
        const float slack = fma_(pz, pz, fma_(py, py, px * px)) * (1.0f / 1099511627776.0f);
#pragma unroll 1
        for (uint32_t c0 = 0;; c0 += 32) {
            const bool act = own && lb + c0 < le;
            uint32_t pending = __ballot_sync(0xffffffffu, act);
            if (!pending) break;
            // A: per froxel of the group, the 32 list entries from c0 on, culled against the
            // bounding box of the group's pixels in that froxel (a chunk of at most four
            // entries goes to the walk as it is: its box would cost more than it saves)
            uint32_t smask = 0;
            while (pending) {
                const uint32_t leader = __ffs(pending) - 1;
                const uint32_t fk = __shfl_sync(0xffffffffu, f, leader);
                const bool mine = act && f == fk;
                pending &= ~__ballot_sync(0xffffffffu, mine);
                const uint32_t j = __shfl_sync(0xffffffffu, lb, leader) + c0 + lane;
                const uint32_t je = __shfl_sync(0xffffffffu, le, leader);
                if (je - (j - lane) <= 4u) {
                    const uint32_t m = __ballot_sync(0xffffffffu, j < je);
                    if (mine) smask = m;
                    continue;
                }
                const float inf = __int_as_float(0x7f800000);
                const float b0x = warp_min(mine ? px : inf), b0y = warp_min(mine ? py : inf),
                            b0z = warp_min(mine ? pz : inf);
                const float b1x = warp_max(mine ? px : -inf), b1y = warp_max(mine ? py : -inf),
                            b1z = warp_max(mine ? pz : -inf);
                const uint32_t lj = j < je ? list_ld<COHERENT>(grid.lists + j) : 0xffffffffu;
                const bool ok = lj < n_lights;
                if (j < je && !ok) raise_status(status, HL_ERR_DEVICE_BOUNDS);
                const float4 c = ok ? __ldg(cand + lj) : make_float4(0.0f, 0.0f, 0.0f, -1.0f);
                // the per-pixel test's operations on the box-clamped differences: for a pixel
                // in the box each |difference| rounds no smaller, so a light the box rejects
                // fails the range test at every pixel of the box
                const float dx = fmaxf(fmaxf(b0x - c.x, c.x - b1x), 0.0f);  // no NaN here: box and
                const float dy = fmaxf(fmaxf(b0y - c.y, c.y - b1y), 0.0f);  // record are finite
                const float dz = fmaxf(fmaxf(b0z - c.z, c.z - b1z), 0.0f);
                const bool keep = ok && (c.w < 0.0f || fma_(dz, dz, fma_(dy, dy, dx * dx)) <= c.w);
                const uint32_t m = __ballot_sync(0xffffffffu, keep);
                if (mine) smask = m;
            }
            // B: every lane walks the survivors of its own froxel, in list order
            const uint32_t cb = lb + c0;
#pragma unroll 1
            while (__any_sync(0xffffffffu, smask != 0u)) {
                bool pass = false;
                uint32_t li = 0;
                if (smask) {
                    const uint32_t bit = __ffs(smask) - 1;
                    smask &= smask - 1;
                    li = list_ld<COHERENT>(grid.lists + cb + bit);
                    if (li < n_lights) {  // (entries of short chunks reach here unchecked)
                        const float4 a = __ldg(cand + li);
                        const float peak = __ldg(reinterpret_cast<const float*>(cand + n_lights) + li);
                        pass = walk_test(px, py, pz, nx, ny, nz, a, peak, slack);
                    } else {
                        raise_status(status, HL_ERR_DEVICE_BOUNDS);
                    }
                }
                const uint32_t pm = __ballot_sync(0xffffffffu, pass);
                if (pass) queue[(head + qlen + __popc(pm & lanemask_lt())) & (kQueue - 1)] = (i << 23) | li;
                qlen += __popc(pm);
                __syncwarp();
                if (qlen >= 32) {
                    flush32(s, queue, head, lane, cam, camp, lights, gb, x0, y0, log);
                    head += 32;
                    qlen -= 32;
                }
            }
        }
    }

    // ---- the pairs left in the warp's queue, then the warp's own pixels ------------------
    // Every pair of a pixel is queued, evaluated and accumulated by the warp that walked
    // its group, so once the warp's queue is empty its pixels are final: no CTA barrier.
    if (qlen > 0) {
        const bool act = lane < qlen;
        const uint32_t e = act ? queue[(head + lane) & (kQueue - 1)] : 0u;
        const uint32_t q = e >> 23, li = e & 0x7fffffu;
        float4 o = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(kCut));
        if (act) o = eval_pair(s, q, li, cam, camp, lights, gb, x0, y0);
        const bool lit = act && __float_as_int(o.w) == kLit;
        log_pair(log, lit, lane, x0 + q % TW, y0 + q / TW, gb.width, li);
        accumulate(s, lit, q, o.x, o.y, o.z);
        __syncwarp();
    }

    // ---- 5. output -----------------------------------------------------------------------
    const uint32_t debug_mode = glb->debug_mode, lcount = glb->light_count;
    // without shadow maps bound, the light-space projection view (mode 11) has no matrix
    if (t == 0 && (glb->has_rc_gi != 0u || (debug_mode == 11u && lcount > 0u)))
        raise_status(status, HL_ERR_NOT_SUPPORTED);
    const float amb = glb->ambient_intensity;
    const float skr = glb->ambient_color[0] * amb, skg = glb->ambient_color[1] * amb,
                skb = glb->ambient_color[2] * amb;
#pragma unroll 1
    while (mine) {
        const uint32_t g = __ffs(mine) - 1;
        mine &= mine - 1;
        const uint32_t gs = g * 32 + lane;
        if (gs >= n_valid) continue;
        const uint32_t i = s.w.order[gs];
        const uint32_t x = x0 + i % TW, y = y0 + i / TW;
        const float4 rd = s.D4[i], rn = s.N4[i];
        const float ar = rd.x, ag = rd.y, ab = rd.z;
        const float ny = rn.y;
        const float ht = fma_(ny, 0.5f, 0.5f);
        // hemisphere ambient (deferred_lighting.wgsl:1196-1199) times ao (1, white SSAO)
        const float hr = fma_(skr, ht, skr * 0.15f * (1.0f - ht)) * ar;
        const float hg = fma_(skg, ht, skg * 0.15f * (1.0f - ht)) * ag;
        const float hb = fma_(skb, ht, skb * 0.15f * (1.0f - ht)) * ab;
        const float4 sum = s.acc[0][i];
        float4 c;
        c.x = sum.x + hr;
        c.y = sum.y + hg;
        c.z = sum.z + hb;
        c.w = 1.0f;
        if (debug_mode == 1u || debug_mode == 2u || debug_mode == 4u || debug_mode == 20u || debug_mode == 21u) {
            c = make_float4(ar, ag, ab, 1.0f);
        } else if (debug_mode == 5u) {
            c = make_float4(fma_(rn.x, 0.5f, 0.5f), fma_(ny, 0.5f, 0.5f), fma_(rn.z, 0.5f, 0.5f), 1.0f);
        } else if (debug_mode == 10u) {
            // shadow factor heatmap (deferred_lighting.wgsl:1049-1064): without shadow maps
            // every light's factor is 1, so the mean is 1 (0 with no light)
            const float sf = lcount > 0u ? 1.0f : 0.0f;
            c = make_float4(sf, sf, sf, 1.0f);
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

template <uint32_t TARGET>
__global__ void __launch_bounds__(f16k::kThreads, 3) shade_f16_kernel(
    const GpuCamera* __restrict__ cam, const DeferredGlobals* __restrict__ glb, const __grid_constant__ GBufView gb,
    const GpuLight* __restrict__ lights, uint32_t n_lights, const __grid_constant__ GridView grid,
    const __grid_constant__ SliceTable tabz, const __grid_constant__ TargetView out, int* __restrict__ status,
    const float4* __restrict__ cand, const __grid_constant__ PairLog log) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    f16k::Smem& s = *reinterpret_cast<f16k::Smem*>(smem_raw);
    // the tile one wave (3 CTAs x SMs) further on is the next to start on this SM
    uint32_t nsm;
    asm("mov.u32 %0, %%nsmid;" : "=r"(nsm));
    const uint32_t next = blockIdx.y * gridDim.x + blockIdx.x + 3u * nsm;
    shade_tile_f16<TARGET>(s, cam, glb, gb, lights, n_lights, grid, tabz.z, out, status, cand, log, blockIdx.x,
                           blockIdx.y, gridDim.x, next < gridDim.x * gridDim.y ? next : ~0u);
}

// Every tile of every view of a batch: CTA b lights tile b - tile_start of the view
// whose [tile_start, next tile_start) holds b.
template <uint32_t TARGET>
__global__ void __launch_bounds__(f16k::kThreads, 3) shade_f16_batched_kernel(const ShadeViewDesc* __restrict__ d,
                                                                             uint32_t n_views,
                                                                             const DeferredGlobals* __restrict__ glb,
                                                                             const GpuLight* __restrict__ lights,
                                                                             uint32_t n_lights, int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    f16k::Smem& s = *reinterpret_cast<f16k::Smem*>(smem_raw);
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
    shade_tile_f16<TARGET>(s, static_cast<const GpuCamera*>(v.camera), glb, gb, lights, n_lights, grid, v.tabz, out,
                           status, v.cand, PairLog{nullptr, nullptr, 0}, local % v.tiles_x, local / v.tiles_x,
                           v.tiles_x, ~0u);
}

// ---- batched views in one persistent launch ------------------------------------------
//
// CTAs take work items by ticket from a device counter: first the froxel binning items
// of every view (bin::bin_item, a slice group of one froxel column), then the (view,
// 32x16 tile) shading items, both in the plan's view order (views with the longest
// lists first); the work list `tiles` names each ticket's view and item or tile.
// A shading item waits until every binning item of its view has finished: that view's
// counter reaches its item count times the launch's epoch. The wait polls with a bound
// (~0.5 s), after which the item reports HL_ERR_TIMEOUT and is skipped instead of
// hanging; it can only wait on items with smaller tickets, which CTAs already running
// hold. Lists written in this launch are read from L2 (COHERENT). The last CTA to
// finish advances the ticket base and the epoch, so a graph replays the launch.
constexpr uint32_t kViewWaitSpins = 1u << 21;

// The two kinds of work item, out of line so that each keeps its own register
// allocation inside the persistent kernel.
__device__ __noinline__ void persistent_bin_item(unsigned char* smem, const BinViewDesc& v, const GpuLight* lights,
                                                 uint32_t n_lights, uint32_t item, uint32_t epoch,
                                                 unsigned long long* chain, int* status) {
    const hl_froxel_params p = v.p;
    bin::bin_item(*reinterpret_cast<bin::ItemSmem*>(smem), static_cast<const GpuCamera*>(v.camera), lights, n_lights,
                  p, v.tab.z, item, v.groups, epoch, chain + v.item_start, v.offsets, v.indices, v.capacity, status,
                  bin::StallTest{~0u, bin::kLookbackSpins});
}

template <uint32_t TARGET>
__device__ __noinline__ void persistent_tile(unsigned char* smem, const ShadeViewDesc& v,
                                             const DeferredGlobals* glb, const GpuLight* lights, uint32_t n_lights,
                                             uint32_t tile, int* status) {
    const GBufView gb = v.gb;
    const GridView grid = v.grid;
    const TargetView out = v.out;
    shade_tile_f16<TARGET, true>(*reinterpret_cast<f16k::Smem*>(smem), static_cast<const GpuCamera*>(v.camera), glb,
                                 gb, lights, n_lights, grid, v.tabz, out, status, v.cand, PairLog{nullptr, nullptr, 0},
                                 tile % v.tiles_x, tile / v.tiles_x, v.tiles_x, ~0u);
}

template <uint32_t TARGET>
__global__ void __launch_bounds__(f16k::kThreads, 3) batch_persistent_kernel(
    const BinViewDesc* __restrict__ bd, const ShadeViewDesc* __restrict__ sd, uint32_t n_views,
    const uint2* __restrict__ tiles, uint32_t total_bin, uint32_t total_tiles, const DeferredGlobals* __restrict__ glb,
    const GpuLight* __restrict__ lights, uint32_t n_lights, unsigned long long* __restrict__ chain,
    BinChainState* __restrict__ state, uint32_t* __restrict__ view_done, int* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    __shared__ uint32_t s_ticket, s_ok;
    __shared__ unsigned long long s_base;
    __shared__ uint32_t s_epoch;
    const uint32_t t = threadIdx.x;
    if (t == 0) {
        // every CTA of the previous launch has finished before this one starts (stream
        // order), so base and epoch are that launch's final values
        s_base = *reinterpret_cast<volatile unsigned long long*>(&state->base);
        s_epoch = *reinterpret_cast<volatile uint32_t*>(&state->epoch) + 1u;
    }
    const uint32_t total = total_bin + total_tiles;
    for (;;) {
        __syncthreads();
        if (t == 0) s_ticket = uint32_t(atomicAdd(&state->ticket, 1ull) - s_base);
        __syncthreads();
        const uint32_t tk = s_ticket, epoch = s_epoch;
        if (tk >= total) break;
        const uint2 it = __ldg(&tiles[tk]);  // (view, binning item) or (view, tile)
        if (tk < total_bin) {
            persistent_bin_item(smem_raw, bd[it.x], lights, n_lights, it.y, epoch, chain, status);
            if (t == 0) {
                __threadfence();
                atomicAdd(&view_done[it.x], 1u);
            }
        } else {
            const ShadeViewDesc& v = sd[it.x];
            if (t == 0) {
                const BinViewDesc& b = bd[it.x];
                const uint32_t items = b.p.grid_x * b.p.grid_y * b.groups;
                const uint32_t want = items * epoch;  // the view's items of this launch have finished
                uint32_t ok = 1, spins = 0;
                while (*reinterpret_cast<volatile uint32_t*>(&view_done[it.x]) < want) {
                    if (++spins > kViewWaitSpins) {
                        raise_status(status, HL_ERR_TIMEOUT);
                        ok = 0;
                        break;
                    }
                    __nanosleep(256);
                }
                __threadfence();
                s_ok = ok;
            }
            __syncthreads();
            if (s_ok) persistent_tile<TARGET>(smem_raw, v, glb, lights, n_lights, it.y, status);
        }
    }
    // the last CTA to finish advances the ticket base and the epoch for the next launch
    if (t == 0) {
        __threadfence();
        if (atomicAdd(&state->done, 1u) == gridDim.x - 1u) {
            state->done = 0u;
            state->base += total + gridDim.x;  // every CTA drew one ticket past the end
            state->epoch = s_epoch;
            __threadfence();
        }
    }
}

// Raises KERN's dynamic shared-memory limit once per device. The kernel is a template
// argument so that every kernel has its own record: instantiations of one kernel
// template for different targets share a signature but are different functions.
template <auto KERN>
cudaError_t smem_attr(int smem) {
    static unsigned long long attr_devices = 0;  // devices on which KERN's limit is raised
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 64 && !(attr_devices & (1ull << dev))) {
        cudaError_t e = cudaFuncSetAttribute(KERN, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
        if (e != cudaSuccess) return e;
        attr_devices |= 1ull << dev;
    }
    return cudaSuccess;
}

template <uint32_t TARGET>
cudaError_t launch_target(const void* camera, const void* globals, const GBufView& gb, const void* lights, uint32_t n,
                          const GridView& grid, const SliceTable& tab, const TargetView& out, int* status,
                          float4* cand, const PairLog& log, cudaStream_t stream) {
    auto kern = shade_f16_kernel<TARGET>;
    const int smem = int(sizeof(f16k::Smem));
    cudaError_t ea = smem_attr<shade_f16_kernel<TARGET>>(smem);
    if (ea != cudaSuccess) return ea;
    if (n > 0) {
        cudaError_t e = launch_prep_cand(camera, lights, n, true, cand, stream);
        if (e != cudaSuccess) return e;
    }
    const dim3 g((gb.width + f16k::TW - 1) / f16k::TW, (gb.height + f16k::TH - 1) / f16k::TH);
    return launch_pdl(kern, g, dim3(f16k::kThreads), smem, stream, static_cast<const GpuCamera*>(camera),
                      static_cast<const DeferredGlobals*>(globals), gb, static_cast<const GpuLight*>(lights), n, grid,
                      tab, out, status, static_cast<const float4*>(cand), log);
}

}  // namespace

size_t batch_persistent_smem() { return std::max(sizeof(bin::ItemSmem), sizeof(f16k::Smem)); }

cudaError_t launch_batch_persistent(uint32_t target_format, const BinViewDesc* bd, const ShadeViewDesc* sd,
                                    uint32_t n_views, const uint2* tiles, uint32_t total_bin, uint32_t total_tiles,
                                    uint32_t grid, const void* globals, const void* lights, uint32_t n,
                                    unsigned long long* chain, BinChainState* state, uint32_t* view_done,
                                    int* status, cudaStream_t stream) {
    const int smem = int(batch_persistent_smem());
    const bool h = target_format == HL_TARGET_RGBA16F;
    auto kern = h ? batch_persistent_kernel<HL_TARGET_RGBA16F> : batch_persistent_kernel<HL_TARGET_RGBA32F>;
    cudaError_t e = h ? smem_attr<batch_persistent_kernel<HL_TARGET_RGBA16F>>(smem)
                      : smem_attr<batch_persistent_kernel<HL_TARGET_RGBA32F>>(smem);
    if (e != cudaSuccess) return e;
    kern<<<grid, f16k::kThreads, smem, stream>>>(bd, sd, n_views, tiles, total_bin, total_tiles,
                                                  static_cast<const DeferredGlobals*>(globals),
                                                  static_cast<const GpuLight*>(lights), n, chain, state, view_done,
                                                  status);
    return cudaGetLastError();
}

uint32_t batch_persistent_grid(int device) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess || sms <= 0) sms = 1;
    int per_sm = 0;
    // the shared-memory limit first: the occupancy query respects the kernel's attribute
    if (smem_attr<batch_persistent_kernel<HL_TARGET_RGBA32F>>(int(batch_persistent_smem())) != cudaSuccess ||
        smem_attr<batch_persistent_kernel<HL_TARGET_RGBA16F>>(int(batch_persistent_smem())) != cudaSuccess)
        cudaGetLastError();
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_persistent_kernel<HL_TARGET_RGBA32F>,
                                                      f16k::kThreads, batch_persistent_smem()) != cudaSuccess ||
        per_sm <= 0)
        per_sm = 1;
    return uint32_t(sms) * uint32_t(per_sm);
}

cudaError_t launch_shade_f16_batched(uint32_t target_format, const ShadeViewDesc* descs, uint32_t n_views,
                                     uint32_t total_tiles, const void* globals, const void* lights, uint32_t n,
                                     int* status, cudaStream_t stream) {
    const int smem = int(sizeof(f16k::Smem));
    const bool h = target_format == HL_TARGET_RGBA16F;
    auto kern = h ? shade_f16_batched_kernel<HL_TARGET_RGBA16F> : shade_f16_batched_kernel<HL_TARGET_RGBA32F>;
    cudaError_t e = h ? smem_attr<shade_f16_batched_kernel<HL_TARGET_RGBA16F>>(smem)
                      : smem_attr<shade_f16_batched_kernel<HL_TARGET_RGBA32F>>(smem);
    if (e != cudaSuccess) return e;
    kern<<<total_tiles, f16k::kThreads, smem, stream>>>(descs, n_views, static_cast<const DeferredGlobals*>(globals),
                                                         static_cast<const GpuLight*>(lights), n, status);
    return cudaGetLastError();
}

cudaError_t launch_shade_f16(uint32_t target_format, const void* camera, const void* globals, const GBufView& gb,
                             const void* lights, uint32_t n_lights, const GridView& grid, const SliceTable& tab,
                             const TargetView& out, int* status, float4* cand, const PairLog& log,
                             cudaStream_t stream) {
    if (target_format == HL_TARGET_RGBA16F)
        return launch_target<HL_TARGET_RGBA16F>(camera, globals, gb, lights, n_lights, grid, tab, out, status, cand,
                                                 log, stream);
    return launch_target<HL_TARGET_RGBA32F>(camera, globals, gb, lights, n_lights, grid, tab, out, status, cand, log,
                                             stream);
}

}  // namespace hl
