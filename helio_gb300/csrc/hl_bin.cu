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
#include "hl_bin_item.cuh"
#include "hl_common.cuh"
#include "hl_internal.h"

namespace hl {

namespace {

using namespace bin;
constexpr int kBinWarps = bin::kWarps;
constexpr int kBinThreads = bin::kThreads;
// CTAs of the single-launch binning: 16 warps, two resident per SM
constexpr int kItemWarps = 16;
constexpr int kItemMinBlocks = 2;

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

// ---- single launch: count, chained scan across work items, fill ---------------------
//
// Each CTA takes a work item by ticket (a device counter, so item k waits only for
// items that started before it) and bins it (bin::bin_item: its lights transformed to
// view space as it gathers them, so no separate preparation launch). The ticket base
// and the epoch live on the device and the last CTA of a launch advances them, so a
// launch recorded in a CUDA graph can be replayed.
template <int NW>
__global__ void __launch_bounds__(NW * 32, kItemMinBlocks) bin_froxels_items_kernel(
    const GpuCamera* __restrict__ cam, const GpuLight* __restrict__ lights, uint32_t n, hl_froxel_params p,
    const __grid_constant__ SliceTable tab, uint32_t groups, uint32_t* __restrict__ offsets,
    uint32_t* __restrict__ indices, uint32_t capacity, int* __restrict__ status,
    unsigned long long* __restrict__ chain, BinChainState* __restrict__ state, StallTest test) {
    __shared__ ItemSmemT<NW> sm;
    __shared__ uint32_t s_item, s_epoch;
    const uint32_t items = p.grid_x * p.grid_y * groups;
    if (threadIdx.x == 0) {
        // every CTA of the previous launch has finished before this one starts (stream
        // order), so base and epoch are that launch's final values
        const unsigned long long base = *reinterpret_cast<volatile unsigned long long*>(&state->base);
        s_epoch = *reinterpret_cast<volatile uint32_t*>(&state->epoch) + 1u;
        s_item = uint32_t(atomicAdd(&state->ticket, 1ull) - base);
    }
    // while the ticket is drawn: the camera and the lights of the first gather step
    // (one 128-byte line each, every item reads them) on their way to this SM's L1
    if (threadIdx.x < 3) prefetch_l1(reinterpret_cast<const unsigned char*>(cam) + 128 * threadIdx.x);
#pragma unroll
    for (uint32_t u = 0; u < kGatherU; ++u) {
        const uint32_t i = u * NW * 32 + threadIdx.x;
        if (i < n) prefetch_l1(lights + i);
    }
    __syncthreads();
    const uint32_t item = s_item, epoch = s_epoch;
    if (item >= items) {  // launches overlapping on one context: refused
        if (threadIdx.x == 0) raise_status(status, HL_ERR_DEVICE_BOUNDS);
        return;
    }
    pdl_launch_dependents();  // the shading launch's light table and pixel set-up may start
    bin_item<NW>(sm, cam, lights, n, p, tab.z, item, groups, epoch, chain, offsets, indices, capacity, status, test);
    // the last CTA to finish advances the ticket base and the epoch for the next launch
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&state->done, 1u) == items - 1u) {
            state->done = 0u;
            state->base += items;
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

uint32_t bin_item_groups(int device, const hl_froxel_params& p) {
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device) != cudaSuccess) sms = 1;
    // each item gathers all the lights for its column: split columns into slice groups
    // only when there are too few columns to give every other SM one
    return item_groups(p, uint32_t(sms > 1 ? sms : 2) / 2u);
}

cudaError_t launch_bin_froxels_items(const void* camera, const void* lights, uint32_t n, const hl_froxel_params& p,
                                     const SliceTable& tab, uint32_t groups, uint32_t* offsets, uint32_t* indices,
                                     uint32_t capacity, int* status, unsigned long long* chain, BinChainState* state,
                                     uint32_t stall_item, uint32_t stall_spins, cudaStream_t stream) {
    const uint32_t items = p.grid_x * p.grid_y * groups;
    const StallTest test{stall_item, stall_item == ~0u ? kLookbackSpins : stall_spins};
    // launched plainly: it starts after its predecessor has finished, so two binning
    // launches of one context (sharing ticket and chain) never overlap
    bin_froxels_items_kernel<kItemWarps><<<items, kItemWarps * 32, 0, stream>>>(
        static_cast<const GpuCamera*>(camera), static_cast<const GpuLight*>(lights), n, p, tab, groups, offsets,
        indices, capacity, status, chain, state, test);
    return cudaGetLastError();
}

}  // namespace hl
