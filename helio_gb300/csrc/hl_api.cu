// hl_api.cu — the C ABI (include/helio_gb300.h): context, argument validation,
// scratch memory and dispatch to the sm_103a kernels. Host code only.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "hl_common.cuh"
#include "hl_host.h"
#include "hl_internal.h"

namespace {

using namespace hl_host;

hl_status shade_common(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                       const void* lights, uint32_t n_lights, const hl_light_grid* grid, const hl_target* radiance,
                       uint32_t* stats, void* stream, const hl_shadow_maps* shadows = nullptr,
                       const hl_rc_cascade* rc = nullptr) {
    hl_status s = check_common(ctx, camera, lights, n_lights);
    if (s != HL_OK) return s;
    if (!globals || !aligned(globals, 16)) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "globals is NULL or misaligned");
    hl::GBufView gv;
    if ((s = check_gbuffer(ctx, gbuffer, gv)) != HL_OK) return s;
    hl::GridView grv;
    hl::SliceTable tab;
    std::memset(&tab, 0, sizeof tab);
    if ((s = check_grid(ctx, grid, gbuffer->width, gbuffer->height, grv, tab)) != HL_OK) return s;
    hl::TargetView tv{};
    if (!stats) {
        if ((s = check_target(ctx, radiance, gbuffer->width, tv)) != HL_OK) return s;
    } else if (!aligned(stats, 4)) {
        return fail(ctx, HL_ERR_LAYOUT, "stats pointer not 4-byte aligned");
    }
    hl::ExtView sv{};
    if (shadows) {
        const hl_shadow_maps& m = *shadows;
        if (!m.dynamic_atlas || !m.static_atlas || !m.matrices || !m.config)
            return fail(ctx, HL_ERR_INVALID_ARGUMENT, "shadow maps: an atlas, the matrices or the config is NULL");
        if (!aligned(m.dynamic_atlas, 4) || !aligned(m.static_atlas, 4) || !aligned(m.matrices, 16) ||
            !aligned(m.config, 16))
            return fail(ctx, HL_ERR_LAYOUT, "shadow maps: atlases need 4-byte, matrices and config 16-byte alignment");
        if (m.size == 0 || m.size > 16384 || m.layers == 0 || m.layers > 65536)
            return fail(ctx, HL_ERR_SIZE, "shadow maps: %u layers of %u texels (1..65536 layers, 1..16384 texels)",
                        m.layers, m.size);
        if (m.reserved != 0) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "shadow maps: reserved field must be 0");
        sv = hl::ExtView{m.dynamic_atlas, m.static_atlas, static_cast<const float*>(m.matrices),
                            static_cast<const unsigned char*>(m.config), ctx->d_status,
                            reinterpret_cast<const float*>(static_cast<const unsigned char*>(globals) + 64), m.size,
                            m.layers, m.max_shadow_lights, float(m.size)};
    }
    if (rc) {
        const uint32_t need_w = HL_RC_PROBE_DIM * HL_RC_DIR_DIM, need_h = HL_RC_PROBE_DIM * HL_RC_PROBE_DIM * HL_RC_DIR_DIM;
        if (!rc->texels) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "rc cascade texels are NULL");
        if (!aligned(rc->texels, 16) || rc->pitch % 16 != 0)
            return fail(ctx, HL_ERR_LAYOUT, "rc cascade pointer/pitch not 16-byte aligned");
        if (rc->width < need_w || rc->height < need_h || rc->pitch < uint64_t(rc->width) * 8)
            return fail(ctx, HL_ERR_SIZE, "rc cascade is %ux%u (pitch %llu), needs at least %ux%u", rc->width,
                        rc->height, (unsigned long long)rc->pitch, need_w, need_h);
        sv.rc = static_cast<const unsigned char*>(rc->texels);
        sv.rc_pitch = rc->pitch;
        sv.status = ctx->d_status;
    }
    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    if ((s = ensure(ctx, ctx->shade_cand, ctx->shade_cand_cap, hl::cand_table_len(n_lights > 0 ? n_lights : 1),
                    "shade light table")) !=
        HL_OK)
        return s;
    cudaError_t e = hl::launch_shade(gbuffer->layout, grid->kind, stats ? HL_TARGET_RGBA32F : radiance->format, camera,
                                     globals, gv, lights, n_lights, grv, tab, tv, stats, ctx->d_status,
                                     ctx->shade_cand, ctx->pair_log, as_stream(stream), (shadows || rc) ? &sv : nullptr);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "shade launch");
    return HL_OK;
}

}  // namespace

extern "C" {

uint32_t hl_abi_version(void) { return HL_ABI_VERSION; }

const char* hl_status_string(hl_status s) {
    switch (s) {
        case HL_OK: return "ok";
        case HL_ERR_INVALID_ARGUMENT: return "invalid argument";
        case HL_ERR_LAYOUT: return "layout or alignment mismatch";
        case HL_ERR_SIZE: return "size beyond supported limits";
        case HL_ERR_CUDA: return "CUDA runtime error";
        case HL_ERR_TIMEOUT: return "device-side wait timed out";
        case HL_ERR_CAPACITY: return "froxel index capacity exceeded";
        case HL_ERR_DEVICE_BOUNDS: return "device-side bounds check failed";
        case HL_ERR_NOT_SUPPORTED: return "not supported";
        default: return "unknown status";
    }
}

hl_status hl_create(hl_ctx** out, int device) {
    if (!out) return HL_ERR_INVALID_ARGUMENT;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return HL_ERR_CUDA;
    }
    if (device < 0 || device >= n) return HL_ERR_INVALID_ARGUMENT;
    DeviceGuard dg(device);
    if (!dg.ok) return HL_ERR_CUDA;
    hl_ctx* ctx = new hl_ctx();
    ctx->device = device;
    if (cudaMalloc(&ctx->d_status, sizeof(int)) != cudaSuccess || cudaMemset(ctx->d_status, 0, sizeof(int)) != cudaSuccess) {
        cudaFree(ctx->d_status);
        delete ctx;
        return HL_ERR_CUDA;
    }
    *out = ctx;
    return HL_OK;
}

hl_status hl_destroy(hl_ctx* ctx) {
    if (!ctx) return HL_OK;
    DeviceGuard dg(ctx->device);
    cudaDeviceSynchronize();
    cudaFree(ctx->d_status);
    cudaFree(ctx->bin_lights);
    cudaFree(ctx->froxel_counts);
    cudaFree(ctx->adjoint_partials);
    cudaFree(ctx->shade_cand);
    cudaFree(ctx->froxel_chain);
    cudaFree(ctx->bin_state);
    cudaFree(ctx->frag_lights);
    delete ctx;
    return HL_OK;
}

const char* hl_last_error_message(const hl_ctx* ctx) { return ctx ? ctx->last_error.c_str() : ""; }

hl_status hl_sync_status(hl_ctx* ctx, void* stream) {
    if (!ctx) return HL_ERR_INVALID_ARGUMENT;
    DeviceGuard dg(ctx->device);
    cudaError_t e = cudaStreamSynchronize(as_stream(stream));
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
    int v = 0;
    e = cudaMemcpy(&v, ctx->d_status, sizeof v, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "status readback");
    if (v != 0) {
        cudaMemset(ctx->d_status, 0, sizeof(int));
        return fail(ctx, v, "device reported: %s", hl_status_string(v));
    }
    return HL_OK;
}

uint32_t hl_tile_count(uint32_t w, uint32_t h) {
    const uint64_t t = uint64_t((w + 15ull) / 16ull) * uint64_t((h + 15ull) / 16ull);
    return (t == 0 || t * hl::kMaxPerTile > 0xFFFFFFFFull) ? 0u : uint32_t(t);
}

hl_status hl_bin_tiles_ref(hl_ctx* ctx, const void* camera, const void* lights, uint32_t n, uint32_t W, uint32_t H,
                           uint32_t* lists, uint32_t* counts, void* stream) {
    hl_status s = check_common(ctx, camera, lights, n);
    if (s != HL_OK) return s;
    if (W == 0 || H == 0) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "viewport %ux%u", W, H);
    const uint32_t tiles = hl_tile_count(W, H);
    if (tiles == 0) return fail(ctx, HL_ERR_SIZE, "tile grid overflow: viewport %ux%u too large", W, H);
    if (!lists || !counts) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "tile lists/counts is NULL");
    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    cudaStream_t st = as_stream(stream);
    if (n == 0) {  // LightCullPass::execute clears both buffers (light-cull/src/lib.rs:285-292)
        cudaError_t e = cudaMemsetAsync(lists, 0, size_t(tiles) * hl::kMaxPerTile * 4, st);
        if (e == cudaSuccess) e = cudaMemsetAsync(counts, 0, size_t(tiles) * 4, st);
        return e == cudaSuccess ? HL_OK : cuda_fail(ctx, e, "clear tile lists");
    }
    if ((s = ensure(ctx, ctx->bin_lights, ctx->bin_lights_cap, n, "bin light scratch")) != HL_OK) return s;
    cudaError_t e = hl::launch_prep_bin_lights(camera, lights, n, false, ctx->bin_lights, st);
    if (e == cudaSuccess) e = hl::launch_bin_tiles_ref(camera, ctx->bin_lights, n, W, H, lists, counts, st);
    return e == cudaSuccess ? HL_OK : cuda_fail(ctx, e, "bin_tiles_ref launch");
}

hl_status hl_froxel_slice_table(const hl_froxel_params* p, float* out) {
    hl_status s = check_froxel_params(nullptr, p);
    if (s != HL_OK) return s;
    if (!out) return HL_ERR_INVALID_ARGUMENT;
    slice_table(*p, out);
    return HL_OK;
}

hl_status hl_bin_froxels(hl_ctx* ctx, const void* camera, const void* lights, uint32_t n,
                         const hl_froxel_params* p, const hl_froxel_lists* out, void* stream) {
    hl_status s = check_common(ctx, camera, lights, n);
    if (s != HL_OK) return s;
    if ((s = check_froxel_params(ctx, p)) != HL_OK) return s;
    if (!out || !out->offsets) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "froxel output offsets is NULL");
    if (out->capacity > 0 && !out->indices) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "froxel indices is NULL");
    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    // single-launch binning state: chain words (zeroed when allocated: epoch 0 is never
    // used) and the work-item ticket counter
    const uint32_t groups = hl::bin_item_groups(ctx->device, *p);
    const uint64_t items = uint64_t(p->grid_x) * p->grid_y * groups;
    if (items > 0x7FFFFFFFull) return fail(ctx, HL_ERR_SIZE, "froxel grid has %llu work items", (unsigned long long)items);
    unsigned long long* old_chain = ctx->froxel_chain;
    if ((s = ensure(ctx, ctx->froxel_chain, ctx->froxel_chain_cap, items, "froxel chain scratch")) != HL_OK) return s;
    cudaStream_t st = as_stream(stream);
    cudaError_t e = cudaSuccess;
    if (ctx->froxel_chain != old_chain)
        e = cudaMemsetAsync(ctx->froxel_chain, 0, sizeof(unsigned long long) * ctx->froxel_chain_cap, st);
    if (e == cudaSuccess && !ctx->bin_state) {
        e = cudaMalloc(&ctx->bin_state, sizeof(hl::BinChainState));
        if (e == cudaSuccess) e = cudaMemsetAsync(ctx->bin_state, 0, sizeof(hl::BinChainState), st);
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "froxel chain set-up");
    hl::SliceTable tab;
    std::memset(&tab, 0, sizeof tab);
    slice_table(*p, tab.z);
    const uint32_t stall_item = ctx->stall_item, stall_spins = ctx->stall_spins;
    ctx->stall_item = ~0u;  // one call only
    e = hl::launch_bin_froxels_items(camera, lights, n, *p, tab, groups, out->offsets, out->indices, out->capacity,
                                     ctx->d_status, ctx->froxel_chain, ctx->bin_state, stall_item, stall_spins, st);
    return e == cudaSuccess ? HL_OK : cuda_fail(ctx, e, "bin_froxels launch");
}

hl_status hl_inject_binning_stall(hl_ctx* ctx, uint32_t item, uint32_t spins) {
    if (!ctx) return HL_ERR_INVALID_ARGUMENT;
    if (spins == 0 || spins > (1u << 20))
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "stall test: %u polls (1..2^20)", spins);
    ctx->stall_item = item;
    ctx->stall_spins = spins;
    return HL_OK;
}

hl_status hl_shade(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer, const void* lights,
                   uint32_t n_lights, const hl_light_grid* grid, const hl_target* radiance, void* stream) {
    return shade_common(ctx, camera, globals, gbuffer, lights, n_lights, grid, radiance, nullptr, stream);
}

hl_status hl_shade_shadowed(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                            const void* lights, uint32_t n_lights, const hl_light_grid* grid,
                            const hl_shadow_maps* shadows, const hl_target* radiance, void* stream) {
    return shade_common(ctx, camera, globals, gbuffer, lights, n_lights, grid, radiance, nullptr, stream, shadows);
}

hl_status hl_shade_ex(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                      const void* lights, uint32_t n_lights, const hl_light_grid* grid,
                      const hl_shade_bindings* bindings, const hl_target* radiance, void* stream) {
    return shade_common(ctx, camera, globals, gbuffer, lights, n_lights, grid, radiance, nullptr, stream,
                        bindings ? bindings->shadows : nullptr, bindings ? bindings->rc : nullptr);
}

hl_status hl_shade_stats(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                         const void* lights, uint32_t n_lights, const hl_light_grid* grid, uint32_t* counts,
                         void* stream) {
    if (!counts) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "stats counts is NULL");
    return shade_common(ctx, camera, globals, gbuffer, lights, n_lights, grid, nullptr, counts, stream);
}

hl_status hl_set_pair_log(hl_ctx* ctx, uint32_t* pairs, uint32_t capacity, uint32_t* count) {
    if (!ctx) return HL_ERR_INVALID_ARGUMENT;
    if (!pairs) {
        ctx->pair_log = hl::PairLog{nullptr, nullptr, 0};
        return HL_OK;
    }
    if (!count || !aligned(pairs, 8) || !aligned(count, 4))
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "pair log: count is NULL or pairs/count misaligned");
    ctx->pair_log = hl::PairLog{reinterpret_cast<uint2*>(pairs), count, capacity};
    return HL_OK;
}

hl_status hl_shade_adjoint(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                           const void* lights, uint32_t n_lights, const hl_light_grid* grid, const float* d_radiance,
                           uint64_t d_radiance_pitch, double* d_lights, float* d_pixels, void* stream) {
    hl_status s = check_common(ctx, camera, lights, n_lights);
    if (s != HL_OK) return s;
    if (n_lights > HL_ADJOINT_MAX_LIGHTS)
        return fail(ctx, HL_ERR_SIZE, "adjoint: n_lights %u exceeds %u", n_lights, HL_ADJOINT_MAX_LIGHTS);
    if (!globals || !aligned(globals, 16)) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "globals is NULL or misaligned");
    hl::GBufView gv;
    if ((s = check_gbuffer(ctx, gbuffer, gv)) != HL_OK) return s;
    hl::GridView grv;
    hl::SliceTable tab;
    std::memset(&tab, 0, sizeof tab);
    if ((s = check_grid(ctx, grid, gbuffer->width, gbuffer->height, grv, tab)) != HL_OK) return s;
    const uint32_t W = gbuffer->width, H = gbuffer->height;
    if (!d_radiance || !aligned(d_radiance, 16) || d_radiance_pitch % 16 != 0 || d_radiance_pitch < uint64_t(W) * 16)
        return fail(ctx, HL_ERR_LAYOUT, "d_radiance must be RGBA32F, 16-byte aligned, pitch >= %u bytes", W * 16);
    if (n_lights > 0 && (!d_lights || !aligned(d_lights, 8)))
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "d_lights is NULL or not 8-byte aligned");
    if (!d_pixels || !aligned(d_pixels, 4)) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "d_pixels is NULL or misaligned");
    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    const uint32_t G = hl::adjoint_grid_size(ctx->device, W, H);
    const size_t need = size_t(G) * (n_lights > 0 ? n_lights : 1) * 8;
    if ((s = ensure(ctx, ctx->adjoint_partials, ctx->adjoint_partials_cap, need, "adjoint partials")) != HL_OK) return s;
    cudaError_t e = hl::launch_shade_adjoint(gbuffer->layout, grid->kind, camera, globals, gv, lights, n_lights, grv, tab,
                                             d_radiance, d_radiance_pitch, ctx->adjoint_partials, G, d_lights,
                                             d_pixels, ctx->d_status, as_stream(stream));
    return e == cudaSuccess ? HL_OK : cuda_fail(ctx, e, "shade adjoint launch");
}

hl_status hl_shade_fragments(hl_ctx* ctx, const void* camera, const hl_fragment_params* params, const void* fragments,
                             uint32_t n_fragments, const void* lights, uint32_t n_lights,
                             const uint32_t* light_entity_indices, const void* transforms, uint32_t n_transforms,
                             const hl_light_grid* grid, float* out_rgba, void* stream) {
    hl_status s = check_common(ctx, camera, lights, n_lights);
    if (s != HL_OK) return s;
    if (!params) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "fragment params is NULL");
    if (params->mode > HL_FRAGMENTS_TRANSPARENT)
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "unknown fragment mode %u", params->mode);
    if (n_fragments > 0 && (!fragments || !aligned(fragments, 16) || !out_rgba || !aligned(out_rgba, 16)))
        return fail(ctx, HL_ERR_LAYOUT, "fragments / out_rgba NULL or not 16-byte aligned");
    if (n_fragments > (1u << 30)) return fail(ctx, HL_ERR_SIZE, "%u fragments exceed 2^30", n_fragments);
    if (light_entity_indices) {
        if (params->mode != HL_FRAGMENTS_FORWARD)
            return fail(ctx, HL_ERR_INVALID_ARGUMENT, "light entity indices are read in the forward mode only");
        if (!aligned(light_entity_indices, 4) || (n_transforms > 0 && (!transforms || !aligned(transforms, 4))))
            return fail(ctx, HL_ERR_LAYOUT, "entity indices / transforms NULL or not 4-byte aligned");
    }
    if (!grid || !grid->lists || !grid->counts) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "light grid is NULL");
    hl::GridView gv;
    hl::SliceTable tab;
    std::memset(&gv, 0, sizeof gv);
    std::memset(&tab, 0, sizeof tab);
    gv.lists = grid->lists;
    gv.counts = grid->counts;
    if (grid->kind == HL_GRID_TILES) {
        // the fragments name their tiles through num_tiles_x; lists_capacity bounds them
        if (grid->lists_capacity < hl::kMaxPerTile || params->num_tiles_x == 0)
            return fail(ctx, HL_ERR_INVALID_ARGUMENT,
                        "tile grid for fragments needs lists_capacity (tiles x 64) and num_tiles_x");
        gv.tiles = grid->lists_capacity / hl::kMaxPerTile;
        gv.lists_capacity = grid->lists_capacity;
    } else if (grid->kind == HL_GRID_FROXELS) {
        if ((s = check_froxel_params(ctx, &grid->froxel)) != HL_OK) return s;
        gv.fp = grid->froxel;
        gv.lists_capacity = grid->lists_capacity ? grid->lists_capacity : 0xFFFFFFFFu;
        slice_table(grid->froxel, tab.z);
    } else {
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "unknown light grid kind %u", grid->kind);
    }
    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    const size_t need = size_t(n_lights > 0 ? n_lights : 1) * hl::frag_light_bytes();
    if ((s = ensure(ctx, ctx->frag_lights, ctx->frag_lights_cap, need, "fragment light records")) != HL_OK) return s;
    cudaError_t e = hl::launch_shade_fragments(camera, *params, fragments, n_fragments, lights, n_lights,
                                               light_entity_indices, transforms, n_transforms, grid->kind, gv, tab,
                                               ctx->frag_lights, out_rgba, ctx->d_status, as_stream(stream));
    return e == cudaSuccess ? HL_OK : cuda_fail(ctx, e, "shade fragments launch");
}

hl_status hl_probe_fp32_peak(hl_ctx* ctx, double* tflops) {
    if (!ctx || !tflops) return HL_ERR_INVALID_ARGUMENT;
    DeviceGuard dg(ctx->device);
    cudaError_t e = hl::run_fp32_probe(ctx->device, tflops);
    return e == cudaSuccess ? HL_OK : cuda_fail(ctx, e, "fp32 probe");
}

}  // extern "C"
