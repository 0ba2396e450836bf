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
#include "hl_internal.h"

struct hl_ctx {
    int device = 0;
    int* d_status = nullptr;          // device status word (first error wins)
    hl::BinLight* bin_lights = nullptr;
    uint32_t bin_lights_cap = 0;
    uint32_t* froxel_counts = nullptr;
    uint32_t froxel_counts_cap = 0;
    std::string last_error;
};

namespace {

using hl::BinLight;

struct DeviceGuard {
    int prev = -1;
    bool ok = true;
    explicit DeviceGuard(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        if (prev != dev) ok = cudaSetDevice(dev) == cudaSuccess;
    }
    ~DeviceGuard() {
        int cur = -1;
        if (prev >= 0 && cudaGetDevice(&cur) == cudaSuccess && cur != prev) cudaSetDevice(prev);
    }
};

hl_status fail(hl_ctx* ctx, hl_status code, const char* fmt, ...) {
    if (ctx) {
        char buf[512];
        va_list ap;
        va_start(ap, fmt);
        std::vsnprintf(buf, sizeof buf, fmt, ap);
        va_end(ap);
        ctx->last_error = buf;
    }
    return code;
}

hl_status cuda_fail(hl_ctx* ctx, cudaError_t e, const char* where) {
    return fail(ctx, HL_ERR_CUDA, "%s: %s (%s)", where, cudaGetErrorName(e), cudaGetErrorString(e));
}

inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// Grows a device scratch buffer; waits for the device before freeing the old one.
template <class T>
hl_status ensure(hl_ctx* ctx, T*& buf, uint32_t& cap, size_t need, const char* what) {
    if (need <= cap && buf) return HL_OK;
    if (need > 0xFFFFFFFFull) return fail(ctx, HL_ERR_SIZE, "%s: %zu entries exceed the 32-bit limit", what, need);
    if (buf) {
        cudaDeviceSynchronize();
        cudaFree(buf);
        buf = nullptr;
        cap = 0;
    }
    size_t n = need < 64 ? 64 : need;
    n = n + n / 4;
    if (n > 0xFFFFFFFFull) n = need;
    cudaError_t e = cudaMalloc(&buf, n * sizeof(T));
    if (e != cudaSuccess) return cuda_fail(ctx, e, what);
    cap = uint32_t(n);
    return HL_OK;
}

hl_status check_froxel_params(hl_ctx* ctx, const hl_froxel_params* p) {
    if (!p) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "froxel params is NULL");
    if (p->grid_x == 0 || p->grid_y == 0 || p->grid_z == 0 || p->width == 0 || p->height == 0)
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "froxel grid %ux%ux%u over %ux%u has a zero dimension", p->grid_x,
                    p->grid_y, p->grid_z, p->width, p->height);
    if (p->grid_z > hl::kMaxSlices)
        return fail(ctx, HL_ERR_SIZE, "froxel grid_z %u exceeds %u slices", p->grid_z, hl::kMaxSlices);
    if (p->grid_x > p->width || p->grid_y > p->height)
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "froxel grid %ux%u is finer than the %ux%u viewport", p->grid_x,
                    p->grid_y, p->width, p->height);
    const uint64_t F = uint64_t(p->grid_x) * p->grid_y * p->grid_z;
    if (F + 1 > 0xFFFFFFFFull || uint64_t(p->grid_x) * p->grid_y > 0x7FFFFFFFull)
        return fail(ctx, HL_ERR_SIZE, "froxel grid has %llu froxels", (unsigned long long)F);
    if (!(p->slice_near > 0.0f) || !std::isfinite(p->slice_near) || !std::isfinite(p->slice_far))
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "froxel slice_near %g / slice_far %g", double(p->slice_near),
                    double(p->slice_far));
    if (p->reserved != 0) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "froxel params reserved field must be 0");
    return HL_OK;
}

void slice_table(const hl_froxel_params& p, float* out) {
    const double nr = double(p.slice_near);
    const double F = std::fmax(double(p.slice_far), 2.0 * nr);
    out[0] = 0.0f;
    for (uint32_t k = 1; k < p.grid_z; ++k) out[k] = float(nr * std::pow(F / nr, double(k) / double(p.grid_z)));
    out[p.grid_z] = float(F);
}

// Bytes per texel of each plane, per layout, and the access alignment.
struct PlaneSpec {
    int planes;
    uint32_t bpp[HL_GBUF_MAX_PLANES];
    uint32_t align[HL_GBUF_MAX_PLANES];
};
const PlaneSpec kPlaneSpecs[3] = {
    {5, {4, 8, 4, 8, 4, 0}, {4, 8, 4, 8, 4, 1}},  // reference
    {3, {16, 16, 4, 0, 0, 0}, {16, 16, 4, 1, 1, 1}},  // F32
    {4, {8, 4, 2, 4, 0, 0}, {8, 4, 2, 4, 1, 1}},  // F16
};

hl_status check_gbuffer(hl_ctx* ctx, const hl_gbuffer* g, hl::GBufView& v) {
    if (!g) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "gbuffer is NULL");
    if (g->layout > HL_GBUF_F16) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "unknown gbuffer layout %u", g->layout);
    if (g->width == 0 || g->height == 0) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "gbuffer is %ux%u", g->width, g->height);
    if (g->width > (1u << 16) || g->height > (1u << 16))
        return fail(ctx, HL_ERR_SIZE, "gbuffer %ux%u exceeds 65536 pixels per side", g->width, g->height);
    const PlaneSpec& s = kPlaneSpecs[g->layout];
    std::memset(&v, 0, sizeof v);
    for (int i = 0; i < s.planes; ++i) {
        if (!g->planes[i]) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "gbuffer plane %d is NULL", i);
        if (!aligned(g->planes[i], s.align[i]) || g->pitch[i] % s.align[i] != 0)
            return fail(ctx, HL_ERR_LAYOUT, "gbuffer plane %d pointer/pitch not %u-byte aligned", i, s.align[i]);
        if (g->pitch[i] < uint64_t(g->width) * s.bpp[i])
            return fail(ctx, HL_ERR_LAYOUT, "gbuffer plane %d pitch %llu < %u x %u bytes", i,
                        (unsigned long long)g->pitch[i], g->width, s.bpp[i]);
        v.plane[i] = static_cast<const unsigned char*>(g->planes[i]);
        v.pitch[i] = g->pitch[i];
    }
    v.width = g->width;
    v.height = g->height;
    return HL_OK;
}

hl_status check_common(hl_ctx* ctx, const void* camera, const void* lights, uint32_t n_lights) {
    if (!ctx) return HL_ERR_INVALID_ARGUMENT;
    if (!camera) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "camera is NULL");
    if (!aligned(camera, 16)) return fail(ctx, HL_ERR_LAYOUT, "camera pointer not 16-byte aligned");
    if (n_lights > 0 && !lights) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "lights is NULL with n_lights=%u", n_lights);
    if (lights && !aligned(lights, 16)) return fail(ctx, HL_ERR_LAYOUT, "lights pointer not 16-byte aligned");
    if (n_lights > (1u << 23)) return fail(ctx, HL_ERR_SIZE, "n_lights %u exceeds 2^23", n_lights);
    return HL_OK;
}

hl_status check_grid(hl_ctx* ctx, const hl_light_grid* grid, uint32_t W, uint32_t H, hl::GridView& gv,
                     hl::SliceTable& tab) {
    if (!grid) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "light grid is NULL");
    std::memset(&gv, 0, sizeof gv);
    gv.lists = grid->lists;
    gv.counts = grid->counts;
    if (!grid->lists || !grid->counts) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "light grid lists/counts is NULL");
    if (grid->kind == HL_GRID_TILES) {
        gv.tiles = hl_tile_count(W, H);
        if (gv.tiles == 0) return fail(ctx, HL_ERR_SIZE, "tile grid of %ux%u overflows", W, H);
        gv.lists_capacity = grid->lists_capacity ? grid->lists_capacity : gv.tiles * hl::kMaxPerTile;
    } else if (grid->kind == HL_GRID_FROXELS) {
        hl_status s = check_froxel_params(ctx, &grid->froxel);
        if (s != HL_OK) return s;
        if (grid->froxel.width != W || grid->froxel.height != H)
            return fail(ctx, HL_ERR_INVALID_ARGUMENT, "froxel grid is for %ux%u, gbuffer is %ux%u", grid->froxel.width,
                        grid->froxel.height, W, H);
        gv.fp = grid->froxel;
        gv.lists_capacity = grid->lists_capacity ? grid->lists_capacity : 0xFFFFFFFFu;
        slice_table(grid->froxel, tab.z);
    } else {
        return fail(ctx, HL_ERR_INVALID_ARGUMENT, "unknown light grid kind %u", grid->kind);
    }
    return HL_OK;
}

hl_status check_target(hl_ctx* ctx, const hl_target* t, uint32_t W, hl::TargetView& tv) {
    if (!t || !t->data) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "radiance target is NULL");
    if (t->format > HL_TARGET_RGBA16F) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "unknown target format %u", t->format);
    const uint32_t bpp = t->format == HL_TARGET_RGBA32F ? 16 : 8;
    if (!aligned(t->data, bpp) || t->pitch % bpp != 0)
        return fail(ctx, HL_ERR_LAYOUT, "radiance target pointer/pitch not %u-byte aligned", bpp);
    if (t->pitch < uint64_t(W) * bpp) return fail(ctx, HL_ERR_LAYOUT, "radiance target pitch too small");
    tv.data = static_cast<unsigned char*>(t->data);
    tv.pitch = t->pitch;
    return HL_OK;
}

hl_status shade_common(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                       const void* lights, uint32_t n_lights, const hl_light_grid* grid, const hl_target* radiance,
                       uint32_t* stats, void* stream) {
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
    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    cudaError_t e = hl::launch_shade(gbuffer->layout, grid->kind, stats ? HL_TARGET_RGBA32F : radiance->format, camera,
                                     globals, gv, lights, n_lights, grv, tab, tv, stats, ctx->d_status,
                                     as_stream(stream));
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
    const uint32_t F = p->grid_x * p->grid_y * p->grid_z;
    DeviceGuard dg(ctx->device);
    if (!dg.ok) return fail(ctx, HL_ERR_CUDA, "cudaSetDevice(%d) failed", ctx->device);
    if ((s = ensure(ctx, ctx->bin_lights, ctx->bin_lights_cap, n > 0 ? n : 1, "bin light scratch")) != HL_OK) return s;
    if ((s = ensure(ctx, ctx->froxel_counts, ctx->froxel_counts_cap, F, "froxel count scratch")) != HL_OK) return s;
    hl::SliceTable tab;
    std::memset(&tab, 0, sizeof tab);
    slice_table(*p, tab.z);
    cudaStream_t st = as_stream(stream);
    cudaError_t e = hl::launch_prep_bin_lights(camera, lights, n, true, ctx->bin_lights, st);
    if (e == cudaSuccess)
        e = hl::launch_bin_froxels(camera, ctx->bin_lights, n, *p, tab, ctx->froxel_counts, out->offsets, out->indices,
                                   out->capacity, ctx->d_status, st);
    return e == cudaSuccess ? HL_OK : cuda_fail(ctx, e, "bin_froxels launch");
}

hl_status hl_shade(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer, const void* lights,
                   uint32_t n_lights, const hl_light_grid* grid, const hl_target* radiance, void* stream) {
    return shade_common(ctx, camera, globals, gbuffer, lights, n_lights, grid, radiance, nullptr, stream);
}

hl_status hl_shade_stats(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                         const void* lights, uint32_t n_lights, const hl_light_grid* grid, uint32_t* counts,
                         void* stream) {
    if (!counts) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "stats counts is NULL");
    return shade_common(ctx, camera, globals, gbuffer, lights, n_lights, grid, nullptr, counts, stream);
}

hl_status hl_shade_adjoint(hl_ctx* ctx, const void*, const void*, const hl_gbuffer*, const void*, uint32_t,
                           const hl_light_grid*, const float*, uint64_t, double*, float*, void*) {
    return fail(ctx, HL_ERR_NOT_SUPPORTED, "hl_shade_adjoint: not built yet");
}

hl_status hl_batch_plan_create(hl_ctx* ctx, const hl_view*, uint32_t, const void*, uint32_t, const void*,
                               const hl_batch_config*, hl_batch_plan** out, void*) {
    if (out) *out = nullptr;
    return fail(ctx, HL_ERR_NOT_SUPPORTED, "hl_batch_plan_create: not built yet");
}
hl_status hl_batch_execute(hl_ctx* ctx, hl_batch_plan*, void*) {
    return fail(ctx, HL_ERR_NOT_SUPPORTED, "hl_batch_execute: not built yet");
}
hl_status hl_batch_plan_view_grid(const hl_batch_plan*, uint32_t, uint32_t*) { return HL_ERR_NOT_SUPPORTED; }
hl_status hl_batch_plan_destroy(hl_batch_plan*) { return HL_OK; }

hl_status hl_probe_fp32_peak(hl_ctx* ctx, double* tflops) {
    if (!ctx || !tflops) return HL_ERR_INVALID_ARGUMENT;
    DeviceGuard dg(ctx->device);
    cudaError_t e = hl::run_fp32_probe(ctx->device, tflops);
    return e == cudaSuccess ? HL_OK : cuda_fail(ctx, e, "fp32 probe");
}

}  // extern "C"
