// hl_host.h — host-side pieces shared by the C-ABI translation units: the context,
// error reporting, scratch growth and the argument validation of G-buffers, grids and
// targets. Host code only; not part of the public interface.
#pragma once

#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>

#include "hl_common.cuh"
#include "hl_internal.h"

struct hl_ctx {
    int device = 0;
    int* d_status = nullptr;          // device status word (first error wins)
    hl::BinLight* bin_lights = nullptr;
    uint32_t bin_lights_cap = 0;
    uint32_t* froxel_counts = nullptr;
    uint32_t froxel_counts_cap = 0;
    unsigned long long* froxel_chain = nullptr;  // per-item words of the single-launch binning
    uint32_t froxel_chain_cap = 0;
    uint32_t stall_item = ~0u, stall_spins = 0;  // one-shot failure injection (hl_inject_binning_stall)
    hl::BinChainState* bin_state = nullptr;      // ticket counter and epoch of the single-pass binning
    float4* shade_cand = nullptr;       // candidate-test light table of hl_shade
    uint32_t shade_cand_cap = 0;
    unsigned char* frag_lights = nullptr;  // light records of hl_shade_fragments
    uint32_t frag_lights_cap = 0;
    float* adjoint_partials = nullptr;  // per-CTA light-gradient partials of hl_shade_adjoint
    uint32_t adjoint_partials_cap = 0;
    hl::PairLog pair_log{nullptr, nullptr, 0};  // lit-pair record of the shading launches (hl_set_pair_log)
    std::string last_error;
};

namespace hl_host {



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

inline hl_status fail(hl_ctx* ctx, hl_status code, const char* fmt, ...) {
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

inline hl_status cuda_fail(hl_ctx* ctx, cudaError_t e, const char* where) {
    return fail(ctx, HL_ERR_CUDA, "%s: %s (%s)", where, cudaGetErrorName(e), cudaGetErrorString(e));
}

inline bool aligned(const void* p, size_t a) { return (reinterpret_cast<uintptr_t>(p) % a) == 0; }

inline cudaStream_t as_stream(void* s) { return static_cast<cudaStream_t>(s); }

// Grows a device scratch buffer; waits for the device before freeing the old one.
template <class T>
inline hl_status ensure(hl_ctx* ctx, T*& buf, uint32_t& cap, size_t need, const char* what) {
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

inline hl_status check_froxel_params(hl_ctx* ctx, const hl_froxel_params* p) {
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

inline void slice_table(const hl_froxel_params& p, float* out) {
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
inline constexpr PlaneSpec kPlaneSpecs[3] = {
    {5, {4, 8, 4, 8, 4, 0}, {4, 8, 4, 8, 4, 1}},  // reference
    {3, {16, 16, 4, 0, 0, 0}, {16, 16, 4, 1, 1, 1}},  // F32
    {4, {8, 4, 2, 4, 0, 0}, {8, 4, 2, 4, 1, 1}},  // F16
};

inline hl_status check_gbuffer(hl_ctx* ctx, const hl_gbuffer* g, hl::GBufView& v) {
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

inline hl_status check_common(hl_ctx* ctx, const void* camera, const void* lights, uint32_t n_lights) {
    if (!ctx) return HL_ERR_INVALID_ARGUMENT;
    if (!camera) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "camera is NULL");
    if (!aligned(camera, 16)) return fail(ctx, HL_ERR_LAYOUT, "camera pointer not 16-byte aligned");
    if (n_lights > 0 && !lights) return fail(ctx, HL_ERR_INVALID_ARGUMENT, "lights is NULL with n_lights=%u", n_lights);
    if (lights && !aligned(lights, 16)) return fail(ctx, HL_ERR_LAYOUT, "lights pointer not 16-byte aligned");
    if (n_lights > (1u << 23)) return fail(ctx, HL_ERR_SIZE, "n_lights %u exceeds 2^23", n_lights);
    return HL_OK;
}

inline hl_status check_grid(hl_ctx* ctx, const hl_light_grid* grid, uint32_t W, uint32_t H, hl::GridView& gv,
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

inline hl_status check_target(hl_ctx* ctx, const hl_target* t, uint32_t W, hl::TargetView& tv) {
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

}  // namespace hl_host
