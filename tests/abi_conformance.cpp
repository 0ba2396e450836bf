// C-ABI conformance test of libhelio_gb300: what a host binding in another language
// (a Rust RenderPass shim, a cgo or JNI wrapper) relies on, exercised from plain C++
// through include/helio_gb300.h only.
//
//   abi_conformance cpu   entry points that need no GPU: version, status strings,
//                         tile counts, slice tables and their argument errors
//   abi_conformance gpu   a context on device 0: argument errors before any launch,
//                         the reference tile lists (cleared with no lights, a directional
//                         light in every tile), shading of a 32x32 FP32 G-buffer lit by
//                         one directional light against a closed form, sky pixels left
//                         untouched, froxel lists, the batch plan and the adjoint
// Prints one line per check and exits non-zero on the first failure.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "helio_gb300.h"

namespace {

int g_checks = 0;

void check(bool ok, const char* what) {
    ++g_checks;
    std::printf("%s %s\n", ok ? "ok  " : "FAIL", what);
    if (!ok) std::exit(1);
}

void check_cuda(cudaError_t e, const char* what) {
    if (e != cudaSuccess) {
        std::printf("FAIL %s: %s\n", what, cudaGetErrorString(e));
        std::exit(1);
    }
}

// ---- byte records (GpuCameraUniforms 368 B, GpuLight 128 B, DeferredGlobals 112 B) ----
struct Camera {
    float view[16], proj[16], view_proj[16], inv_view_proj[16];
    float position_near[4], forward_far[4], jitter_frame[4], prev_view_proj[16];
};
struct Light {
    float position_range[4], direction_outer[4], color_intensity[4];
    uint32_t shadow_index, light_type;
    float inner_angle;
    uint32_t pad;
    uint32_t god_rays_enabled;
    float god_rays[4];
    uint32_t flare_enabled, flare_type;
    float flare_intensity, flare_scale, flare_tint[3];
    int32_t ies_profile_index, light_function_index;
    float ies_angle_scale, ies_angle_offset;
};
struct Globals {
    uint32_t frame;
    float delta_time;
    uint32_t light_count;
    float ambient_intensity, ambient_color[4], rc_world_min[4], rc_world_max[4], csm_splits[4];
    uint32_t debug_mode, has_rc_gi, num_tiles_x, reflection_capture_count, enable_reflections,
        enable_env_reflections, pad[2];
};
static_assert(sizeof(Camera) == HL_SIZEOF_GPU_CAMERA, "camera record");
static_assert(sizeof(Light) == HL_SIZEOF_GPU_LIGHT, "light record");
static_assert(sizeof(Globals) == HL_SIZEOF_DEFERRED_GLOBALS, "globals record");
static_assert(sizeof(hl_reflection_inputs) == 64, "hl_reflection_inputs: 3 x (pointer, pitch) + rc, env pointers");
static_assert(sizeof(hl_reflection_env) == 32, "hl_reflection_env: captures, 4 sizes, texels");

// 4x4 inverse by Gauss-Jordan (column-major in and out).
void invert(const double* m, double* out) {
    double a[4][8];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            a[r][c] = m[c * 4 + r];
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; ++c) {
        int p = c;
        for (int r = c + 1; r < 4; ++r)
            if (std::fabs(a[r][c]) > std::fabs(a[p][c])) p = r;
        for (int k = 0; k < 8; ++k) std::swap(a[c][k], a[p][k]);
        const double d = a[c][c];
        for (int k = 0; k < 8; ++k) a[c][k] /= d;
        for (int r = 0; r < 4; ++r)
            if (r != c) {
                const double f = a[r][c];
                for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
            }
    }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) out[c * 4 + r] = a[r][c + 4];
}

// Eye at the origin looking down -Z; DirectX right-handed perspective, NDC z in [0, 1].
Camera make_camera(int W, int H, double fov_y_deg, double n, double f, double inv_vp[16]) {
    Camera c;
    std::memset(&c, 0, sizeof c);
    const double ys = 1.0 / std::tan(fov_y_deg * M_PI / 360.0), xs = ys * H / W;
    double P[16] = {0};
    P[0] = xs;
    P[5] = ys;
    P[10] = f / (n - f);
    P[11] = -1.0;
    P[14] = n * f / (n - f);
    invert(P, inv_vp);
    for (int i = 0; i < 16; ++i) {
        c.view[i] = (i % 5 == 0) ? 1.0f : 0.0f;
        c.proj[i] = float(P[i]);
        c.view_proj[i] = float(P[i]);
        c.inv_view_proj[i] = float(inv_vp[i]);
        c.prev_view_proj[i] = float(P[i]);
    }
    c.position_near[3] = float(n);
    c.forward_far[2] = -1.0f;
    c.forward_far[3] = float(f);
    return c;
}

Light directional(float dx, float dy, float dz, float intensity) {
    Light l;
    std::memset(&l, 0, sizeof l);
    l.direction_outer[0] = dx;
    l.direction_outer[1] = dy;
    l.direction_outer[2] = dz;
    l.color_intensity[0] = l.color_intensity[1] = l.color_intensity[2] = 1.0f;
    l.color_intensity[3] = intensity;
    l.shadow_index = 0xFFFFFFFFu;
    l.light_type = 0;
    l.ies_profile_index = -1;
    l.light_function_index = -1;
    return l;
}

void cpu_checks() {
    check(hl_abi_version() == HL_ABI_VERSION, "hl_abi_version matches the header");
    for (int s = 0; s >= -8; --s) check(hl_status_string(s) != nullptr, "hl_status_string is never NULL");
    check(hl_status_string(-1000) != nullptr, "hl_status_string of an unknown code");
    check(hl_tile_count(1920, 1080) == 120 * 68, "hl_tile_count 1080p = 8160 (ceil 16-px tiles)");
    check(hl_tile_count(0, 1080) == 0, "hl_tile_count of an empty viewport is 0");
    hl_froxel_params p{16, 9, 24, 1920, 1080, 0.5f, 100.0f, 0};
    std::vector<float> tab(25);
    check(hl_froxel_slice_table(&p, tab.data()) == HL_OK, "hl_froxel_slice_table ok");
    check(tab[0] == 0.0f && tab[24] == 100.0f && tab[1] > 0.5f && tab[12] < tab[13], "slice table shape");
    hl_froxel_params bad = p;
    bad.grid_z = 0;
    check(hl_froxel_slice_table(&bad, tab.data()) == HL_ERR_INVALID_ARGUMENT, "zero slices rejected");
    bad = p;
    bad.grid_z = 129;
    check(hl_froxel_slice_table(&bad, tab.data()) == HL_ERR_SIZE, "more than 128 slices rejected");
    check(hl_froxel_slice_table(nullptr, tab.data()) == HL_ERR_INVALID_ARGUMENT, "NULL params rejected");
    check(hl_create(nullptr, 0) == HL_ERR_INVALID_ARGUMENT, "hl_create(NULL) rejected");
    check(hl_destroy(nullptr) == HL_OK, "hl_destroy(NULL) is a no-op");
    // every pass entry point rejects a NULL context before touching a device
    check(hl_shade(nullptr, nullptr, nullptr, nullptr, nullptr, 0, nullptr, nullptr, nullptr) ==
              HL_ERR_INVALID_ARGUMENT,
          "hl_shade(NULL ctx) rejected");
    check(hl_shade_ex(nullptr, nullptr, nullptr, nullptr, nullptr, 0, nullptr, nullptr, nullptr, nullptr) ==
              HL_ERR_INVALID_ARGUMENT,
          "hl_shade_ex(NULL ctx) rejected");
    check(hl_shade_reflections(nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr) ==
              HL_ERR_INVALID_ARGUMENT,
          "hl_shade_reflections(NULL ctx) rejected");
    check(hl_write_gbuffer(nullptr, nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr, 0, nullptr, nullptr) ==
              HL_ERR_INVALID_ARGUMENT,
          "hl_write_gbuffer(NULL ctx) rejected");
}

void gpu_checks() {
    hl_ctx* ctx = nullptr;
    check(hl_create(&ctx, -1) == HL_ERR_INVALID_ARGUMENT && ctx == nullptr, "hl_create rejects device -1");
    check(hl_create(&ctx, 0) == HL_OK && ctx, "hl_create on device 0");
    const int W = 32, H = 32;
    const double n = 0.1, f = 100.0, depth_lin = 5.0;
    double inv_vp[16];
    const Camera cam = make_camera(W, H, 60.0, n, f, inv_vp);
    const Light sun = directional(0.0f, 0.0f, -1.0f, 2.0f);  // shines along -Z: L = +Z
    Globals glb;
    std::memset(&glb, 0, sizeof glb);
    glb.light_count = 1;
    glb.num_tiles_x = (W + 15) / 16;

    void *d_cam, *d_light, *d_glb;
    check_cuda(cudaMalloc(&d_cam, sizeof cam), "cudaMalloc camera");
    check_cuda(cudaMalloc(&d_light, sizeof sun), "cudaMalloc light");
    check_cuda(cudaMalloc(&d_glb, sizeof glb), "cudaMalloc globals");
    check_cuda(cudaMemcpy(d_cam, &cam, sizeof cam, cudaMemcpyHostToDevice), "copy camera");
    check_cuda(cudaMemcpy(d_light, &sun, sizeof sun, cudaMemcpyHostToDevice), "copy light");
    check_cuda(cudaMemcpy(d_glb, &glb, sizeof glb, cudaMemcpyHostToDevice), "copy globals");

    // ---- argument errors come back before any launch ----
    const uint32_t tiles = hl_tile_count(W, H);
    uint32_t *d_lists, *d_counts;
    check_cuda(cudaMalloc(&d_lists, tiles * 64 * 4), "cudaMalloc lists");
    check_cuda(cudaMalloc(&d_counts, tiles * 4), "cudaMalloc counts");
    check(hl_bin_tiles_ref(ctx, nullptr, d_light, 1, W, H, d_lists, d_counts, nullptr) == HL_ERR_INVALID_ARGUMENT,
          "hl_bin_tiles_ref rejects a NULL camera");
    check(hl_bin_tiles_ref(ctx, static_cast<char*>(d_cam) + 4, d_light, 1, W, H, d_lists, d_counts, nullptr) ==
              HL_ERR_LAYOUT,
          "hl_bin_tiles_ref rejects a misaligned camera");
    check(std::strlen(hl_last_error_message(ctx)) > 0, "hl_last_error_message explains the error");

    // ---- reference tile lists ----
    check_cuda(cudaMemset(d_counts, 0xFF, tiles * 4), "poison counts");
    check(hl_bin_tiles_ref(ctx, d_cam, d_light, 0, W, H, d_lists, d_counts, nullptr) == HL_OK, "bin 0 lights");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "sync after bin 0 lights");
    std::vector<uint32_t> counts(tiles), lists(tiles * 64);
    check_cuda(cudaMemcpy(counts.data(), d_counts, tiles * 4, cudaMemcpyDeviceToHost), "read counts");
    bool zero = true;
    for (uint32_t c : counts) zero = zero && c == 0;
    check(zero, "no lights: every tile count cleared to 0");
    check(hl_bin_tiles_ref(ctx, d_cam, d_light, 1, W, H, d_lists, d_counts, nullptr) == HL_OK, "bin 1 light");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "sync after bin 1 light");
    check_cuda(cudaMemcpy(counts.data(), d_counts, tiles * 4, cudaMemcpyDeviceToHost), "read counts");
    check_cuda(cudaMemcpy(lists.data(), d_lists, tiles * 64 * 4, cudaMemcpyDeviceToHost), "read lists");
    bool all = true;
    for (uint32_t t = 0; t < tiles; ++t) all = all && counts[t] == 1 && lists[t * 64] == 0;
    check(all, "a directional light is listed in every tile");

    // ---- FP32 G-buffer: albedo 0.5 grey, roughness 0.5, normal +Z, depth 5 (sky at x = 0) ----
    const float z_ndc = float((f / (f - n)) * (1.0 - n / depth_lin));
    std::vector<float> p0(W * H * 4), p1(W * H * 4), p2(W * H);
    for (int i = 0; i < W * H; ++i) {
        p0[4 * i + 0] = p0[4 * i + 1] = p0[4 * i + 2] = 0.5f;
        p0[4 * i + 3] = 0.5f;
        p1[4 * i + 0] = 0.0f;
        p1[4 * i + 1] = 0.0f;
        p1[4 * i + 2] = 1.0f;
        p1[4 * i + 3] = 0.0f;
        p2[i] = (i % W == 0) ? 1.0f : z_ndc;
    }
    void *g0, *g1, *g2, *d_out;
    check_cuda(cudaMalloc(&g0, p0.size() * 4), "cudaMalloc plane 0");
    check_cuda(cudaMalloc(&g1, p1.size() * 4), "cudaMalloc plane 1");
    check_cuda(cudaMalloc(&g2, p2.size() * 4), "cudaMalloc plane 2");
    check_cuda(cudaMalloc(&d_out, W * H * 16), "cudaMalloc radiance");
    check_cuda(cudaMemcpy(g0, p0.data(), p0.size() * 4, cudaMemcpyHostToDevice), "copy plane 0");
    check_cuda(cudaMemcpy(g1, p1.data(), p1.size() * 4, cudaMemcpyHostToDevice), "copy plane 1");
    check_cuda(cudaMemcpy(g2, p2.data(), p2.size() * 4, cudaMemcpyHostToDevice), "copy plane 2");
    std::vector<float> sentinel(W * H * 4, -7.0f);
    check_cuda(cudaMemcpy(d_out, sentinel.data(), W * H * 16, cudaMemcpyHostToDevice), "poison radiance");
    hl_gbuffer gb;
    std::memset(&gb, 0, sizeof gb);
    gb.layout = HL_GBUF_F32;
    gb.width = W;
    gb.height = H;
    gb.planes[0] = g0;
    gb.planes[1] = g1;
    gb.planes[2] = g2;
    gb.pitch[0] = W * 16;
    gb.pitch[1] = W * 16;
    gb.pitch[2] = W * 4;
    hl_light_grid grid;
    std::memset(&grid, 0, sizeof grid);
    grid.kind = HL_GRID_TILES;
    grid.lists = d_lists;
    grid.counts = d_counts;
    hl_target tgt{d_out, uint64_t(W) * 16, HL_TARGET_RGBA32F, 0};
    hl_gbuffer bad = gb;
    bad.pitch[0] = W * 16 - 16;
    check(hl_shade(ctx, d_cam, d_glb, &bad, d_light, 1, &grid, &tgt, nullptr) == HL_ERR_LAYOUT,
          "hl_shade rejects a pitch shorter than a row");
    check(hl_shade(ctx, d_cam, d_glb, &gb, d_light, 1, &grid, &tgt, nullptr) == HL_OK, "hl_shade");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "sync after hl_shade");
    // the reflection draw with every input at its fallback adds nothing (checked below)
    hl_reflection_inputs refl;
    std::memset(&refl, 0, sizeof refl);
    check(hl_shade_reflections(ctx, d_cam, d_glb, &gb, &refl, &tgt, nullptr) == HL_OK, "hl_shade_reflections");
    check(hl_shade_reflections(ctx, d_cam, d_glb, &gb, nullptr, &tgt, nullptr) == HL_OK,
          "hl_shade_reflections without inputs");
    refl.ssr = static_cast<const char*>(d_out) + 2;
    refl.ssr_pitch = W * 8;
    check(hl_shade_reflections(ctx, d_cam, d_glb, &gb, &refl, &tgt, nullptr) == HL_ERR_LAYOUT,
          "hl_shade_reflections rejects a misaligned SSR image");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "sync after hl_shade_reflections");
    std::vector<float> out(W * H * 4);
    check_cuda(cudaMemcpy(out.data(), d_out, W * H * 16, cudaMemcpyDeviceToHost), "read radiance");
    bool sky_ok = true;
    for (int y = 0; y < H; ++y) sky_ok = sky_ok && out[(y * W) * 4] == -7.0f;
    check(sky_ok, "sky pixels (depth 1) are left untouched");
    // closed form at pixel (17, 9): pbr_direct_light of a directional light, N = L = +Z
    const int px = 17, py = 9;
    const double ndx = (px + 0.5) / W * 2 - 1, ndy = 1 - (py + 0.5) / H * 2;
    double hw[4];
    for (int r = 0; r < 4; ++r)
        hw[r] = inv_vp[r] * ndx + inv_vp[4 + r] * ndy + inv_vp[8 + r] * double(z_ndc) + inv_vp[12 + r];
    double V[3] = {-hw[0] / hw[3], -hw[1] / hw[3], -hw[2] / hw[3]};
    const double vl = std::sqrt(V[0] * V[0] + V[1] * V[1] + V[2] * V[2]);
    for (double& v : V) v /= vl;
    const double pi = 3.14159265359, rough = 0.5, NdL = 1.0, NdV = V[2];
    double Hv[3] = {V[0], V[1], V[2] + 1.0};
    const double hl = std::sqrt(Hv[0] * Hv[0] + Hv[1] * Hv[1] + Hv[2] * Hv[2]);
    const double NdH = Hv[2] / hl, HdV = (Hv[0] * V[0] + Hv[1] * V[1] + Hv[2] * V[2]) / hl;
    const double F = 0.04 + 0.96 * std::pow(1.0 - HdV, 5.0);
    const double a2 = std::pow(rough, 4.0), den = NdH * NdH * (a2 - 1) + 1, D = a2 / (pi * den * den + 1e-4);
    const double k = (rough + 1) * (rough + 1) / 8;
    const double G = NdV / (NdV * (1 - k) + k + 1e-4) * NdL / (NdL * (1 - k) + k + 1e-4);
    const double spec = D * G * F / (4 * NdV * NdL + 1e-4);
    const double want = ((1 - F) * 0.5 / pi + spec) * 2.0 * NdL;
    const float got = out[(py * W + px) * 4];
    check(std::fabs(got - want) <= 1e-5 * want, "radiance of one pixel = closed form within 1e-5");
    check(out[(py * W + px) * 4 + 3] == 1.0f, "alpha is 1");

    // ---- froxel lists ----
    hl_froxel_params fp{4, 4, 8, W, H, 0.5f, float(f), 0};
    uint32_t *d_off, *d_idx;
    check_cuda(cudaMalloc(&d_off, (4 * 4 * 8 + 1) * 4), "cudaMalloc offsets");
    check_cuda(cudaMalloc(&d_idx, 4 * 4 * 8 * 4), "cudaMalloc indices");
    hl_froxel_lists fl{d_off, d_idx, 4 * 4 * 8, 0};
    check(hl_bin_froxels(ctx, d_cam, d_light, 1, &fp, &fl, nullptr) == HL_OK, "hl_bin_froxels");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "sync after hl_bin_froxels");
    std::vector<uint32_t> off(4 * 4 * 8 + 1);
    check_cuda(cudaMemcpy(off.data(), d_off, off.size() * 4, cudaMemcpyDeviceToHost), "read offsets");
    check(off[0] == 0 && off.back() == 4 * 4 * 8, "a directional light is listed in every froxel");
    hl_froxel_lists small{d_off, d_idx, 10, 0};
    check(hl_bin_froxels(ctx, d_cam, d_light, 1, &fp, &small, nullptr) == HL_OK, "hl_bin_froxels, small capacity");
    check(hl_sync_status(ctx, nullptr) == HL_ERR_CAPACITY, "capacity overflow reported by hl_sync_status");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "the status word is cleared after it is reported");

    // ---- froxel-grid shading equals tile-grid shading (one directional light) ----
    hl_light_grid fg;
    std::memset(&fg, 0, sizeof fg);
    fg.kind = HL_GRID_FROXELS;
    fg.lists = d_idx;
    fg.counts = d_off;
    fg.lists_capacity = 4 * 4 * 8;
    fg.froxel = fp;
    check(hl_bin_froxels(ctx, d_cam, d_light, 1, &fp, &fl, nullptr) == HL_OK, "rebin froxels");
    void* d_out2;
    check_cuda(cudaMalloc(&d_out2, W * H * 16), "cudaMalloc radiance 2");
    hl_target tgt2{d_out2, uint64_t(W) * 16, HL_TARGET_RGBA32F, 0};
    check(hl_shade(ctx, d_cam, d_glb, &gb, d_light, 1, &fg, &tgt2, nullptr) == HL_OK, "hl_shade, froxel grid");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "sync after froxel shading");
    std::vector<float> out2(W * H * 4);
    check_cuda(cudaMemcpy(out2.data(), d_out2, W * H * 16, cudaMemcpyDeviceToHost), "read radiance 2");
    bool same = true;
    for (int i = 0; i < W * H; ++i)
        if (i % W != 0) same = same && std::memcmp(&out[4 * i], &out2[4 * i], 16) == 0;
    check(same, "froxel and tile grids give identical radiance");

    // ---- adjoint: d/d intensity of sum(radiance.rgb) = sum(radiance.rgb) / intensity ----
    std::vector<float> ones(W * H * 4, 1.0f);
    void *d_w, *d_dl, *d_dp;
    check_cuda(cudaMalloc(&d_w, W * H * 16), "cudaMalloc weights");
    check_cuda(cudaMalloc(&d_dl, 7 * 8), "cudaMalloc d_lights");
    check_cuda(cudaMalloc(&d_dp, W * H * 5 * 4), "cudaMalloc d_pixels");
    check_cuda(cudaMemcpy(d_w, ones.data(), W * H * 16, cudaMemcpyHostToDevice), "copy weights");
    check(hl_shade_adjoint(ctx, d_cam, d_glb, &gb, d_light, 1, &fg, static_cast<const float*>(d_w), W * 16,
                           static_cast<double*>(d_dl), static_cast<float*>(d_dp), nullptr) == HL_OK,
          "hl_shade_adjoint");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "sync after hl_shade_adjoint");
    double dl[7];
    check_cuda(cudaMemcpy(dl, d_dl, sizeof dl, cudaMemcpyDeviceToHost), "read d_lights");
    double sum = 0;
    for (int i = 0; i < W * H; ++i)
        if (i % W != 0) sum += double(out[4 * i]) + out[4 * i + 1] + out[4 * i + 2];
    check(std::fabs(dl[3] - sum / 2.0) <= 1e-4 * sum, "adjoint intensity gradient = radiance / intensity");
    check(dl[0] == 0.0 && dl[1] == 0.0 && dl[2] == 0.0, "a directional light has no position gradient");

    // ---- batch plan of two views = the single-view result ----
    hl_view views[2];
    void* d_out3;
    check_cuda(cudaMalloc(&d_out3, W * H * 16), "cudaMalloc radiance 3");
    views[0] = hl_view{d_cam, gb, tgt2};
    views[1] = hl_view{d_cam, gb, hl_target{d_out3, uint64_t(W) * 16, HL_TARGET_RGBA32F, 0}};
    hl_batch_config cfg{0, 4, 4, 8, nullptr};
    hl_batch_plan* plan = nullptr;
    check(hl_batch_plan_create(ctx, views, 2, d_light, 1, d_glb, &cfg, &plan, nullptr) == HL_OK && plan,
          "hl_batch_plan_create");
    check(hl_batch_execute(ctx, plan, nullptr) == HL_OK, "hl_batch_execute");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "sync after the batch");
    uint32_t g3[3];
    check(hl_batch_plan_view_grid(plan, 1, g3) == HL_OK && g3[0] == 4 && g3[1] == 4 && g3[2] == 8, "plan view grid");
    check(hl_batch_plan_view_grid(plan, 2, g3) == HL_ERR_INVALID_ARGUMENT, "plan view index checked");
    std::vector<float> out3(W * H * 4);
    check_cuda(cudaMemcpy(out3.data(), d_out3, W * H * 16, cudaMemcpyDeviceToHost), "read radiance 3");
    same = true;
    for (int i = 0; i < W * H; ++i)
        if (i % W != 0) same = same && std::memcmp(&out[4 * i], &out3[4 * i], 16) == 0;
    check(same, "batched view = single-view radiance");
    check(hl_batch_plan_destroy(plan) == HL_OK, "hl_batch_plan_destroy");

    // ---- G-buffer write: one untextured metallic material over a 32x32 target ----
    // GpuMaterial (96 B): base_color, emissive, roughness_metallic, 5 texture ids, workflow,
    // flags, class; GpuMaterialTextures (352 B): 7 slots of 48 B (texture_index first),
    // then params (normal_scale, occlusion_strength, alpha_cutoff, -).
    unsigned char mat[96] = {}, mtex[352] = {}, gglb[HL_SIZEOF_GBUFFER_GLOBALS] = {};
    const float mf[12] = {0.6f, 0.4f, 0.2f, 1.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.5f, 1.0f, 1.5f, 0.5f};
    std::memcpy(mat, mf, sizeof mf);
    const uint32_t no_tex = HL_NO_TEXTURE;
    for (int s = 0; s < 7; ++s) std::memcpy(mtex + 48 * s, &no_tex, 4);
    const float prm[4] = {1.0f, 1.0f, 0.5f, 0.0f};
    std::memcpy(mtex + 336, prm, sizeof prm);
    std::vector<hl_surface> srf(W * H);
    for (auto& s : srf) {
        s = hl_surface{{0.0f, 0.0f, 3.0f}, 1.0f, {1.0f, 0.0f, 0.0f}, 0u, {0.5f, 0.5f}, {-1.0f, -1.0f},
                       {0.0f, 0.0f, 0.5f, 1.0f}};
    }
    srf[5].material_id = HL_NO_FRAGMENT;
    void *d_mat, *d_mtex, *d_gglb, *d_srf, *d_t[4];
    check_cuda(cudaMalloc(&d_mat, sizeof mat), "cudaMalloc material");
    check_cuda(cudaMalloc(&d_mtex, sizeof mtex), "cudaMalloc material textures");
    check_cuda(cudaMalloc(&d_gglb, sizeof gglb), "cudaMalloc G-buffer globals");
    check_cuda(cudaMalloc(&d_srf, W * H * sizeof(hl_surface)), "cudaMalloc surfaces");
    check_cuda(cudaMemcpy(d_mat, mat, sizeof mat, cudaMemcpyHostToDevice), "copy material");
    check_cuda(cudaMemcpy(d_mtex, mtex, sizeof mtex, cudaMemcpyHostToDevice), "copy material textures");
    check_cuda(cudaMemcpy(d_gglb, gglb, sizeof gglb, cudaMemcpyHostToDevice), "copy G-buffer globals");
    check_cuda(cudaMemcpy(d_srf, srf.data(), W * H * sizeof(hl_surface), cudaMemcpyHostToDevice), "copy surfaces");
    const uint32_t bpp[4] = {4, 8, 4, 8};
    hl_gbuffer_targets tg;
    std::memset(&tg, 0, sizeof tg);
    tg.width = W;
    tg.height = H;
    for (int i = 0; i < 4; ++i) {
        check_cuda(cudaMalloc(&d_t[i], W * H * bpp[i]), "cudaMalloc G-buffer target");
        check_cuda(cudaMemset(d_t[i], 0xAB, W * H * bpp[i]), "fill G-buffer target");
        tg.planes[i] = d_t[i];
        tg.pitch[i] = uint64_t(W) * bpp[i];
    }
    hl_gbuffer_targets bad_tg = tg;
    bad_tg.planes[1] = nullptr;
    check(hl_write_gbuffer(ctx, d_gglb, static_cast<const hl_surface*>(d_srf), W * sizeof(hl_surface), d_mat,
                           d_mtex, 1, nullptr, 0, &bad_tg, nullptr) == HL_ERR_INVALID_ARGUMENT,
          "hl_write_gbuffer rejects a missing normal target");
    check(hl_write_gbuffer(ctx, d_gglb, static_cast<const hl_surface*>(d_srf), W * sizeof(hl_surface), d_mat,
                           d_mtex, 1, nullptr, 0, &tg, nullptr) == HL_OK,
          "hl_write_gbuffer");
    check(hl_sync_status(ctx, nullptr) == HL_OK, "sync after hl_write_gbuffer");
    std::vector<uint32_t> alb(W * H);
    check_cuda(cudaMemcpy(alb.data(), d_t[0], W * H * 4, cudaMemcpyDeviceToHost), "read albedo");
    // round(255 * (0.6, 0.4, 0.2, 1.0)) = (153, 102, 51, 255)
    check(alb[0] == (153u | 102u << 8 | 51u << 16 | 255u << 24), "albedo = RGBA8 of the base colour");
    check(alb[5] == 0xABABABABu, "an uncovered pixel is left untouched");
    std::vector<uint16_t> nrm(W * H * 4);
    check_cuda(cudaMemcpy(nrm.data(), d_t[1], W * H * 8, cudaMemcpyDeviceToHost), "read normal");
    // normal (0, 0, 1) in f16 and F0.r = 0.6 (metallic 1): 0x0000 0x0000 0x3C00, 0x38CD
    check(nrm[0] == 0 && nrm[1] == 0 && nrm[2] == 0x3C00 && nrm[3] == 0x38CD,
          "normal = normalize(world_normal), F0.r = albedo at metallic 1");

    for (void* p : {d_cam, d_light, d_glb, static_cast<void*>(d_lists), static_cast<void*>(d_counts), g0, g1, g2,
                    d_out, static_cast<void*>(d_off), static_cast<void*>(d_idx), d_out2, d_w, d_dl, d_dp, d_out3,
                    d_mat, d_mtex, d_gglb, d_srf, d_t[0], d_t[1], d_t[2], d_t[3]})
        cudaFree(p);
    check(hl_destroy(ctx) == HL_OK, "hl_destroy");
}

}  // namespace

int main(int argc, char** argv) {
    const bool gpu = argc > 1 && std::strcmp(argv[1], "gpu") == 0;
    cpu_checks();
    if (gpu) gpu_checks();
    std::printf("%d checks passed\n", g_checks);
    return 0;
}
