// hl_common.cuh — device-side layouts, status flags and arithmetic helpers shared by
// the sm_103a kernels of the deferred-lighting engine.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include "../../include/helio_gb300.h"

namespace hl {

// ----------------------------------------------------------------------------------
// Reference byte layouts (libhelio/src/light.rs:60-115, libhelio/src/camera.rs:12-29,
// helio-pass-deferred-light/src/lib.rs:17-52, helio-pass-light-cull/src/lib.rs:26-35,
// libhelio/src/material.rs:231-254)
// ----------------------------------------------------------------------------------
struct alignas(16) GpuLight {
    float position_range[4];   // xyz position, w range
    float direction_outer[4];  // xyz direction, w cos(outer)
    float color_intensity[4];  // xyz colour, w intensity
    uint32_t shadow_index;
    uint32_t light_type;       // 0 directional, 1 point, 2 spot, 3 area
    float inner_angle;         // cos(inner)
    uint32_t pad0;
    uint32_t god_rays_enabled;
    float god_rays_density, god_rays_weight, god_rays_decay, god_rays_exposure;
    uint32_t flare_enabled, flare_type;
    float flare_intensity, flare_scale, flare_tint[3];
    int32_t ies_profile_index, light_function_index;
    float ies_angle_scale, ies_angle_offset;
};
static_assert(sizeof(GpuLight) == 128, "GpuLight must be 128 bytes (light.rs:111)");
static_assert(offsetof(GpuLight, shadow_index) == 48, "GpuLight.shadow_index offset");
static_assert(offsetof(GpuLight, light_type) == 52, "GpuLight.light_type offset");
static_assert(offsetof(GpuLight, inner_angle) == 56, "GpuLight.inner_angle offset");
static_assert(offsetof(GpuLight, god_rays_enabled) == 64, "GpuLight.god_rays offset");
static_assert(offsetof(GpuLight, flare_enabled) == 84, "GpuLight.flare offset");
static_assert(offsetof(GpuLight, ies_profile_index) == 112, "GpuLight.ies offset");
static_assert(offsetof(GpuLight, ies_angle_offset) == 124, "GpuLight tail offset");

struct alignas(16) GpuCamera {
    float view[16], proj[16], view_proj[16], inv_view_proj[16];
    float position_near[4], forward_far[4], jitter_frame[4], prev_view_proj[16];
};
static_assert(sizeof(GpuCamera) == 368, "GpuCameraUniforms must be 368 bytes");
static_assert(offsetof(GpuCamera, proj) == 64, "camera.proj offset");
static_assert(offsetof(GpuCamera, inv_view_proj) == 192, "camera.inv_view_proj offset");
static_assert(offsetof(GpuCamera, position_near) == 256, "camera.position_near offset");
static_assert(offsetof(GpuCamera, prev_view_proj) == 304, "camera.prev_view_proj offset");

struct alignas(16) DeferredGlobals {
    uint32_t frame;
    float delta_time;
    uint32_t light_count;
    float ambient_intensity;
    float ambient_color[4];
    float rc_world_min[4], rc_world_max[4], csm_splits[4];
    uint32_t debug_mode, has_rc_gi, num_tiles_x, reflection_capture_count;
    uint32_t enable_reflections, enable_env_reflections, pad[2];
};
static_assert(sizeof(DeferredGlobals) == 112, "DeferredGlobals must be 112 bytes");
static_assert(offsetof(DeferredGlobals, debug_mode) == 80, "globals.debug_mode offset");
static_assert(offsetof(DeferredGlobals, num_tiles_x) == 88, "globals.num_tiles_x offset");

struct LightCullParams {
    uint32_t num_tiles_x, num_tiles_y, num_lights, screen_width, screen_height, pad[3];
};
static_assert(sizeof(LightCullParams) == 32, "LightCullParams must be 32 bytes");

struct alignas(16) GpuMaterial {
    float base_color[4], emissive[4], roughness_metallic[4];
    uint32_t tex_base_color, tex_normal, tex_roughness, tex_emissive, tex_occlusion;
    uint32_t workflow, flags, material_class;
    float class_params[4];
};
static_assert(sizeof(GpuMaterial) == 96, "GpuMaterial must be 96 bytes");

static_assert(sizeof(hl_froxel_params) == 32, "hl_froxel_params must be 32 bytes");

constexpr uint32_t kTile = HL_TILE_SIZE;
constexpr uint32_t kMaxPerTile = HL_MAX_LIGHTS_PER_TILE;

// ----------------------------------------------------------------------------------
// Device status word (one per context): the first error code wins.
// ----------------------------------------------------------------------------------
__device__ __forceinline__ void raise_status(int* status, int code) {
    if (status) atomicCAS(status, 0, code);
}

// ----------------------------------------------------------------------------------
// Programmatic dependent launch. A kernel launched with launch_pdl may have its CTAs
// start while the previous kernel of the stream still runs, once that kernel has called
// pdl_launch_dependents; pdl_wait then blocks until the previous kernel has completed
// and its writes are visible. For a kernel launched without the attribute both are
// no-ops. A kernel reads nothing its predecessor writes before its pdl_wait.
// ----------------------------------------------------------------------------------
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_pdl(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t stream,
                              Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kern, static_cast<KArgs>(args)...);
}

// ----------------------------------------------------------------------------------
// Correctly rounded f32 operations: with these the binning kernels reproduce the
// declared operation order bit for bit (no FMA contraction, IEEE division and sqrt).
// ----------------------------------------------------------------------------------
__device__ __forceinline__ float xadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float xsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float xmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float xdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ float xsqrt(float a) { return __fsqrt_rn(a); }
__device__ __forceinline__ float xmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float xmax(float a, float b) { return a < b ? b : a; }

struct f3 {
    float x, y, z;
};
__device__ __forceinline__ f3 mk3(float x, float y, float z) { return f3{x, y, z}; }
// dot(a,b) = (a.x*b.x + a.y*b.y) + a.z*b.z
__device__ __forceinline__ float xdot(f3 a, f3 b) {
    return xadd(xadd(xmul(a.x, b.x), xmul(a.y, b.y)), xmul(a.z, b.z));
}
__device__ __forceinline__ f3 xcross(f3 a, f3 b) {
    return mk3(xsub(xmul(a.y, b.z), xmul(a.z, b.y)), xsub(xmul(a.z, b.x), xmul(a.x, b.z)),
               xsub(xmul(a.x, b.y), xmul(a.y, b.x)));
}
__device__ __forceinline__ f3 xnormalize(f3 v) {
    float len = xsqrt(xdot(v, v));
    return mk3(xdiv(v.x, len), xdiv(v.y, len), xdiv(v.z, len));
}
// Column-major M * (x,y,z,w), row r = ((M[0][r]*x + M[1][r]*y) + M[2][r]*z) + M[3][r]*w
__device__ __forceinline__ float xmat_row(const float* m, int r, float x, float y, float z, float w) {
    return xadd(xadd(xadd(xmul(m[r], x), xmul(m[4 + r], y)), xmul(m[8 + r], z)), xmul(m[12 + r], w));
}

// ----------------------------------------------------------------------------------
// Prepared light record used by the binning kernels (view space).
// ----------------------------------------------------------------------------------
struct alignas(16) BinLight {
    float cx, cy, cz;  // view-space centre
    float r;           // range (tile mode) or margin radius (froxel mode)
    float ax, ay, az;  // view-space unit axis (spots)
    float cos_o;       // cos(outer)
    float sin_o;
    uint32_t type;
    uint32_t cone;     // cone test applies
    uint32_t pad;
};
static_assert(sizeof(BinLight) == 48, "BinLight is 48 bytes");

// ----------------------------------------------------------------------------------
// Kernel launch helpers (defined in the .cu files)
// ----------------------------------------------------------------------------------
struct SliceTable {
    float z[129];  // up to 128 slices
};
constexpr uint32_t kMaxSlices = 128;

// Device-side state of the single-pass froxel binning (zeroed when allocated).
struct BinChainState {
    unsigned long long ticket;  // column tickets handed out, over all launches
    unsigned long long base;    // tickets handed out before the current launch
    uint32_t epoch;             // epoch of the last finished launch
    uint32_t done;              // CTAs of the current launch that have finished
};

// One view of a batch, as the batched froxel binning kernels read it.
struct BinViewDesc {
    const void* camera;         // GpuCameraUniforms
    BinLight* bl;               // n_lights records in this view's space
    uint32_t* counts;           // F per-froxel counts
    uint32_t* offsets;          // F + 1
    uint32_t* indices;          // capacity entries
    hl_froxel_params p;
    uint32_t capacity;
    uint32_t col_start;         // first column of this view in the batch's column range
    uint32_t groups;            // slice groups per column of the persistent launch's binning items
    uint32_t item_start;        // first binning item of this view in the persistent launch
    SliceTable tab;
};

}  // namespace hl
