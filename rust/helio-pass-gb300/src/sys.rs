//! Raw bindings of `include/helio_gb300.h` (the helio_gb300 C ABI): every entry point
//! and every struct, field for field. Pointers marked "device" are CUDA device
//! addresses; `stream` is a `cudaStream_t` (null: the legacy default stream).
#![allow(non_camel_case_types)]

use core::ffi::{c_char, c_int, c_void};

pub type hl_status = i32;
pub const HL_OK: hl_status = 0;
pub const HL_ERR_INVALID_ARGUMENT: hl_status = -1;
pub const HL_ERR_LAYOUT: hl_status = -2;
pub const HL_ERR_SIZE: hl_status = -3;
pub const HL_ERR_CUDA: hl_status = -4;
pub const HL_ERR_TIMEOUT: hl_status = -5;
pub const HL_ERR_CAPACITY: hl_status = -6;
pub const HL_ERR_DEVICE_BOUNDS: hl_status = -7;
pub const HL_ERR_NOT_SUPPORTED: hl_status = -8;

pub const HL_ABI_VERSION: u32 = 1;
pub const HL_TILE_SIZE: u32 = 16;
pub const HL_MAX_LIGHTS_PER_TILE: u32 = 64;
pub const HL_FROXEL_NEAR: f32 = 0.5;
pub const HL_GBUF_REFERENCE: u32 = 0;
pub const HL_GBUF_F32: u32 = 1;
pub const HL_GBUF_F16: u32 = 2;
pub const HL_GBUF_MAX_PLANES: usize = 6;
pub const HL_GRID_TILES: u32 = 0;
pub const HL_GRID_FROXELS: u32 = 1;
pub const HL_TARGET_RGBA32F: u32 = 0;
pub const HL_TARGET_RGBA16F: u32 = 1;
pub const HL_NO_SHADOW: u32 = 0xFFFF_FFFF;
pub const HL_FRAGMENTS_FORWARD: u32 = 0;
pub const HL_FRAGMENTS_TRANSPARENT: u32 = 1;
pub const HL_GBUFFER_TARGETS: usize = 8;
pub const HL_ADJOINT_MAX_LIGHTS: u32 = 65536;
pub const HL_NOALLOC_MAX_LIGHTS: u32 = 4096;
pub const HL_NOALLOC_MAX_FROXELS: u32 = 32768;

#[repr(C)]
pub struct hl_ctx {
    _opaque: [u8; 0],
}
#[repr(C)]
pub struct hl_batch_plan {
    _opaque: [u8; 0],
}

#[repr(C)]
#[derive(Clone, Copy, Debug, Default)]
pub struct hl_froxel_params {
    pub grid_x: u32,
    pub grid_y: u32,
    pub grid_z: u32,
    pub width: u32,
    pub height: u32,
    pub slice_near: f32,
    pub slice_far: f32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_froxel_lists {
    pub offsets: *mut u32,
    pub indices: *mut u32,
    pub capacity: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_gbuffer {
    pub layout: u32,
    pub width: u32,
    pub height: u32,
    pub reserved: u32,
    pub planes: [*const c_void; HL_GBUF_MAX_PLANES],
    pub pitch: [u64; HL_GBUF_MAX_PLANES],
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_light_grid {
    pub kind: u32,
    pub lists_capacity: u32,
    pub lists: *const u32,
    pub counts: *const u32,
    pub froxel: hl_froxel_params,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_target {
    pub data: *mut c_void,
    pub pitch: u64,
    pub format: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_shadow_maps {
    pub dynamic_atlas: *const f32,
    pub static_atlas: *const f32,
    pub matrices: *const c_void,
    pub config: *const c_void,
    pub size: u32,
    pub layers: u32,
    pub max_shadow_lights: u32,
    pub reserved: u32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_rc_cascade {
    pub texels: *const c_void,
    pub pitch: u64,
    pub width: u32,
    pub height: u32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_shade_bindings {
    pub shadows: *const hl_shadow_maps,
    pub rc: *const hl_rc_cascade,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_reflection_env {
    pub captures: *const c_void,
    pub count: u32,
    pub face_size: u32,
    pub mip_levels: u32,
    pub layers: u32,
    pub texels: *const c_void,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_reflection_inputs {
    pub ssr: *const c_void,
    pub ssr_pitch: u64,
    pub planar: *const c_void,
    pub planar_pitch: u64,
    pub lightmap_uv: *const c_void,
    pub lightmap_uv_pitch: u64,
    pub rc: *const hl_rc_cascade,
    pub env: *const hl_reflection_env,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_fragment_params {
    pub mode: u32,
    pub num_tiles_x: u32,
    pub ambient_intensity: f32,
    pub ambient_color: [f32; 3],
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_surface {
    pub world_normal: [f32; 3],
    pub bitangent_sign: f32,
    pub world_tangent: [f32; 3],
    pub material_id: u32,
    pub tex_coords: [f32; 2],
    pub lightmap_uv: [f32; 2],
    pub prev_clip: [f32; 4],
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_texture {
    pub texels: *const c_void,
    pub pitch: u64,
    pub width: u32,
    pub height: u32,
    pub format: u32,
    pub address_u: u32,
    pub address_v: u32,
    pub filter: u32,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_gbuffer_targets {
    pub width: u32,
    pub height: u32,
    pub reserved: [u32; 2],
    pub planes: [*mut c_void; HL_GBUFFER_TARGETS],
    pub pitch: [u64; HL_GBUFFER_TARGETS],
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_view {
    pub camera: *const c_void,
    pub gbuffer: hl_gbuffer,
    pub radiance: hl_target,
}

#[repr(C)]
#[derive(Clone, Copy)]
pub struct hl_batch_config {
    pub autotune: u32,
    pub grid_x: u32,
    pub grid_y: u32,
    pub grid_z: u32,
    pub cache_path: *const c_char,
}

#[link(name = "helio_gb300")]
extern "C" {
    pub fn hl_abi_version() -> u32;
    pub fn hl_status_string(status: hl_status) -> *const c_char;
    pub fn hl_create(out_ctx: *mut *mut hl_ctx, cuda_device: c_int) -> hl_status;
    pub fn hl_destroy(ctx: *mut hl_ctx) -> hl_status;
    pub fn hl_last_error_message(ctx: *const hl_ctx) -> *const c_char;
    pub fn hl_sync_status(ctx: *mut hl_ctx, stream: *mut c_void) -> hl_status;
    pub fn hl_tile_count(width: u32, height: u32) -> u32;
    pub fn hl_bin_tiles_ref(ctx: *mut hl_ctx, camera: *const c_void, lights: *const c_void, n_lights: u32,
                            width: u32, height: u32, tile_lists: *mut u32, tile_counts: *mut u32,
                            stream: *mut c_void) -> hl_status;
    pub fn hl_froxel_slice_table(params: *const hl_froxel_params, out_host: *mut f32) -> hl_status;
    pub fn hl_bin_froxels(ctx: *mut hl_ctx, camera: *const c_void, lights: *const c_void, n_lights: u32,
                          params: *const hl_froxel_params, out: *const hl_froxel_lists,
                          stream: *mut c_void) -> hl_status;
    pub fn hl_inject_binning_stall(ctx: *mut hl_ctx, item: u32, spins: u32) -> hl_status;
    pub fn hl_bin_froxels_noalloc(camera: *const c_void, lights: *const c_void, n_lights: u32,
                                  params: *const hl_froxel_params, out: *const hl_froxel_lists,
                                  stream: *mut c_void) -> hl_status;
    pub fn hl_shade(ctx: *mut hl_ctx, camera: *const c_void, globals: *const c_void, gbuffer: *const hl_gbuffer,
                    lights: *const c_void, n_lights: u32, grid: *const hl_light_grid, radiance: *const hl_target,
                    stream: *mut c_void) -> hl_status;
    pub fn hl_shade_shadowed(ctx: *mut hl_ctx, camera: *const c_void, globals: *const c_void,
                             gbuffer: *const hl_gbuffer, lights: *const c_void, n_lights: u32,
                             grid: *const hl_light_grid, shadows: *const hl_shadow_maps,
                             radiance: *const hl_target, stream: *mut c_void) -> hl_status;
    pub fn hl_shade_ex(ctx: *mut hl_ctx, camera: *const c_void, globals: *const c_void, gbuffer: *const hl_gbuffer,
                       lights: *const c_void, n_lights: u32, grid: *const hl_light_grid,
                       bindings: *const hl_shade_bindings, radiance: *const hl_target,
                       stream: *mut c_void) -> hl_status;
    pub fn hl_shade_reflections(ctx: *mut hl_ctx, camera: *const c_void, globals: *const c_void,
                                gbuffer: *const hl_gbuffer, inputs: *const hl_reflection_inputs,
                                radiance: *const hl_target, stream: *mut c_void) -> hl_status;
    pub fn hl_shade_stats(ctx: *mut hl_ctx, camera: *const c_void, globals: *const c_void,
                          gbuffer: *const hl_gbuffer, lights: *const c_void, n_lights: u32,
                          grid: *const hl_light_grid, counts: *mut u32, stream: *mut c_void) -> hl_status;
    pub fn hl_set_pair_log(ctx: *mut hl_ctx, pairs: *mut u32, capacity: u32, count: *mut u32) -> hl_status;
    pub fn hl_shade_adjoint(ctx: *mut hl_ctx, camera: *const c_void, globals: *const c_void,
                            gbuffer: *const hl_gbuffer, lights: *const c_void, n_lights: u32,
                            grid: *const hl_light_grid, d_radiance: *const f32, d_radiance_pitch: u64,
                            d_lights: *mut f64, d_pixels: *mut f32, stream: *mut c_void) -> hl_status;
    pub fn hl_shade_fragments(ctx: *mut hl_ctx, camera: *const c_void, params: *const hl_fragment_params,
                              fragments: *const c_void, n_fragments: u32, lights: *const c_void, n_lights: u32,
                              light_entity_indices: *const u32, transforms: *const c_void, n_transforms: u32,
                              grid: *const hl_light_grid, out_rgba: *mut f32, stream: *mut c_void) -> hl_status;
    pub fn hl_write_gbuffer(ctx: *mut hl_ctx, globals: *const c_void, surfaces: *const hl_surface,
                            surfaces_pitch: u64, materials: *const c_void, material_textures: *const c_void,
                            n_materials: u32, textures: *const hl_texture, n_textures: u32,
                            targets: *const hl_gbuffer_targets, stream: *mut c_void) -> hl_status;
    pub fn hl_batch_plan_create(ctx: *mut hl_ctx, views: *const hl_view, n_views: u32, lights: *const c_void,
                                n_lights: u32, globals: *const c_void, config: *const hl_batch_config,
                                out_plan: *mut *mut hl_batch_plan, stream: *mut c_void) -> hl_status;
    pub fn hl_batch_execute(ctx: *mut hl_ctx, plan: *mut hl_batch_plan, stream: *mut c_void) -> hl_status;
    pub fn hl_batch_plan_view_grid(plan: *const hl_batch_plan, view: u32, grid_xyz: *mut u32) -> hl_status;
    pub fn hl_batch_plan_destroy(plan: *mut hl_batch_plan) -> hl_status;
    /// Measurement only (the FP32 roofline denominator of a benchmark); never call it from a frame.
    pub fn hl_probe_fp32_peak(ctx: *mut hl_ctx, tflops: *mut f64) -> hl_status;
}
