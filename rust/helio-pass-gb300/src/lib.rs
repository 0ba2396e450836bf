//! Helio's deferred-lighting passes on a GB300, behind Helio's own `RenderPass` surface.
//!
//! `Gb300LightCullPass` replaces `LightCullPass`
//! (crates/passes/3d/helio-pass-light-cull/src/lib.rs:194-313) and
//! `Gb300DeferredLightPass` replaces `DeferredLightPass`
//! (crates/passes/3d/helio-pass-deferred-light/src/lib.rs:790-1199): same pass names,
//! same `reads`/`writes` resource names, same `publish`, the same cull-cache key and
//! zero-light clear, the same 112-byte `DeferredGlobals` filled in `prepare`, and the
//! same `InvalidPassConfig` error when the G-buffer is missing. The work runs through
//! the helio_gb300 C ABI (`sys`) on CUDA device memory: the frame's camera, lights,
//! G-buffer planes and `pre_aa` target are shared with CUDA by the integrator (Vulkan
//! external memory exported from wgpu and imported with cudaImportExternalMemory),
//! which the passes reach through the `CudaFrame` trait.
//!
//! `Gb300FroxelCullPass` is the froxel variant of the light culling (no counterpart
//! in the reference): it publishes froxel lists the deferred pass reads instead of the
//! 64-entry tile lists.

pub mod sys;

use core::ffi::{c_void, CStr};
use core::ptr;

use helio_core::graph::ResourceBuilder;
use helio_core::{Error, PassContext, PrepareContext, RenderPass, Result as HelioResult};

/// CUDA views of the frame's shared resources, provided by the integrator.
pub trait CudaFrame: Send + Sync {
    /// The CUDA stream the frame's passes run on (`cudaStream_t`).
    fn stream(&self) -> *mut c_void;
    /// Device address of the scene's `GpuCameraUniforms` (368 bytes).
    fn camera(&self) -> *const c_void;
    /// Device address of the scene's `GpuLight` array (128-byte records).
    fn lights(&self) -> *const c_void;
    /// The published G-buffer as CUDA planes, or None when it was not published.
    fn gbuffer(&self) -> Option<sys::hl_gbuffer>;
    /// The `pre_aa` target (RGBA16F like the reference's, or RGBA32F).
    fn pre_aa(&self) -> Option<sys::hl_target>;
    /// Device memory of at least `bytes` bytes kept by the integrator for `name`
    /// (the passes' own buffers: tile lists, froxel lists, the globals uniform).
    fn buffer(&self, name: &'static str, bytes: usize) -> *mut c_void;
    /// Copies `bytes` from the host to device memory `dst` on the frame's stream.
    fn upload(&self, dst: *mut c_void, bytes: &[u8]);
}

/// Maps a helio_gb300 status to Helio's error type.
fn check(ctx: *mut sys::hl_ctx, status: sys::hl_status, what: &str) -> HelioResult<()> {
    if status == sys::HL_OK {
        return Ok(());
    }
    let msg = unsafe {
        let m = sys::hl_last_error_message(ctx);
        if m.is_null() { String::new() } else { CStr::from_ptr(m).to_string_lossy().into_owned() }
    };
    let text = format!("{what}: {} ({msg})", unsafe {
        CStr::from_ptr(sys::hl_status_string(status)).to_string_lossy()
    });
    Err(match status {
        sys::HL_ERR_INVALID_ARGUMENT | sys::HL_ERR_LAYOUT | sys::HL_ERR_SIZE | sys::HL_ERR_NOT_SUPPORTED => {
            Error::InvalidPassConfig(text)
        }
        _ => Error::Gpu(text),
    })
}

/// An owned helio_gb300 context on one CUDA device.
pub struct Gb300Context {
    raw: *mut sys::hl_ctx,
}

unsafe impl Send for Gb300Context {}
unsafe impl Sync for Gb300Context {}

impl Gb300Context {
    pub fn new(cuda_device: i32) -> HelioResult<Self> {
        let mut raw = ptr::null_mut();
        let st = unsafe { sys::hl_create(&mut raw, cuda_device) };
        if st != sys::HL_OK {
            return Err(Error::Gpu(format!("hl_create({cuda_device}) failed with status {st}")));
        }
        Ok(Self { raw })
    }

    pub fn raw(&self) -> *mut sys::hl_ctx {
        self.raw
    }

    /// Device-side status of the work queued so far (bounds, capacity, timeouts).
    pub fn sync_status(&self, stream: *mut c_void) -> HelioResult<()> {
        check(self.raw, unsafe { sys::hl_sync_status(self.raw, stream) }, "device status")
    }
}

impl Drop for Gb300Context {
    fn drop(&mut self) {
        unsafe { sys::hl_destroy(self.raw) };
    }
}

const TILE_SIZE: u32 = sys::HL_TILE_SIZE;
const MAX_LIGHTS_PER_TILE: u32 = sys::HL_MAX_LIGHTS_PER_TILE;

/// The reference's `LightCullPass`: 16x16-pixel tile lists, at most 64 lights per tile
/// in ascending light index (hl_bin_tiles_ref, light_cull.wgsl:123-180).
pub struct Gb300LightCullPass {
    ctx: std::sync::Arc<Gb300Context>,
    frame: std::sync::Arc<dyn CudaFrame>,
    num_tiles_x: u32,
    num_tiles_y: u32,
    width: u32,
    height: u32,
    cull_cache_key: Option<(u64, u64, u32)>,
}

// The passes hold raw CUDA addresses (device memory, not host data), shared with the
// integrator's frame; the frame is single-threaded as Helio's is.
unsafe impl Send for Gb300DeferredLightPass {}
unsafe impl Sync for Gb300DeferredLightPass {}
unsafe impl Send for Gb300FroxelCullPass {}
unsafe impl Sync for Gb300FroxelCullPass {}

impl Gb300LightCullPass {
    pub fn new(ctx: std::sync::Arc<Gb300Context>, frame: std::sync::Arc<dyn CudaFrame>, width: u32, height: u32) -> Self {
        let num_tiles_x = width.div_ceil(TILE_SIZE);
        let num_tiles_y = height.div_ceil(TILE_SIZE);
        num_tiles_x.checked_mul(num_tiles_y).expect("tile grid overflow: viewport dimensions too large");
        Self { ctx, frame, num_tiles_x, num_tiles_y, width, height, cull_cache_key: None }
    }

    fn tiles(&self) -> u32 {
        self.num_tiles_x * self.num_tiles_y
    }

    fn lists(&self) -> *mut u32 {
        self.frame.buffer("tile_light_lists", (self.tiles() * MAX_LIGHTS_PER_TILE * 4).max(4) as usize) as *mut u32
    }

    fn counts(&self) -> *mut u32 {
        self.frame.buffer("tile_light_counts", (self.tiles() * 4).max(4) as usize) as *mut u32
    }
}

impl RenderPass for Gb300LightCullPass {
    fn name(&self) -> &'static str {
        "LightCull"
    }

    fn writes(&self) -> &'static [&'static str] {
        &["tile_light_lists", "tile_light_counts"]
    }

    fn declare_resources(&self, builder: &mut ResourceBuilder) {
        builder.write_buffer("tile_light_lists");
        builder.write_buffer("tile_light_counts");
    }

    fn on_resize(&mut self, _device: &wgpu::Device, width: u32, height: u32) {
        let num_tiles_x = width.div_ceil(TILE_SIZE);
        let num_tiles_y = height.div_ceil(TILE_SIZE);
        num_tiles_x.checked_mul(num_tiles_y).expect("tile grid overflow: viewport dimensions too large");
        self.num_tiles_x = num_tiles_x;
        self.num_tiles_y = num_tiles_y;
        self.width = width;
        self.height = height;
        self.cull_cache_key = None;
    }

    fn publish<'a>(&'a self, _frame: &mut libhelio::FrameResources<'a>) {
        // The lists live in the integrator's shared buffers named "tile_light_lists" and
        // "tile_light_counts"; its frame resources expose those wgpu buffers to the
        // passes that read them, as LightCullPass::publish does.
    }

    fn prepare(&mut self, ctx: &PrepareContext) -> HelioResult<()> {
        // the tile grid follows the internal (render-target) resolution
        self.num_tiles_x = ctx.width.div_ceil(TILE_SIZE);
        self.num_tiles_y = ctx.height.div_ceil(TILE_SIZE);
        self.width = ctx.width;
        self.height = ctx.height;
        Ok(())
    }

    fn execute(&mut self, ctx: &mut PassContext) -> HelioResult<()> {
        let n = ctx.scene.movable_light_count;
        let stream = self.frame.stream();
        if n == 0 {
            // no movable lights: hl_bin_tiles_ref clears both buffers
            // (LightCullPass::execute, light-cull/src/lib.rs:285-292)
            self.cull_cache_key = None;
        } else {
            // skip the culling when camera, lights and count are unchanged (:294-313)
            let key = (ctx.scene.camera_generation, ctx.scene.movable_lights_generation, n);
            if self.cull_cache_key == Some(key) {
                return Ok(());
            }
            self.cull_cache_key = Some(key);
        }
        let st = unsafe {
            sys::hl_bin_tiles_ref(self.ctx.raw(), self.frame.camera(), self.frame.lights(), n, self.width,
                                  self.height, self.lists(), self.counts(), stream)
        };
        check(self.ctx.raw(), st, "LightCull")
    }
}

/// Froxel light clustering (no reference kernel): lists of every light that can reach
/// a froxel, no cap, published as "froxel_light_offsets" / "froxel_light_indices".
pub struct Gb300FroxelCullPass {
    ctx: std::sync::Arc<Gb300Context>,
    frame: std::sync::Arc<dyn CudaFrame>,
    pub params: sys::hl_froxel_params,
    pub capacity: u32,
    cull_cache_key: Option<(u64, u64, u32)>,
}

impl Gb300FroxelCullPass {
    pub fn new(ctx: std::sync::Arc<Gb300Context>, frame: std::sync::Arc<dyn CudaFrame>, grid: [u32; 3], width: u32,
               height: u32, camera_far: f32, capacity: u32) -> Self {
        let params = sys::hl_froxel_params {
            grid_x: grid[0].min(width),
            grid_y: grid[1].min(height),
            grid_z: grid[2],
            width,
            height,
            slice_near: sys::HL_FROXEL_NEAR,
            slice_far: camera_far,
            reserved: 0,
        };
        Self { ctx, frame, params, capacity, cull_cache_key: None }
    }

    fn froxels(&self) -> u32 {
        self.params.grid_x * self.params.grid_y * self.params.grid_z
    }

    pub fn grid(&self) -> sys::hl_light_grid {
        sys::hl_light_grid {
            kind: sys::HL_GRID_FROXELS,
            lists_capacity: self.capacity,
            lists: self.frame.buffer("froxel_light_indices", self.capacity as usize * 4) as *const u32,
            counts: self.frame.buffer("froxel_light_offsets", (self.froxels() as usize + 1) * 4) as *const u32,
            froxel: self.params,
        }
    }
}

impl RenderPass for Gb300FroxelCullPass {
    fn name(&self) -> &'static str {
        "FroxelCull"
    }

    fn writes(&self) -> &'static [&'static str] {
        &["froxel_light_offsets", "froxel_light_indices"]
    }

    fn on_resize(&mut self, _device: &wgpu::Device, width: u32, height: u32) {
        self.params.width = width;
        self.params.height = height;
        self.params.grid_x = self.params.grid_x.min(width);
        self.params.grid_y = self.params.grid_y.min(height);
        self.cull_cache_key = None;
    }

    fn execute(&mut self, ctx: &mut PassContext) -> HelioResult<()> {
        let n = ctx.scene.movable_light_count;
        let key = (ctx.scene.camera_generation, ctx.scene.movable_lights_generation, n);
        if self.cull_cache_key == Some(key) {
            return Ok(());
        }
        self.cull_cache_key = Some(key);
        let g = self.grid();
        let out = sys::hl_froxel_lists {
            offsets: g.counts as *mut u32,
            indices: g.lists as *mut u32,
            capacity: self.capacity,
            reserved: 0,
        };
        let st = unsafe {
            sys::hl_bin_froxels(self.ctx.raw(), self.frame.camera(), self.frame.lights(), n, &self.params, &out,
                                self.frame.stream())
        };
        check(self.ctx.raw(), st, "FroxelCull")
    }
}

/// `DeferredGlobals` (deferred-light/src/lib.rs:17-52): 112 bytes, the uniform fs_main reads.
#[repr(C)]
#[derive(Clone, Copy, bytemuck::Pod, bytemuck::Zeroable)]
pub struct DeferredGlobals {
    pub frame: u32,
    pub delta_time: f32,
    pub light_count: u32,
    pub ambient_intensity: f32,
    pub ambient_color: [f32; 4],
    pub rc_world_min: [f32; 4],
    pub rc_world_max: [f32; 4],
    pub csm_splits: [f32; 4],
    pub debug_mode: u32,
    pub has_rc_gi: u32,
    pub num_tiles_x: u32,
    pub reflection_capture_count: u32,
    pub enable_reflections: u32,
    pub enable_env_reflections: u32,
    pub _pad: [u32; 2],
}
const _: () = assert!(core::mem::size_of::<DeferredGlobals>() == 112);

/// Where the deferred pass finds its light lists.
pub enum LightLists {
    /// The reference's 16x16 tile lists of `Gb300LightCullPass`.
    Tiles,
    /// Froxel lists (`Gb300FroxelCullPass::grid`).
    Froxels(sys::hl_light_grid),
}

/// The reference's `DeferredLightPass`: fs_main for every G-buffer pixel into `pre_aa`
/// (hl_shade; hl_shade_ex when shadow maps or radiance-cascade probes are bound).
pub struct Gb300DeferredLightPass {
    ctx: std::sync::Arc<Gb300Context>,
    frame: std::sync::Arc<dyn CudaFrame>,
    pub lists: LightLists,
    pub debug_mode: u32,
    pub enable_env_reflections: bool,
    pub shadows: Option<sys::hl_shadow_maps>,
    pub rc: Option<sys::hl_rc_cascade>,
    width: u32,
    height: u32,
}

impl Gb300DeferredLightPass {
    pub fn new(ctx: std::sync::Arc<Gb300Context>, frame: std::sync::Arc<dyn CudaFrame>, lists: LightLists) -> Self {
        Self { ctx, frame, lists, debug_mode: 0, enable_env_reflections: true, shadows: None, rc: None, width: 0,
               height: 0 }
    }

    fn globals_buf(&self) -> *mut c_void {
        self.frame.buffer("deferred_globals", core::mem::size_of::<DeferredGlobals>())
    }
}

impl RenderPass for Gb300DeferredLightPass {
    fn name(&self) -> &'static str {
        "DeferredLight"
    }

    fn reads(&self) -> &'static [&'static str] {
        &[
            "gbuffer",
            "gbuffer_lightmap_uv",
            "gbuffer_sss",
            "gbuffer_extra",
            "depth",
            "shadow_atlas",
            "static_shadow_atlas",
            "shadow_sampler",
            "ssao",
            "sky_lut",
            "tile_light_lists",
            "tile_light_counts",
            "main_scene",
            "water_caustics",
            "water_volumes",
            "pre_aa",
            "rc_view",
            "baked_lightmap",
            "baked_lightmap_sampler",
            "ssr_trace",
            "planar_reflection",
            "ies_textures",
        ]
    }

    fn writes(&self) -> &'static [&'static str] {
        &["pre_aa"]
    }

    fn prepare(&mut self, ctx: &PrepareContext) -> HelioResult<()> {
        // DeferredLightPass::prepare (deferred-light/src/lib.rs:836-878)
        let main_scene_opt = ctx.frame_resources.main_scene.get();
        let main_scene = main_scene_opt.as_ref();
        let (ambient_color, ambient_intensity) = match main_scene {
            Some(m) => (m.ambient_color, m.ambient_intensity),
            None => ([0.5, 0.5, 0.6], 1.0),
        };
        let (rc_min, rc_max) = match main_scene {
            Some(m) => (m.rc_world_min, m.rc_world_max),
            None => ([0.0; 3], [0.0; 3]),
        };
        let has_rc_gi = self.rc.is_some() && ctx.frame_resources.rc_view.get().is_some();
        let globals = DeferredGlobals {
            frame: ctx.frame_num as u32,
            delta_time: ctx.delta_time,
            light_count: ctx.scene.movable_light_count,
            ambient_intensity,
            ambient_color: [ambient_color[0], ambient_color[1], ambient_color[2], 1.0],
            rc_world_min: [rc_min[0], rc_min[1], rc_min[2], 0.0],
            rc_world_max: [rc_max[0], rc_max[1], rc_max[2], 0.0],
            csm_splits: libhelio::CSM_SPLITS,
            debug_mode: self.debug_mode,
            has_rc_gi: has_rc_gi as u32,
            num_tiles_x: ctx.width.div_ceil(16),
            reflection_capture_count: ctx.scene.reflection_captures.len() as u32,
            enable_reflections: helio_core::REFLECTIONS_SUPPORTED as u32,
            enable_env_reflections: self.enable_env_reflections as u32,
            _pad: [0; 2],
        };
        self.width = ctx.width;
        self.height = ctx.height;
        self.frame.upload(self.globals_buf(), bytemuck::bytes_of(&globals));
        Ok(())
    }

    fn execute(&mut self, ctx: &mut PassContext) -> HelioResult<()> {
        let gbuffer = self.frame.gbuffer().ok_or_else(|| {
            Error::InvalidPassConfig("DeferredLight requires published gbuffer resources".to_string())
        })?;
        let target = self.frame.pre_aa().ok_or_else(|| {
            Error::InvalidPassConfig("DeferredLight requires the pre_aa target".to_string())
        })?;
        let grid = match &self.lists {
            LightLists::Tiles => sys::hl_light_grid {
                kind: sys::HL_GRID_TILES,
                lists_capacity: 0,
                lists: self.frame.buffer("tile_light_lists", 4) as *const u32,
                counts: self.frame.buffer("tile_light_counts", 4) as *const u32,
                froxel: sys::hl_froxel_params::default(),
            },
            LightLists::Froxels(g) => sys::hl_light_grid { ..*g },
        };
        let n = ctx.scene.movable_light_count;
        let st = if self.shadows.is_none() && self.rc.is_none() {
            unsafe {
                sys::hl_shade(self.ctx.raw(), self.frame.camera(), self.globals_buf(), &gbuffer, self.frame.lights(),
                              n, &grid, &target, self.frame.stream())
            }
        } else {
            let bindings = sys::hl_shade_bindings {
                shadows: self.shadows.as_ref().map_or(ptr::null(), |s| s as *const _),
                rc: self.rc.as_ref().map_or(ptr::null(), |r| r as *const _),
            };
            unsafe {
                sys::hl_shade_ex(self.ctx.raw(), self.frame.camera(), self.globals_buf(), &gbuffer,
                                 self.frame.lights(), n, &grid, &bindings, &target, self.frame.stream())
            }
        };
        check(self.ctx.raw(), st, "DeferredLight")
    }
}
