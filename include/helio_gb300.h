/*
 * helio_gb300.h — C ABI of the GB300 (sm_103a) deferred-lighting engine.
 *
 * This library replaces the two passes on Helio's deferred-lighting path:
 *
 *   LightCullPass     crates/passes/3d/helio-pass-light-cull/src/lib.rs:41-362
 *                     + shaders/light_cull.wgsl:123-180
 *   DeferredLightPass crates/passes/3d/helio-pass-deferred-light/src/lib.rs:110-1199
 *                     + shaders/deferred_lighting.wgsl:699-820,991-1259
 *
 * Conventions
 *   - Every pointer named as "device" is a CUDA device pointer owned by the caller.
 *     Byte layouts are Helio's: GpuLight (128 B, libhelio/src/light.rs:60-115),
 *     GpuCameraUniforms (368 B, libhelio/src/camera.rs:12-29), DeferredGlobals
 *     (112 B, helio-pass-deferred-light/src/lib.rs:17-52).
 *   - `stream` is a cudaStream_t passed as void* (0 = legacy default stream).
 *     All work is enqueued asynchronously on it. hl_bin_froxels and hl_shade enqueue
 *     some kernels as programmatic dependent launches: they may start while this
 *     library's preceding kernel on the stream still runs, and read nothing it writes
 *     before it completes. Work of the caller's between two calls is ordered as usual.
 *   - Argument errors are returned synchronously. Device-side conditions (an
 *     out-of-range light index, froxel index capacity exceeded, a bounded wait that
 *     gave up) raise a flag in the context that hl_sync_status() reports.
 *   - One hl_ctx is not reentrant: calls on one context must come from one host
 *     thread at a time (the reference's frame is single threaded,
 *     helio-core/src/context.rs:13-15). Different contexts are independent.
 *   - No function falls back to the CPU. Without a usable GPU, hl_create fails.
 */
#ifndef HELIO_GB300_H
#define HELIO_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define HL_ABI_VERSION 1u

/* Reference constants (light_cull.wgsl:17-18, deferred_lighting.wgsl:199-200). */
#define HL_TILE_SIZE 16u
#define HL_MAX_LIGHTS_PER_TILE 64u
/* Froxel slice-mapping near plane (helio-core/src/shader/prelude.wgsl:195). */
#define HL_FROXEL_NEAR 0.5f

/* Byte sizes of the reference's POD structs. */
#define HL_SIZEOF_GPU_LIGHT 128u
#define HL_SIZEOF_GPU_CAMERA 368u
#define HL_SIZEOF_DEFERRED_GLOBALS 112u
#define HL_SIZEOF_LIGHT_CULL_PARAMS 32u
#define HL_SIZEOF_GPU_MATERIAL 96u

typedef int32_t hl_status;
#define HL_OK 0
#define HL_ERR_INVALID_ARGUMENT (-1) /* null pointer, zero-sized grid, bad enum     */
#define HL_ERR_LAYOUT (-2)           /* misaligned pointer or pitch for the layout  */
#define HL_ERR_SIZE (-3)             /* a size beyond the limits the kernels support */
#define HL_ERR_CUDA (-4)             /* a CUDA runtime call failed                  */
#define HL_ERR_TIMEOUT (-5)          /* a bounded device-side wait gave up          */
#define HL_ERR_CAPACITY (-6)         /* froxel index buffer too small               */
#define HL_ERR_DEVICE_BOUNDS (-7)    /* a device-side bounds check rejected an index */
#define HL_ERR_NOT_SUPPORTED (-8)    /* valid request this build does not implement */

typedef struct hl_ctx hl_ctx;

/* ---------------------------------------------------------------------------------
 * Context
 * -------------------------------------------------------------------------------*/

/* Library ABI version (HL_ABI_VERSION of the build). */
uint32_t hl_abi_version(void);

/* Human-readable text for a status code. Never NULL. */
const char* hl_status_string(hl_status status);

/* Creates a context bound to `cuda_device`. Holds scratch memory, the device-side
 * status word and cached batch plans. Replaces the per-pass GPU state the reference
 * keeps in LightCullPass / DeferredLightPass (light-cull/src/lib.rs:41-61,
 * deferred-light/src/lib.rs:54-108). */
hl_status hl_create(hl_ctx** out_ctx, int cuda_device);

/* Frees everything the context owns. NULL is accepted. */
hl_status hl_destroy(hl_ctx* ctx);

/* Message of the last error recorded on this context ("" if none). */
const char* hl_last_error_message(const hl_ctx* ctx);

/* Synchronises `stream`, reads and clears the context's device-side status word and
 * returns it (HL_OK, HL_ERR_CAPACITY, HL_ERR_DEVICE_BOUNDS or HL_ERR_TIMEOUT). */
hl_status hl_sync_status(hl_ctx* ctx, void* stream);

/* ---------------------------------------------------------------------------------
 * Tile light culling — the reference's LightCullPass
 * -------------------------------------------------------------------------------*/

/* Number of 16-pixel tiles of a width x height target, ceil(w/16)*ceil(h/16)
 * (light-cull/src/lib.rs:65-69). Returns 0 on overflow. */
uint32_t hl_tile_count(uint32_t width, uint32_t height);

/* Bins lights into 16x16-pixel screen tiles exactly like light_cull.wgsl:123-180:
 * four lateral planes per tile, sphere test in view space, directional lights always
 * listed, at most 64 lights per tile in ascending light index (the 65th and later are
 * dropped). Output buffers have the reference's shapes: tile_lists[tiles*64] (slot
 * tile*64+i) and tile_counts[tiles]. With n_lights == 0 both buffers are cleared, as
 * LightCullPass::execute does (light-cull/src/lib.rs:285-292).
 *   camera : device, GpuCameraUniforms (only view and proj are read)
 *   lights : device, GpuLight[n_lights]
 * Replaces: LightCullPass::prepare + execute (light-cull/src/lib.rs:264-362). */
hl_status hl_bin_tiles_ref(hl_ctx* ctx, const void* camera, const void* lights, uint32_t n_lights,
                           uint32_t width, uint32_t height, uint32_t* tile_lists,
                           uint32_t* tile_counts, void* stream);

/* ---------------------------------------------------------------------------------
 * Froxel light clustering (no reference kernel; slice convention of
 * helio-core/src/shader/prelude.wgsl:185-211)
 * -------------------------------------------------------------------------------*/

typedef struct hl_froxel_params {
    uint32_t grid_x, grid_y, grid_z; /* froxel grid                              */
    uint32_t width, height;          /* viewport in pixels                       */
    float slice_near;                /* first exponential slice boundary (0.5)   */
    float slice_far;                 /* last slice boundary, usually camera far  */
    uint32_t reserved;               /* must be 0                                */
} hl_froxel_params;

typedef struct hl_froxel_lists {
    uint32_t* offsets; /* device, F+1 entries, F = grid_x*grid_y*grid_z; offsets[F] = total */
    uint32_t* indices; /* device, `capacity` entries                                        */
    uint32_t capacity;
    uint32_t reserved;
} hl_froxel_lists;

/* Host helper: the f32 view-depth boundaries of the grid's slices, grid_z+1 values.
 * With F = max(slice_far, 2*slice_near): out[0] = 0 (slice 0 also holds everything
 * nearer than slice_near), out[k] = slice_near*(F/slice_near)^(k/grid_z) for
 * 0<k<grid_z (prelude.wgsl:202-211), out[grid_z] = F. Pixels beyond F fall in the last
 * slice, whose box reaches to max(F, camera far). Computed in double and rounded to
 * f32; binning and shading both use exactly these values. */
hl_status hl_froxel_slice_table(const hl_froxel_params* params, float* out_host);

/* Clusters lights into froxels. A froxel (fx,fy,s) is the view-space box spanned by
 * the pixel columns with (px*grid_x)/width == fx, the rows with (py*grid_y)/height == fy
 * and the slice's depth range, widened by a 2^-10 relative margin. A light is listed
 * when its range sphere meets the box (Arvo), and for a spot with 0 < cos_outer <
 * cos_inner also when its outer cone meets the box's bounding sphere; directional
 * lights are always listed. Lists are in ascending light index with no cap, froxel
 * index f = (fy*grid_x + fx)*grid_z + s, offsets[] is the exclusive prefix sum. The
 * result is deterministic and bit-identical to the documented f32 operation order.
 * If the total exceeds `capacity`, only indices below capacity are written, offsets
 * are still complete, and hl_sync_status reports HL_ERR_CAPACITY. */
hl_status hl_bin_froxels(hl_ctx* ctx, const void* camera, const void* lights, uint32_t n_lights,
                         const hl_froxel_params* params, const hl_froxel_lists* out,
                         void* stream);

/* Failure injection for the device-side wait of hl_bin_froxels (no reference
 * counterpart). The single-launch binning splits the grid into work items (a froxel
 * column, or a group of its slices) and finds where each item's lists start by
 * polling the running totals that earlier items publish; each poll loop is bounded
 * (about 0.1 s), after which the kernel reports HL_ERR_TIMEOUT through hl_sync_status
 * and finishes instead of hanging. After this call, the context's next hl_bin_froxels
 * runs with work item `item` withholding its total and the other items giving up after
 * `spins` polls (1..2^20), so a test can trip the bound: the call reports
 * HL_ERR_TIMEOUT, its lists are not valid, and the context stays usable (the next call
 * bins normally). */
hl_status hl_inject_binning_stall(hl_ctx* ctx, uint32_t item, uint32_t spins);

/* Froxel clustering for callers that cannot allocate device memory. No counterpart in
 * the reference. hl_bin_froxels takes its scratch space from the context, which grows
 * it with cudaMalloc; a caller whose frame runs inside a CUDA stream capture (where
 * allocation is not allowed), or whose device memory is all owned by its own pool
 * under a fixed budget, cannot let the library allocate. This entry point needs no
 * context and allocates nothing: it produces the same lists as hl_bin_froxels, with
 * its scratch in one static device array of HL_NOALLOC_MAX_LIGHTS light records and
 * HL_NOALLOC_MAX_FROXELS counts (320 KiB, held by every GPU that loads the library
 * until the process exits). Larger requests return HL_ERR_SIZE.
 *   - The first call on a device looks the array's address up (cudaGetSymbolAddress,
 *     with that device current); make that first call before any stream capture. The
 *     address is kept for the life of the process: do not call this entry point on a
 *     device after cudaDeviceReset of that device.
 *   - All calls share the array: calls that overlap on the GPU (different streams or
 *     host threads) race and must be serialised by the caller.
 *   - There is no device status word: a total above `capacity` shows as
 *     offsets[F] > capacity (indices are written only below capacity). */
#define HL_NOALLOC_MAX_LIGHTS 4096u
#define HL_NOALLOC_MAX_FROXELS 32768u
hl_status hl_bin_froxels_noalloc(const void* camera, const void* lights, uint32_t n_lights,
                                 const hl_froxel_params* params, const hl_froxel_lists* out,
                                 void* stream);

/* ---------------------------------------------------------------------------------
 * Deferred lighting — the reference's DeferredLightPass (fs_main)
 * -------------------------------------------------------------------------------*/

/* G-buffer layouts.
 *  HL_GBUF_REFERENCE (28 B/px, helio-pass-gbuffer/src/lib.rs:236-282):
 *     plane0 albedo RGBA8 unorm (rgb, alpha)      plane1 normal RGBA16F (N.xyz, F0.r)
 *     plane2 orm RGBA8 unorm (ao, rough, metal, F0.g)
 *     plane3 emissive RGBA16F (rgb, F0.b)         plane4 depth R32F (NDC z in [0,1])
 *  HL_GBUF_F32 (36 B/px):
 *     plane0 RGBA32F (albedo.rgb, roughness)      plane1 RGBA32F (N.xyz, metallic)
 *     plane2 depth R32F
 *  HL_GBUF_F16 (18 B/px):
 *     plane0 RGBA16F (albedo.rgb, roughness)      plane1 RG16F octahedral normal
 *     plane2 R16F metallic                        plane3 depth R32F
 *  For F32/F16, F0 = clamp(mix(0.04, albedo, metallic), 0, 0.999) as gbuffer.wgsl:323-328
 *  writes it, ao = 1, emissive = 0, alpha = 1. */
#define HL_GBUF_REFERENCE 0u
#define HL_GBUF_F32 1u
#define HL_GBUF_F16 2u
#define HL_GBUF_MAX_PLANES 6

typedef struct hl_gbuffer {
    uint32_t layout;
    uint32_t width, height;
    uint32_t reserved;
    const void* planes[HL_GBUF_MAX_PLANES]; /* device */
    uint64_t pitch[HL_GBUF_MAX_PLANES];     /* row pitch in bytes */
} hl_gbuffer;

#define HL_GRID_TILES 0u   /* reference tile lists: lists = tile_light_lists, counts = tile_light_counts */
#define HL_GRID_FROXELS 1u /* froxel lists: lists = indices, counts = offsets[F+1]                        */

typedef struct hl_light_grid {
    uint32_t kind;
    uint32_t lists_capacity; /* entries in `lists`; 0 = tiles*64 (tiles) or offsets[F] (froxels) */
    const uint32_t* lists;   /* device */
    const uint32_t* counts;  /* device */
    hl_froxel_params froxel; /* used when kind == HL_GRID_FROXELS */
} hl_light_grid;

#define HL_TARGET_RGBA32F 0u
#define HL_TARGET_RGBA16F 1u

typedef struct hl_target {
    void* data;     /* device */
    uint64_t pitch; /* row pitch in bytes */
    uint32_t format;
    uint32_t reserved;
} hl_target;

/* Direct + ambient + emissive lighting of every G-buffer pixel, fs_main under the
 * pass's fallback bindings (no shadows, RC GI, lightmap, reflections, SSS, IES):
 *   color = sum over the pixel's list of pbr_direct_light + hemisphere ambient * ao
 *           + emissive, alpha from the G-buffer (deferred_lighting.wgsl:991-1259).
 * Pixels with depth >= 1 are left untouched (the shader discards them, :996-997).
 * Lights are summed in list order in f32 with compensated (Kahan) accumulation.
 *   camera  : device GpuCameraUniforms     globals : device DeferredGlobals (112 B)
 *   lights  : device GpuLight[n_lights]    grid    : tile or froxel lists
 * Replaces: DeferredLightPass::prepare + execute (deferred-light/src/lib.rs:836-1199). */
hl_status hl_shade(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                   const void* lights, uint32_t n_lights, const hl_light_grid* grid,
                   const hl_target* radiance, void* stream);

/* Shadow maps of the lights: the deferred pass's shadow bindings
 * (deferred_lighting.wgsl:129-167; libhelio/src/shadow.rs:33-64, light.rs:150-164).
 *   dynamic_atlas, static_atlas : device, Depth32Float layers, `layers` x size x size texels,
 *                                 layer-major, rows of `size` texels (the shader's
 *                                 shadow_atlas and static_shadow_atlas)
 *   matrices                    : device, GpuShadowMatrix[layers] (64 B: column-major light
 *                                 view-projection); a light's layers start at its
 *                                 shadow_index: 6 cube faces (point), cascades 0-3
 *                                 (directional), one (spot)
 *   config                      : device, ShadowConfig (80 B: four cascades of
 *                                 {split_distance, depth_bias, filter_radius,
 *                                 pcss_light_size}, then enable_pcss, pcss_blocker_samples,
 *                                 pcss_filter_samples, pcf_sample_count)
 *   size                        : texels per side; the shader's ATLAS_SIZE (1024)
 *   max_shadow_lights           : lights with an index >= this cast no shadow (the shader's
 *                                 MAX_SHADOW_LIGHTS, 42) */
#define HL_SIZEOF_SHADOW_CONFIG 80u
#define HL_SIZEOF_SHADOW_MATRIX 64u
#define HL_NO_SHADOW 0xFFFFFFFFu
typedef struct hl_shadow_maps {
    const float* dynamic_atlas;
    const float* static_atlas;
    const void* matrices;
    const void* config;
    uint32_t size;
    uint32_t layers;
    uint32_t max_shadow_lights;
    uint32_t reserved; /* must be 0 */
} hl_shadow_maps;

/* hl_shade with the shadow term of fs_main's light loop (deferred_lighting.wgsl:452-565,
 * 1136-1141): each lit (pixel, light) pair is scaled by shadow_factor, for lights with
 * index < max_shadow_lights and shadow_index != HL_NO_SHADOW: the world position offset
 * along N by 0.01 (1 - N.L), projected by the light's matrix (point lights: the cube
 * face of the largest axis of the offset from the light; directional lights: the CSM
 * cascade of the distance to the camera against globals.csm_splits, blended over 10 %
 * zones), then Vogel-disk PCF (sample_cascade_shadow, :283-329) or, for directional
 * cascades with PCSS enabled and a light size, PCSS (:331-450) over both atlases with
 * a LessEqual, bilinear, clamp-to-edge comparison, lit = min(dynamic, static). Points
 * outside a layer's [0,1] uv or depth range are lit. A layer index >= layers is
 * skipped (lit) and reported through hl_sync_status (HL_ERR_DEVICE_BOUNDS). With
 * shadows == NULL this is hl_shade. */
hl_status hl_shade_shadowed(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                            const void* lights, uint32_t n_lights, const hl_light_grid* grid,
                            const hl_shadow_maps* shadows, const hl_target* radiance, void* stream);

/* Radiance-cascade irradiance probes the pass reads for indirect diffuse light
 * (rc_cascade0, deferred_lighting.wgsl:168, 822-917): Rgba16Float texels, probe (x, y, z)
 * of a 16^3 grid over [globals.rc_world_min, rc_world_max] holds 4x4 octahedral
 * directions at column x*4 + dx, row (y*16 + z)*4 + dy. */
#define HL_RC_PROBE_DIM 16u
#define HL_RC_DIR_DIM 4u
typedef struct hl_rc_cascade {
    const void* texels;     /* device, RGBA16F, rows of `pitch` bytes; both 16-byte aligned */
    uint64_t pitch;
    uint32_t width, height; /* at least 64 x 1024 (probe_dim*dir_dim x probe_dim^2*dir_dim) */
} hl_rc_cascade;

/* The optional bindings of the deferred pass that hl_shade_ex reads. */
typedef struct hl_shade_bindings {
    const hl_shadow_maps* shadows; /* NULL: shadow factor 1                                  */
    const hl_rc_cascade* rc;       /* NULL: no radiance-cascade GI (globals.has_rc_gi must be
                                      0, else hl_sync_status reports HL_ERR_NOT_SUPPORTED)   */
} hl_shade_bindings;

/* hl_shade with the pass's optional bindings: the shadow term (as hl_shade_shadowed) and
 * radiance-cascade indirect diffuse light. With rc given and globals.has_rc_gi != 0, each
 * pixel's ambient term becomes mix(hemisphere, kD_ibl * rc_irradiance * albedo, w),
 * w = clamp(4 |rc_irradiance|, 0, 1), kD_ibl from fresnel_schlick_roughness(NdV, F0,
 * roughness) (pbr_eval.wgsl:63-66), rc_irradiance = sample_rc_irradiance (trilinear over
 * the 8 probes around the pixel, cosine-weighted over their 16 directions, faded out
 * over the volume's outer 5 %) times ao, as fs_main composes it
 * (deferred_lighting.wgsl:1159-1228). bindings == NULL, or both NULL, is hl_shade. */
hl_status hl_shade_ex(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                      const void* lights, uint32_t n_lights, const hl_light_grid* grid,
                      const hl_shade_bindings* bindings, const hl_target* radiance, void* stream);

/* The per-pixel inputs of the pass's reflection draw (deferred_lighting.wgsl:176-180,
 * 1265-1341), each a W x H image read at the pixel's own coordinates and each optional:
 *   ssr         screen-space reflection hits, RGBA16F (rgb colour, a confidence), as the
 *               SSR pass writes them at full resolution (helio-pass-ssr/src/lib.rs:16);
 *               NULL = the pass's black fallback, no contribution
 *   planar      planar reflections, RGBA16F, same encoding; NULL = black fallback
 *   lightmap_uv the G-buffer's lightmap UVs, RG16F (x < -1.5 marks virtual geometry,
 *               x >= 0 a lightmapped surface); NULL = every pixel carries the G-buffer's
 *               no-lightmap sentinel (-1, -1) (gbuffer.wgsl:245)
 *   rc          the radiance-cascade probes for the rough-specular fallback.
 * Pitches in bytes; ssr, planar and the rc texels 8-byte aligned, lightmap_uv 4. */
/* Reflection captures and the pre-filtered cube-map array they sample: the pass's
 * reflection_captures and env_cube bindings (deferred_lighting.wgsl:163-198).
 *   captures : device GpuReflectionCapture[count] (112 B: position_radius, extents_transition,
 *              world_to_local (column major), cubemap_index (i32, -1: none), shape (0 sphere,
 *              1 box), mobility, brightness; libhelio/src/reflection.rs:64-80), in the order
 *              the scene uploads them; globals.reflection_capture_count (at most 64) of them
 *              are read
 *   texels   : device RGBA16F, 8-byte aligned: layer-major, each layer 6 faces (+x, -x, +y, -y,
 *              +z, -z), each face its mip chain from level 0, level m a row-major square of
 *              max(1, face_size >> m) texels. Layer 0 is the skylight.
 * Sampling follows the pass's env sampler (linear within a level, nearest level, clamp to
 * edge): the face of the direction's major axis, bilinear within that face with its edge
 * texels clamped (not blended across faces), level round(lod) clamped to the chain. */
#define HL_SIZEOF_REFLECTION_CAPTURE 112u
typedef struct hl_reflection_env {
    const void* captures;
    uint32_t count;        /* entries in captures                         */
    uint32_t face_size;    /* texels per side of level 0, 1..16384        */
    uint32_t mip_levels;   /* levels per face, 1..15                      */
    uint32_t layers;       /* cube layers, >= 1                           */
    const void* texels;
} hl_reflection_env;

typedef struct hl_reflection_inputs {
    const void* ssr;
    uint64_t ssr_pitch;
    const void* planar;
    uint64_t planar_pitch;
    const void* lightmap_uv;
    uint64_t lightmap_uv_pitch;
    const hl_rc_cascade* rc;
    const hl_reflection_env* env; /* NULL: the pass's black fallback cube, no captures */
} hl_reflection_inputs;

/* The indirect specular of fs_reflection (deferred_lighting.wgsl:1265-1341), added to
 * `radiance` as the pass's additive second draw does (colour One + One, alpha kept;
 * deferred-light/src/lib.rs:448-489): for every pixel with depth < 1,
 *   spec = env (F0 env_brdf.x + env_brdf.y)      when enable_env_reflections, else 0
 *          with env = sample_reflection_environment(P, R, 8 roughness) (:646-694): the
 *          captures covering P blended front to back by capture_weight, each sampled
 *          along its sphere or box parallax direction times its brightness, the
 *          skylight (layer 0, along R) filling the remaining coverage; 0 when
 *          enable_reflections == 0 or inputs->env is NULL (the black fallback cube,
 *          lib.rs:542); env_brdf = env_brdf_approx(NdV, roughness) (pbr_eval.wgsl:70-76)
 *   spec = mix(spec, ssr.rgb F_ibl, ssr.a)       when enable_reflections and ssr.a > 0
 *   spec = mix(spec, planar.rgb F_ibl, planar.a) when enable_reflections and planar.a > 0
 *   spec = mix(spec, rc_specular, smoothstep(0.6, 0.9, r) 0.4)  when has_rc_gi, r > 0.6
 *   radiance.rgb += lightmapped ? spec : spec * ao
 * with F_ibl = fresnel_schlick_roughness(NdV, F0, roughness), R = reflect(-V, N) and
 * rc_specular the probe irradiance along normalize(mix(R, N, 0.5 roughness))
 * (sample_rc_specular, :928-980) and ao = the G-buffer's ao (the SSAO fallback is white).
 * Debug modes 30 / 31 replace the pixel with (ssr.a, ssr.a, ssr.a, 1) / (ssr.rgb, 1), the
 * pass's replacement pipeline (lib.rs:1188-1193); modes 1, 2, 4, 5, 10, 11, 20, 21 add
 * nothing. has_rc_gi != 0 with roughness > 0.6 and no probes bound is reported through
 * hl_sync_status as HL_ERR_NOT_SUPPORTED. Replaces the fs_reflection draw of
 * DeferredLightPass::execute (lib.rs:1188-1197). */
hl_status hl_shade_reflections(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                               const hl_reflection_inputs* inputs, const hl_target* radiance, void* stream);

/* Per-pixel pair statistics of the same shading pass, for FLOP accounting: for every
 * pixel (x,y), counts[(y*W+x)*3 + {0,1,2}] = lights listed for the pixel, lights in
 * range (the reference's light-loop test, deferred_lighting.wgsl:1128-1131), and full
 * BRDF evaluations (past the NdL == 0 and radiance < 0.002 cuts, :778-781). Sky pixels
 * get zeros. No reference counterpart. */
hl_status hl_shade_stats(hl_ctx* ctx, const void* camera, const void* globals, const hl_gbuffer* gbuffer,
                         const void* lights, uint32_t n_lights, const hl_light_grid* grid,
                         uint32_t* counts, void* stream);

/* Records which (pixel, light) pairs the context's later shading launches (hl_shade,
 * hl_shade_shadowed, hl_shade_ex) light, i.e. pass the range, NdL and radiance cuts of
 * pbr_direct_light (deferred_lighting.wgsl:725,779,781) and are added to the pixel. The
 * launches are the ordinary ones; only this record is added. For every lit pair the
 * kernel increments *count and, when the previous value k < capacity, writes
 * pairs[2k] = y*width + x and pairs[2k+1] = the light index, in no particular order.
 * pairs and count are device memory the caller owns and zeroes; pairs == NULL stops
 * recording. A verifier re-evaluates the FP64 reference formula with these branch
 * decisions, so that pixels whose f32 and f64 evaluations fall on different sides of a
 * cut are checked rather than skipped. No reference counterpart. */
hl_status hl_set_pair_log(hl_ctx* ctx, uint32_t* pairs, uint32_t capacity, uint32_t* count);

/* ---------------------------------------------------------------------------------
 * Adjoint of the direct-lighting term (no reference counterpart)
 * -------------------------------------------------------------------------------*/

#define HL_ADJOINT_MAX_LIGHTS 65536u

/* Given dL/d(radiance) for every pixel (RGBA32F with pitch d_radiance_pitch bytes,
 * alpha ignored), returns
 *   d_lights[n_lights*7] (f64): d/d position.xyz, d/d intensity, d/d color.rgb
 *   d_pixels[H][W][5]    (f32, dense): d/d albedo.rgb, d/d roughness, d/d metallic
 * for the radiance hl_shade computes with the same G-buffer (any layout; the pair terms
 * are evaluated on the precise path) and light grid (tiles or froxels). The albedo
 * gradient includes the hemisphere ambient term. BRDF terms are recomputed, not stored.
 * Light gradients are reduced per block in f32 and across blocks in f64 in a fixed
 * order, so results are deterministic. The branch decisions (range, NdL == 0,
 * radiance < 0.002, clamps) are held fixed. d_lights and d_pixels are overwritten;
 * sky pixels get zeros. Requires debug_mode == 0 and has_rc_gi == 0 in the globals
 * (else hl_sync_status reports HL_ERR_NOT_SUPPORTED) and n_lights <=
 * HL_ADJOINT_MAX_LIGHTS. Scratch: (#SMs x resident blocks) x n_lights x 32 bytes,
 * grown in the context. */
hl_status hl_shade_adjoint(hl_ctx* ctx, const void* camera, const void* globals,
                           const hl_gbuffer* gbuffer, const void* lights, uint32_t n_lights,
                           const hl_light_grid* grid, const float* d_radiance,
                           uint64_t d_radiance_pitch, double* d_lights, float* d_pixels,
                           void* stream);

/* ---------------------------------------------------------------------------------
 * Fragment lighting: the other consumers of the light lists
 * -------------------------------------------------------------------------------*/

/* One fragment to light, 80 bytes, records 16-byte aligned. */
typedef struct hl_fragment {
    float position[3]; /* world position                                           */
    uint32_t pixel;    /* x | (y << 16): its pixel, for the tile or froxel lookup   */
    float normal[3];   /* world normal (normalised by the kernel)                  */
    float alpha;
    float albedo[3];
    float roughness;
    float f0[3];       /* specular F0 as the material resolved it (not clamped)     */
    float metallic;
    float emissive[3]; /* forward: emissive; transparent: the surface colour        */
    float ao;
} hl_fragment;

#define HL_FRAGMENTS_FORWARD 0u     /* forward_lit.wgsl:443-494 (Forward+)          */
#define HL_FRAGMENTS_TRANSPARENT 1u /* transparent_base.wgsl:181-220                */

typedef struct hl_fragment_params {
    uint32_t mode;            /* HL_FRAGMENTS_*                                        */
    uint32_t num_tiles_x;     /* tile grid: tiles per row (the pass globals' value)    */
    float ambient_intensity;  /* forward: globals.ambient_intensity                    */
    float ambient_color[3];   /* forward: globals.ambient_color.rgb                    */
} hl_fragment_params;

/* Size of the scene's Transform record (position[3], rotation[3] in degrees as
 * pitch x / yaw y / roll z, scale[3]; forward_lit.wgsl:118-122). */
#define HL_SIZEOF_TRANSFORM 36u

/* Lights `n_fragments` fragments from the tile or froxel lists of `grid` and writes
 * out_rgba[i] (RGBA32F) for fragment i:
 *   HL_FRAGMENTS_FORWARD      Lo + ambient_color * ambient_intensity * albedo * ao
 *                             + emissive, alpha; fragments with alpha <= 0.001 are
 *                             discarded (their output untouched); no 0.002 radiance
 *                             cut. With light_entity_indices, light i's position and
 *                             direction come from transforms[light_entity_indices[i]]
 *                             (direction = rotation applied to -Z, Euler order Y X Z),
 *                             as the Forward+ pass reads them; otherwise from the
 *                             GpuLight records.
 *   HL_FRAGMENTS_TRANSPARENT  emissive (the surface colour) + Lo, alpha; lights from
 *                             the GpuLight records; the 0.002 radiance cut applies.
 * Lo sums pbr_direct_light over the fragment's list in list order, skipping lights out
 * of range. A tile grid takes the tile (y/16) * num_tiles_x + x/16 of the pixel; a froxel
 * grid the pixel's column and the slice of the view depth -(view * position).z.
 * Entity indices >= n_transforms and list entries >= n_lights are skipped and
 * reported through hl_sync_status (HL_ERR_DEVICE_BOUNDS). No reference counterpart
 * as one call: it replaces the light loops of the two fragment shaders named above. */
hl_status hl_shade_fragments(hl_ctx* ctx, const void* camera, const hl_fragment_params* params,
                             const void* fragments, uint32_t n_fragments, const void* lights,
                             uint32_t n_lights, const uint32_t* light_entity_indices,
                             const void* transforms, uint32_t n_transforms,
                             const hl_light_grid* grid, float* out_rgba, void* stream);

/* ---------------------------------------------------------------------------------
 * G-buffer write — the fragment stage of the reference's GBufferPass
 * -------------------------------------------------------------------------------*/

#define HL_SIZEOF_GBUFFER_GLOBALS 96u    /* GBufferGlobals, helio-pass-gbuffer/src/lib.rs:43-56 */
#define HL_SIZEOF_MATERIAL_TEXTURES 352u /* GpuMaterialTextures, helio/src/material.rs:178-187  */
#define HL_MAX_MATERIAL_TEXTURES 256u    /* libhelio/src/material.rs:12                         */
#define HL_NO_TEXTURE 0xFFFFFFFFu        /* GpuMaterial::NO_TEXTURE                             */
#define HL_NO_FRAGMENT 0xFFFFFFFFu       /* hl_surface.material_id of a pixel nothing covers    */

/* The interpolated vertex outputs gbuffer.wgsl's fs_main reads for one pixel
 * (VertexOutput, gbuffer.wgsl:147-157), 64 bytes, records 16-byte aligned, one per
 * pixel in row-major order (row pitch = `surfaces_pitch` bytes). */
typedef struct hl_surface {
    float world_normal[3];   /* interpolated, not normalised                          */
    float bitangent_sign;
    float world_tangent[3];  /* interpolated, not normalised                          */
    uint32_t material_id;    /* index into materials; HL_NO_FRAGMENT: pixel untouched */
    float tex_coords[2];     /* UV0                                                   */
    float lightmap_uv[2];    /* already mapped into the atlas, or (-1,-1)             */
    float prev_clip[4];      /* previous frame's clip position (velocity)             */
} hl_surface;

#define HL_TEX_RGBA8_UNORM 0u
#define HL_TEX_RGBA8_SRGB 1u /* decoded to linear per texel before filtering */
#define HL_TEX_RGBA16F 2u
#define HL_TEX_RGBA32F 3u
#define HL_ADDRESS_REPEAT 0u
#define HL_ADDRESS_CLAMP_TO_EDGE 1u
#define HL_ADDRESS_MIRROR_REPEAT 2u
#define HL_FILTER_NEAREST 0u
#define HL_FILTER_LINEAR 1u

/* One entry of the material texture table: a texture's level 0 and its sampler
 * (helio/src/material.rs:11-31 TextureSamplerDesc, :34-41 TextureUpload). */
typedef struct hl_texture {
    const void* texels;     /* device, row-major, aligned to the texel size        */
    uint64_t pitch;         /* row pitch in bytes                                  */
    uint32_t width, height; /* 1..16384                                            */
    uint32_t format;        /* HL_TEX_*                                            */
    uint32_t address_u;     /* HL_ADDRESS_*                                        */
    uint32_t address_v;
    uint32_t filter;        /* HL_FILTER_*: magnification and minification filter  */
} hl_texture;

/* The G-buffer targets the pass writes (helio-pass-gbuffer/src/lib.rs:236-282).
 * planes 0-3 are required, 4-7 optional (NULL: not written):
 *   0 albedo RGBA8 unorm   1 normal RGBA16F   2 orm RGBA8 unorm   3 emissive RGBA16F
 *   4 lightmap_uv RG16F    5 sss RGBA16F      6 extra RGBA16F     7 velocity RG16F
 * Planes 0-3 with the caller's depth plane form an HL_GBUF_REFERENCE G-buffer. */
#define HL_GBUFFER_TARGETS 8
typedef struct hl_gbuffer_targets {
    uint32_t width, height;
    uint32_t reserved[2];
    void* planes[HL_GBUFFER_TARGETS];     /* device */
    uint64_t pitch[HL_GBUFFER_TARGETS];   /* row pitch in bytes */
} hl_gbuffer_targets;

/* Writes the G-buffer of every covered pixel as fs_main of gbuffer.wgsl:425-497 does
 * under the default PBR template (default_pbr_surface, :333-364; resolve_specular_f0,
 * :308-329; select_uv / sample_texture, :287-306; compute_velocity, :417-423):
 *   albedo   = (material.base_color * base_colour sample).rgb, alpha
 *   normal   = (N, F0.r)   N = normalize(world_normal), normal-mapped when the
 *                          material has FLAG_HAS_NORMAL_MAP (1<<3) and a normal texture
 *   orm      = (ao, roughness, metallic, F0.g)    emissive = (emissive, F0.b)
 *   lightmap_uv passed through; sss = 0; extra = 0 (the default template's values);
 *   velocity = (x+0.5, y+0.5) - previous pixel position from prev_clip.
 * Pixels whose alpha <= 0.001 or below the material's alpha cutoff are discarded (all
 * targets untouched), as are pixels with material_id == HL_NO_FRAGMENT. globals'
 * debug_mode 1 (UVs), 2 (base texture) and 3 (geometry normals) write the debug
 * outputs of :443-489. Textures are sampled at level 0 (the level a magnified or 1:1
 * texel footprint selects); bilinear weights are exact in f32. Colour targets clamp to
 * [0,1] and round to nearest (RGBA8), or round to nearest even (RGBA16F).
 *   globals           : device GBufferGlobals (96 B; debug_mode at byte 80)
 *   surfaces          : device hl_surface[height rows of surfaces_pitch bytes]
 *   materials         : device GpuMaterial[n_materials] (96 B each)
 *   material_textures : device GpuMaterialTextures[n_materials] (352 B each)
 *   textures          : HOST array of n_textures <= HL_MAX_MATERIAL_TEXTURES entries;
 *                       slots index it by texture_index
 * A material_id >= n_materials (pixel untouched) or a texture_index >= n_textures (the
 * slot's fallback value used) is reported through hl_sync_status as
 * HL_ERR_DEVICE_BOUNDS. Replaces: GBufferPass's fragment stage (gbuffer.wgsl:425-497;
 * the rasteriser that produces the surfaces and the depth stays the caller's). */
hl_status hl_write_gbuffer(hl_ctx* ctx, const void* globals, const hl_surface* surfaces,
                           uint64_t surfaces_pitch, const void* materials,
                           const void* material_textures, uint32_t n_materials,
                           const hl_texture* textures, uint32_t n_textures,
                           const hl_gbuffer_targets* targets, void* stream);

/* ---------------------------------------------------------------------------------
 * Batched views (no reference counterpart)
 * -------------------------------------------------------------------------------*/

typedef struct hl_view {
    const void* camera; /* device GpuCameraUniforms */
    hl_gbuffer gbuffer;
    hl_target radiance;
} hl_view;

typedef struct hl_batch_config {
    uint32_t autotune;        /* 1: time candidate froxel/tile shapes and keep the fastest */
    uint32_t grid_x, grid_y;  /* used when autotune == 0: froxel grid for every view        */
    uint32_t grid_z;
    const char* cache_path;   /* optional autotuner cache file (read and written), or NULL  */
} hl_batch_config;

typedef struct hl_batch_plan hl_batch_plan;

/* Builds a plan that lights all views with one shared light list: one batched froxel
 * binning launch over every view and one persistent shading launch over a
 * (view, tile) work list, captured together in a CUDA graph. View buffers and the
 * light buffer are baked into the plan; change them by building a new plan. */
hl_status hl_batch_plan_create(hl_ctx* ctx, const hl_view* views, uint32_t n_views,
                               const void* lights, uint32_t n_lights, const void* globals,
                               const hl_batch_config* config, hl_batch_plan** out_plan,
                               void* stream);

/* Replays the plan's graph on `stream`. */
hl_status hl_batch_execute(hl_ctx* ctx, hl_batch_plan* plan, void* stream);

/* Chosen froxel grid of the plan for one view (after autotuning). */
hl_status hl_batch_plan_view_grid(const hl_batch_plan* plan, uint32_t view, uint32_t* grid_xyz);

hl_status hl_batch_plan_destroy(hl_batch_plan* plan);

/* ---------------------------------------------------------------------------------
 * Diagnostics (no reference counterpart)
 * -------------------------------------------------------------------------------*/

/* Measurement only, not part of the rendering interface: measures the device's FP32
 * FMA throughput with a register-resident FFMA loop (best of 5 timed launches), the
 * denominator of the FP32 roofline a benchmark reports. Synchronous; occupies the whole
 * GPU for a few milliseconds, so never call it from a frame. */
hl_status hl_probe_fp32_peak(hl_ctx* ctx, double* tflops);

#ifdef __cplusplus
}
#endif

#endif /* HELIO_GB300_H */
