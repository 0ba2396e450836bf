"""Byte layouts of the reference's GPU structs, as numpy structured dtypes.

These are the contracts at the C-ABI boundary. Each dtype has exactly the size and
field offsets of the reference's `#[repr(C)]` Rust struct:

- ``GPU_LIGHT``           libhelio/src/light.rs:60-115 (128 B; const-assert at :111)
- ``GPU_CAMERA``          libhelio/src/camera.rs:12-29 (368 B; column-major matrices
                          from glam ``to_cols_array``, camera.rs:47-54)
- ``DEFERRED_GLOBALS``    helio-pass-deferred-light/src/lib.rs:17-52 (112 B; the
                          96 B in the reference's tests/layout_tests.rs:71 is stale)
- ``LIGHT_CULL_PARAMS``   helio-pass-light-cull/src/lib.rs:26-35 (32 B)
- ``GPU_MATERIAL``        libhelio/src/material.rs:231-254 (96 B)
"""
from __future__ import annotations

import numpy as np

# LightType discriminants (libhelio/src/light.rs:8-13)
LIGHT_DIRECTIONAL = 0
LIGHT_POINT = 1
LIGHT_SPOT = 2
LIGHT_AREA = 3

NO_SHADOW = 0xFFFFFFFF  # shadow_index that disables shadow_factor (deferred_lighting.wgsl:459)

TILE_SIZE = 16  # light_cull.wgsl:17
MAX_LIGHTS_PER_TILE = 64  # light_cull.wgsl:18
FROXEL_NEAR = 0.5  # prelude.wgsl:195

GPU_LIGHT = np.dtype(
    [
        ("position_range", "<f4", (4,)),
        ("direction_outer", "<f4", (4,)),
        ("color_intensity", "<f4", (4,)),
        ("shadow_index", "<u4"),
        ("light_type", "<u4"),
        ("inner_angle", "<f4"),
        ("_pad", "<u4"),
        ("god_rays_enabled", "<u4"),
        ("god_rays_density", "<f4"),
        ("god_rays_weight", "<f4"),
        ("god_rays_decay", "<f4"),
        ("god_rays_exposure", "<f4"),
        ("flare_enabled", "<u4"),
        ("flare_type", "<u4"),
        ("flare_intensity", "<f4"),
        ("flare_scale", "<f4"),
        ("flare_tint", "<f4", (3,)),
        ("ies_profile_index", "<i4"),
        ("light_function_index", "<i4"),
        ("ies_angle_scale", "<f4"),
        ("ies_angle_offset", "<f4"),
    ]
)

GPU_CAMERA = np.dtype(
    [
        ("view", "<f4", (16,)),
        ("proj", "<f4", (16,)),
        ("view_proj", "<f4", (16,)),
        ("inv_view_proj", "<f4", (16,)),
        ("position_near", "<f4", (4,)),
        ("forward_far", "<f4", (4,)),
        ("jitter_frame", "<f4", (4,)),
        ("prev_view_proj", "<f4", (16,)),
    ]
)

DEFERRED_GLOBALS = np.dtype(
    [
        ("frame", "<u4"),
        ("delta_time", "<f4"),
        ("light_count", "<u4"),
        ("ambient_intensity", "<f4"),
        ("ambient_color", "<f4", (4,)),
        ("rc_world_min", "<f4", (4,)),
        ("rc_world_max", "<f4", (4,)),
        ("csm_splits", "<f4", (4,)),
        ("debug_mode", "<u4"),
        ("has_rc_gi", "<u4"),
        ("num_tiles_x", "<u4"),
        ("reflection_capture_count", "<u4"),
        ("enable_reflections", "<u4"),
        ("enable_env_reflections", "<u4"),
        ("_pad", "<u4", (2,)),
    ]
)

LIGHT_CULL_PARAMS = np.dtype(
    [
        ("num_tiles_x", "<u4"),
        ("num_tiles_y", "<u4"),
        ("num_lights", "<u4"),
        ("screen_width", "<u4"),
        ("screen_height", "<u4"),
        ("_pad", "<u4", (3,)),
    ]
)

GPU_MATERIAL = np.dtype(
    [
        ("base_color", "<f4", (4,)),
        ("emissive", "<f4", (4,)),
        ("roughness_metallic", "<f4", (4,)),
        ("tex_base_color", "<u4"),
        ("tex_normal", "<u4"),
        ("tex_roughness", "<u4"),
        ("tex_emissive", "<u4"),
        ("tex_occlusion", "<u4"),
        ("workflow", "<u4"),
        ("flags", "<u4"),
        ("material_class", "<u4"),
        ("class_params", "<f4", (4,)),
    ]
)

FROXEL_PARAMS = np.dtype(
    [
        ("grid_x", "<u4"),
        ("grid_y", "<u4"),
        ("grid_z", "<u4"),
        ("width", "<u4"),
        ("height", "<u4"),
        ("slice_near", "<f4"),
        ("slice_far", "<f4"),
        ("reserved", "<u4"),
    ]
)

# One fragment for hl_shade_fragments (the inputs of the Forward+ and transparent
# fragment shaders' light loops, forward_lit.wgsl:443-494, transparent_base.wgsl:181-220)
FRAGMENT = np.dtype(
    [
        ("position", "<f4", (3,)),
        ("pixel", "<u4"),
        ("normal", "<f4", (3,)),
        ("alpha", "<f4"),
        ("albedo", "<f4", (3,)),
        ("roughness", "<f4"),
        ("f0", "<f4", (3,)),
        ("metallic", "<f4"),
        ("emissive", "<f4", (3,)),
        ("ao", "<f4"),
    ]
)

# The scene's Transform record (forward_lit.wgsl:118-122); rotation in degrees
TRANSFORM = np.dtype([("position", "<f4", (3,)), ("rotation", "<f4", (3,)), ("scale", "<f4", (3,))])

FRAGMENT_PARAMS = np.dtype(
    [
        ("mode", "<u4"),
        ("num_tiles_x", "<u4"),
        ("ambient_intensity", "<f4"),
        ("ambient_color", "<f4", (3,)),
    ]
)
FRAGMENTS_FORWARD, FRAGMENTS_TRANSPARENT = 0, 1

# GBufferGlobals (helio-pass-gbuffer/src/lib.rs:43-56), the uniform of the G-buffer pass
GBUFFER_GLOBALS = np.dtype(
    [
        ("frame", "<u4"),
        ("delta_time", "<f4"),
        ("light_count", "<u4"),
        ("ambient_intensity", "<f4"),
        ("ambient_color", "<f4", (4,)),
        ("rc_world_min", "<f4", (4,)),
        ("rc_world_max", "<f4", (4,)),
        ("csm_splits", "<f4", (4,)),
        ("debug_mode", "<u4"),
        ("screen_width", "<f4"),
        ("screen_height", "<f4"),
        ("_pad0", "<u4"),
    ]
)

# One texture slot of GpuMaterialTextures (helio/src/material.rs:154-162)
MATERIAL_TEXTURE_SLOT = np.dtype(
    [
        ("texture_index", "<u4"),
        ("uv_channel", "<u4"),
        ("_pad", "<u4", (2,)),
        ("offset_scale", "<f4", (4,)),  # offset.xy, scale.xy
        ("rotation", "<f4", (4,)),      # sin, cos, 0, 0
    ]
)

# GpuMaterialTextures (helio/src/material.rs:176-187); params = (normal_scale,
# occlusion_strength, alpha_cutoff, 0)
MATERIAL_TEXTURES = np.dtype(
    [
        ("base_color", MATERIAL_TEXTURE_SLOT),
        ("normal", MATERIAL_TEXTURE_SLOT),
        ("roughness_metallic", MATERIAL_TEXTURE_SLOT),
        ("emissive", MATERIAL_TEXTURE_SLOT),
        ("occlusion", MATERIAL_TEXTURE_SLOT),
        ("specular_color", MATERIAL_TEXTURE_SLOT),
        ("specular_weight", MATERIAL_TEXTURE_SLOT),
        ("params", "<f4", (4,)),
    ]
)
MATERIAL_SLOTS = ("base_color", "normal", "roughness_metallic", "emissive", "occlusion", "specular_color",
                  "specular_weight")
NO_TEXTURE = 0xFFFFFFFF
NO_FRAGMENT = 0xFFFFFFFF
FLAG_HAS_NORMAL_MAP = 1 << 3  # libhelio/src/material.rs:189
WORKFLOW_METALLIC, WORKFLOW_SPECULAR = 0, 1

# hl_surface: the interpolated vertex outputs gbuffer.wgsl's fs_main reads (:147-157)
SURFACE = np.dtype(
    [
        ("world_normal", "<f4", (3,)),
        ("bitangent_sign", "<f4"),
        ("world_tangent", "<f4", (3,)),
        ("material_id", "<u4"),
        ("tex_coords", "<f4", (2,)),
        ("lightmap_uv", "<f4", (2,)),
        ("prev_clip", "<f4", (4,)),
    ]
)

# hl_texture (include/helio_gb300.h): a texture level 0 and its sampler
TEXTURE = np.dtype(
    [
        ("texels", "<u8"),
        ("pitch", "<u8"),
        ("width", "<u4"),
        ("height", "<u4"),
        ("format", "<u4"),
        ("address_u", "<u4"),
        ("address_v", "<u4"),
        ("filter", "<u4"),
    ]
)
TEX_RGBA8_UNORM, TEX_RGBA8_SRGB, TEX_RGBA16F, TEX_RGBA32F = 0, 1, 2, 3
ADDRESS_REPEAT, ADDRESS_CLAMP_TO_EDGE, ADDRESS_MIRROR_REPEAT = 0, 1, 2
FILTER_NEAREST, FILTER_LINEAR = 0, 1


def missing_material_textures(n: int = 1) -> np.ndarray:
    """``n`` GpuMaterialTextures as GpuMaterialTextures::missing() makes them
    (helio/src/material.rs:164-200): no textures, identity transforms, params
    (1, 1, 0.5, 0)."""
    m = np.zeros(n, MATERIAL_TEXTURES)
    for slot in MATERIAL_SLOTS:
        m[slot]["texture_index"] = NO_TEXTURE
        m[slot]["offset_scale"] = (0.0, 0.0, 1.0, 1.0)
        m[slot]["rotation"] = (0.0, 1.0, 0.0, 0.0)
    m["params"] = (1.0, 1.0, 0.5, 0.0)
    return m


# ShadowConfig (libhelio/src/shadow.rs:33-64): four cascades of (split_distance,
# depth_bias, filter_radius, pcss_light_size), then the PCSS toggle and sample counts.
# 80 bytes (the struct's doc comment says 96).
SHADOW_CONFIG = np.dtype(
    [
        ("cascades", "<f4", (4, 4)),
        ("enable_pcss", "<u4"),
        ("pcss_blocker_samples", "<u4"),
        ("pcss_filter_samples", "<u4"),
        ("pcf_sample_count", "<u4"),
    ]
)

# hl_shadow_maps (include/helio_gb300.h)
SHADOW_MAPS = np.dtype(
    [
        ("dynamic_atlas", "<u8"),
        ("static_atlas", "<u8"),
        ("matrices", "<u8"),
        ("config", "<u8"),
        ("size", "<u4"),
        ("layers", "<u4"),
        ("max_shadow_lights", "<u4"),
        ("reserved", "<u4"),
    ]
)
# hl_rc_cascade (include/helio_gb300.h): the radiance-cascade probe texture rc_cascade0
RC_CASCADE = np.dtype([("texels", "<u8"), ("pitch", "<u8"), ("width", "<u4"), ("height", "<u4")])

# GpuReflectionCapture (libhelio/src/reflection.rs:64-80): the captures the reflection
# draw blends (deferred_lighting.wgsl:189-198)
REFLECTION_CAPTURE = np.dtype(
    [
        ("position_radius", "<f4", (4,)),
        ("extents_transition", "<f4", (4,)),
        ("world_to_local", "<f4", (16,)),  # column major
        ("cubemap_index", "<i4"),
        ("shape", "<u4"),  # 0 sphere, 1 box
        ("mobility", "<u4"),
        ("brightness", "<f4"),
    ]
)
CAPTURE_SPHERE, CAPTURE_BOX = 0, 1
# hl_reflection_env: captures and their cube-map array (texels RGBA16F)
REFLECTION_ENV = np.dtype([("captures", "<u8"), ("count", "<u4"), ("face_size", "<u4"), ("mip_levels", "<u4"),
                           ("layers", "<u4"), ("texels", "<u8")])
RC_PROBE_DIM, RC_DIR_DIM = 16, 4  # deferred_lighting.wgsl:824-825

SHADOW_ATLAS_SIZE = 1024  # the shader's ATLAS_SIZE (deferred_lighting.wgsl:235)
MAX_SHADOW_LIGHTS = 42    # MAX_SHADOW_LIGHTS (deferred_lighting.wgsl:20)

# The quality presets of ShadowConfig::from_quality (libhelio/src/shadow.rs:74-205):
# per cascade (split, bias, filter radius, PCSS light size), then (enable_pcss,
# blocker samples, filter samples, PCF samples).
SHADOW_PRESETS = {
    "low": ([(16.0, 0.00010, 1.0, 0.0), (80.0, 0.00015, 1.5, 0.0), (300.0, 0.00020, 2.0, 0.0),
             (1400.0, 0.00030, 3.0, 0.0)], (0, 4, 4, 8)),
    "medium": ([(16.0, 0.00010, 1.5, 0.0), (80.0, 0.00015, 2.0, 0.0), (300.0, 0.00020, 2.5, 0.0),
                (1400.0, 0.00030, 3.5, 0.0)], (0, 8, 8, 12)),
    "high": ([(16.0, 0.00008, 2.0, 2.0), (80.0, 0.00012, 2.5, 4.0), (300.0, 0.00018, 3.0, 8.0),
              (1400.0, 0.00025, 4.0, 16.0)], (1, 8, 16, 12)),
    "ultra": ([(16.0, 0.00008, 2.5, 2.0), (80.0, 0.00012, 3.0, 4.0), (300.0, 0.00018, 3.5, 8.0),
               (1400.0, 0.00025, 4.5, 16.0)], (1, 16, 32, 16)),
}


def shadow_config(quality: str = "medium") -> np.ndarray:
    """A ShadowConfig of one of the reference's presets (default: Medium, the
    reference's Default)."""
    cascades, (pcss, nb, nf, npcf) = SHADOW_PRESETS[quality]
    c = np.zeros(1, SHADOW_CONFIG)
    c["cascades"] = np.array(cascades, np.float32)
    c["enable_pcss"], c["pcss_blocker_samples"], c["pcss_filter_samples"], c["pcf_sample_count"] = pcss, nb, nf, npcf
    return c


# CSM split distances written into DeferredGlobals (libhelio/src/shadow.rs:13)
CSM_SPLITS = (16.0, 80.0, 300.0, 1400.0)

EXPECTED_SIZES = {
    "GPU_LIGHT": 128,
    "GPU_CAMERA": 368,
    "DEFERRED_GLOBALS": 112,
    "LIGHT_CULL_PARAMS": 32,
    "GPU_MATERIAL": 96,
    "FROXEL_PARAMS": 32,
    "FRAGMENT": 80,
    "TRANSFORM": 36,
    "FRAGMENT_PARAMS": 24,
    "GBUFFER_GLOBALS": 96,
    "MATERIAL_TEXTURE_SLOT": 48,
    "MATERIAL_TEXTURES": 352,
    "SURFACE": 64,
    "TEXTURE": 40,
    "SHADOW_CONFIG": 80,
    "SHADOW_MAPS": 48,
    "RC_CASCADE": 24,
    "REFLECTION_CAPTURE": 112,
    "REFLECTION_ENV": 32,
}

for _name, _size in EXPECTED_SIZES.items():
    assert globals()[_name].itemsize == _size, (_name, globals()[_name].itemsize)


def default_light() -> np.ndarray:
    """One ``GpuLight`` with the reference's ``Default`` values (light.rs:117-148):
    a white point light with shadows off and no IES profile or light function."""
    lt = np.zeros(1, GPU_LIGHT)
    lt["direction_outer"] = (0.0, -1.0, 0.0, 0.0)
    lt["color_intensity"] = (1.0, 1.0, 1.0, 1.0)
    lt["shadow_index"] = NO_SHADOW
    lt["light_type"] = LIGHT_POINT
    lt["god_rays_density"] = 1.0
    lt["god_rays_weight"] = 0.6
    lt["god_rays_decay"] = 1.0
    lt["god_rays_exposure"] = 0.7
    lt["flare_intensity"] = 1.0
    lt["flare_scale"] = 1.0
    lt["flare_tint"] = (1.0, 1.0, 1.0)
    lt["ies_profile_index"] = -1
    lt["light_function_index"] = -1
    lt["ies_angle_scale"] = 1.0
    return lt


def make_lights(n: int) -> np.ndarray:
    """``n`` default lights, to be filled by the caller."""
    base = default_light()
    return np.repeat(base, n)


def make_globals(
    num_tiles_x: int,
    light_count: int,
    ambient_color=(0.0, 0.0, 0.0),
    ambient_intensity: float = 0.0,
    debug_mode: int = 0,
) -> np.ndarray:
    """A ``DeferredGlobals`` as DeferredLightPass::prepare fills it
    (deferred-light/src/lib.rs:836-878) under fallback bindings: no RC GI, no
    reflections captures. Ambient defaults to black (the bench's metric case); the
    pass's own fallback is (0.5, 0.5, 0.6) x 1.0."""
    g = np.zeros(1, DEFERRED_GLOBALS)
    g["light_count"] = light_count
    g["ambient_intensity"] = ambient_intensity
    g["ambient_color"] = (*ambient_color, 1.0)
    g["csm_splits"] = CSM_SPLITS
    g["debug_mode"] = debug_mode
    g["has_rc_gi"] = 0
    g["num_tiles_x"] = num_tiles_x
    g["enable_reflections"] = 1
    g["enable_env_reflections"] = 0
    return g


def froxel_params(grid_x, grid_y, grid_z, width, height, slice_far, slice_near=FROXEL_NEAR) -> np.ndarray:
    p = np.zeros(1, FROXEL_PARAMS)
    p["grid_x"], p["grid_y"], p["grid_z"] = grid_x, grid_y, grid_z
    p["width"], p["height"] = width, height
    p["slice_near"], p["slice_far"] = slice_near, slice_far
    return p


def tile_grid(width: int, height: int):
    """(tiles_x, tiles_y) of the reference's 16-pixel tiling (light-cull/src/lib.rs:65-66)."""
    return (width + TILE_SIZE - 1) // TILE_SIZE, (height + TILE_SIZE - 1) // TILE_SIZE
