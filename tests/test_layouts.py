"""Byte layouts and constants at the C-ABI boundary, pinned to the reference.

The reference's own tests for this path are layout and constant checks only
(helio-pass-deferred-light/tests/layout_tests.rs, globals_tests.rs; light.rs:111,115
const-asserts). These restate them against this project's dtypes and header."""
import re
from pathlib import Path

import numpy as np

from helio_gb300 import layouts as L

ROOT = Path(__file__).resolve().parent.parent
HEADER = (ROOT / "include" / "helio_gb300.h").read_text()


def off(dt, name):
    return dt.fields[name][1]


def test_gpu_light_layout():
    # light.rs:60-115, const-asserts at :111 (size 128) and :115 (multiple of 16)
    assert L.GPU_LIGHT.itemsize == 128 and L.GPU_LIGHT.itemsize % 16 == 0
    expect = {"position_range": 0, "direction_outer": 16, "color_intensity": 32, "shadow_index": 48,
              "light_type": 52, "inner_angle": 56, "_pad": 60, "god_rays_enabled": 64, "flare_enabled": 84,
              "flare_tint": 100, "ies_profile_index": 112, "light_function_index": 116, "ies_angle_scale": 120,
              "ies_angle_offset": 124}
    for k, v in expect.items():
        assert off(L.GPU_LIGHT, k) == v, k


def test_gpu_light_default_matches_reference():
    d = L.default_light()[0]
    assert d["shadow_index"] == 0xFFFFFFFF and d["light_type"] == L.LIGHT_POINT
    assert d["ies_profile_index"] == -1 and d["light_function_index"] == -1
    assert tuple(d["direction_outer"]) == (0.0, -1.0, 0.0, 0.0)


def test_camera_layout():
    assert L.GPU_CAMERA.itemsize == 368
    expect = {"view": 0, "proj": 64, "view_proj": 128, "inv_view_proj": 192, "position_near": 256,
              "forward_far": 272, "jitter_frame": 288, "prev_view_proj": 304}
    for k, v in expect.items():
        assert off(L.GPU_CAMERA, k) == v, k
    # proj[0][0] and proj[1][1] are floats 16 and 21 of the struct (column major)
    assert (off(L.GPU_CAMERA, "proj") + 0 * 4) // 4 == 16 and (off(L.GPU_CAMERA, "proj") + 5 * 4) // 4 == 21


def test_deferred_globals_layout():
    # deferred-light/src/lib.rs:17-52 is 112 bytes; layout_tests.rs:71 asserts a stale 96
    assert L.DEFERRED_GLOBALS.itemsize == 112
    assert L.DEFERRED_GLOBALS.itemsize % 16 == 0
    expect = {"frame": 0, "delta_time": 4, "light_count": 8, "ambient_intensity": 12, "ambient_color": 16,
              "rc_world_min": 32, "rc_world_max": 48, "csm_splits": 64, "debug_mode": 80, "has_rc_gi": 84,
              "num_tiles_x": 88, "reflection_capture_count": 92, "enable_reflections": 96,
              "enable_env_reflections": 100, "_pad": 104}
    for k, v in expect.items():
        assert off(L.DEFERRED_GLOBALS, k) == v, k


def test_light_cull_params_and_material():
    assert L.LIGHT_CULL_PARAMS.itemsize == 32
    assert L.GPU_MATERIAL.itemsize == 96
    assert off(L.GPU_MATERIAL, "class_params") == 80


def test_csm_splits_ascending():
    s = list(L.CSM_SPLITS)
    assert s == sorted(s) and len(s) == 4


def test_header_constants_match():
    def define(name):
        return re.search(rf"#define {name} \(?(-?[0-9.]+)", HEADER).group(1)

    assert int(define("HL_TILE_SIZE").rstrip("u")) == L.TILE_SIZE == 16
    assert int(define("HL_MAX_LIGHTS_PER_TILE").rstrip("u")) == L.MAX_LIGHTS_PER_TILE == 64
    assert float(define("HL_FROXEL_NEAR").rstrip("f")) == L.FROXEL_NEAR
    assert int(define("HL_SIZEOF_GPU_LIGHT").rstrip("u")) == 128
    assert int(define("HL_SIZEOF_GPU_CAMERA").rstrip("u")) == 368
    assert int(define("HL_SIZEOF_DEFERRED_GLOBALS").rstrip("u")) == 112


def test_tile_grid():
    assert L.tile_grid(1920, 1080) == (120, 68)
    assert L.tile_grid(1280, 720) == (80, 45)
    assert L.tile_grid(3840, 2160) == (240, 135)
    assert L.tile_grid(1, 1) == (1, 1)


def test_globals_fallback_fields():
    g = L.make_globals(120, 1024)[0]
    assert g["has_rc_gi"] == 0 and g["num_tiles_x"] == 120 and g["light_count"] == 1024
    assert np.allclose(g["csm_splits"], L.CSM_SPLITS)
