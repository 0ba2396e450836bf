"""Known-answer tests of the G-buffer pass oracle (oracle/gbuffer_write.cpp), the
checker of hl_write_gbuffer: closed-form values of gbuffer.wgsl's fs_main
(default_pbr_surface, resolve_specular_f0, select_uv, the debug modes, the alpha
discard) and of level-0 texture sampling (texel centres, repeat / clamp-to-edge /
mirrored-repeat, nearest / linear, sRGB decode). CPU only."""
import math

import numpy as np
import pytest

import oracle
from helio_gb300 import layouts as L


def _scene(n=1, debug=0):
    glb = np.zeros(1, L.GBUFFER_GLOBALS)
    glb["debug_mode"] = debug
    glb["screen_width"], glb["screen_height"] = n, 1
    mats = np.zeros(1, L.GPU_MATERIAL)
    mats["base_color"] = (0.6, 0.4, 0.2, 1.0)
    mats["emissive"] = (0.5, 0.25, 1.0, 2.0)
    mats["roughness_metallic"] = (0.5, 0.25, 1.5, 0.8)
    for f in ("tex_base_color", "tex_normal", "tex_roughness", "tex_emissive", "tex_occlusion"):
        mats[f] = L.NO_TEXTURE
    mtex = L.missing_material_textures(1)
    srf = np.zeros((1, n), L.SURFACE)
    srf["world_normal"] = (0.0, 2.0, 0.0)
    srf["world_tangent"] = (1.0, 0.0, 0.0)
    srf["bitangent_sign"] = 1.0
    srf["material_id"] = 0
    srf["tex_coords"] = (0.25, 0.75)
    srf["lightmap_uv"] = (-1.0, -1.0)
    srf["prev_clip"] = (0.0, 0.0, 0.5, 1.0)
    return glb, srf, mats, mtex


def _run(glb, srf, mats, mtex, textures=()):
    return oracle.write_gbuffer(glb, srf, mats, mtex, list(textures))


def test_untextured_metallic_surface():
    glb, srf, mats, mtex = _scene()
    v, wr, bounds = _run(glb, srf, mats, mtex)
    assert wr[0, 0] and not bounds
    o = v[0, 0]
    np.testing.assert_allclose(o[0:4], [0.6, 0.4, 0.2, 1.0], rtol=1e-7)
    np.testing.assert_allclose(o[4:7], [0.0, 1.0, 0.0], atol=1e-15)  # normalize(world_normal)
    m = 0.25
    f0 = [0.04 * (1 - m) + a * m for a in (0.6, 0.4, 0.2)]
    np.testing.assert_allclose([o[7], o[11], o[15]], f0, rtol=1e-7)
    np.testing.assert_allclose(o[8:11], [1.0, 0.5, 0.25], rtol=1e-7)  # ao, roughness, metallic
    np.testing.assert_allclose(o[12:15], [0.5 * 2.0, 0.25 * 2.0, 1.0 * 2.0], rtol=1e-7)
    np.testing.assert_allclose(o[16:18], [-1.0, -1.0])
    # velocity: prev clip at the view centre, pixel (0,0) of a 1x1 target -> (0.5,0.5)-(0.5,0.5)
    np.testing.assert_allclose(o[18:20], [0.0, 0.0], atol=1e-12)


def test_roughness_and_metallic_clamps():
    glb, srf, mats, mtex = _scene()
    mats["roughness_metallic"] = (0.01, 3.0, 1.5, 0.8)
    o = _run(glb, srf, mats, mtex)[0][0, 0]
    assert o[9] == pytest.approx(0.045) and o[10] == 1.0
    assert o[7] == pytest.approx(0.6) and o[11] == pytest.approx(0.4)  # F0 = albedo at metallic 1


def test_specular_workflow_f0():
    glb, srf, mats, mtex = _scene()
    mats["workflow"] = L.WORKFLOW_SPECULAR
    mats["roughness_metallic"] = (0.5, 0.0, 1.5, 0.8)
    o = _run(glb, srf, mats, mtex)[0][0, 0]
    f0 = 0.8 * ((1.5 - 1) / (1.5 + 1)) ** 2
    np.testing.assert_allclose([o[7], o[11], o[15]], [f0] * 3, rtol=1e-7)
    mats["roughness_metallic"] = (0.5, 0.0, 0.7, 0.8)  # ior clamped to 1 -> F0 = 0
    o = _run(glb, srf, mats, mtex)[0][0, 0]
    assert o[7] == 0.0 and o[11] == 0.0 and o[15] == 0.0


@pytest.mark.parametrize("alpha,cutoff,written", [(0.4, 0.5, False), (0.4, 0.0, True), (0.0005, 0.0, False),
                                                  (0.5, 0.5, True)])
def test_alpha_discard(alpha, cutoff, written):
    glb, srf, mats, mtex = _scene()
    mats["base_color"] = (0.6, 0.4, 0.2, alpha)
    mtex["params"] = (1.0, 1.0, cutoff, 0.0)
    assert _run(glb, srf, mats, mtex)[1][0, 0] == written


def test_uncovered_and_out_of_range_material():
    glb, srf, mats, mtex = _scene(n=2)
    srf["material_id"] = (L.NO_FRAGMENT, 5)
    v, wr, bounds = _run(glb, srf, mats, mtex)
    assert not wr.any() and bounds


def _tex(texels, fmt=L.TEX_RGBA8_UNORM, au=L.ADDRESS_REPEAT, av=L.ADDRESS_REPEAT, filt=L.FILTER_LINEAR):
    return (np.ascontiguousarray(texels), fmt, au, av, filt)


def _sample(tex, uvs, rotation=0.0, offset=(0.0, 0.0), scale=(1.0, 1.0)):
    """Base-colour samples of ``tex`` at ``uvs`` (white material, no cutoff)."""
    glb, srf, mats, mtex = _scene(n=len(uvs))
    mats["base_color"] = (1.0, 1.0, 1.0, 1.0)
    mtex["params"] = (1.0, 1.0, 0.0, 0.0)
    s = mtex["base_color"][0]
    s["texture_index"] = 0
    s["offset_scale"] = (*offset, *scale)
    s["rotation"] = (math.sin(rotation), math.cos(rotation), 0.0, 0.0)
    mtex["base_color"][0] = s
    srf["tex_coords"][0] = np.asarray(uvs, np.float32)
    v, wr, _ = _run(glb, srf, mats, mtex, [tex])
    assert wr.all()
    return v[0, :, 0:4]


def _ramp(w=4, h=2):
    t = np.zeros((h, w, 4), np.uint8)
    for y in range(h):
        for x in range(w):
            t[y, x] = (10 + 40 * x, 20 + 100 * y, 7 * (x + y), 255)
    return t


def test_linear_sampling_at_texel_centres_returns_the_texel():
    t = _ramp()
    uvs = [((x + 0.5) / 4, (y + 0.5) / 2) for y in range(2) for x in range(4)]
    got = _sample(_tex(t), uvs)
    want = np.array([t[y, x] for y in range(2) for x in range(4)], np.float64) / 255.0
    np.testing.assert_allclose(got, want, rtol=1e-12)


def test_linear_sampling_midway_blends_neighbours():
    t = _ramp()
    got = _sample(_tex(t), [(1.0 / 4, 0.25)])  # halfway between texels 0 and 1 of row 0
    np.testing.assert_allclose(got[0], (t[0, 0].astype(float) + t[0, 1]) / 2 / 255.0, rtol=1e-12)


def test_address_modes():
    t = _ramp()
    u0 = 1.5 / 4
    rep = _sample(_tex(t, au=L.ADDRESS_REPEAT), [(u0, 0.25), (u0 + 1, 0.25), (u0 - 3, 0.25)])
    np.testing.assert_allclose(rep[1], rep[0], rtol=1e-12)
    np.testing.assert_allclose(rep[2], rep[0], rtol=1e-12)
    mir = _sample(_tex(t, au=L.ADDRESS_MIRROR_REPEAT), [(u0, 0.25), (-u0, 0.25), (2 - u0, 0.25)])
    np.testing.assert_allclose(mir[1], mir[0], rtol=1e-12)
    np.testing.assert_allclose(mir[2], mir[0], rtol=1e-12)
    clm = _sample(_tex(t, au=L.ADDRESS_CLAMP_TO_EDGE), [(-5.0, 0.25), (7.0, 0.25)])
    np.testing.assert_allclose(clm[0], t[0, 0] / 255.0, rtol=1e-12)
    np.testing.assert_allclose(clm[1], t[0, 3] / 255.0, rtol=1e-12)


def test_nearest_filter_picks_the_covering_texel():
    t = _ramp()
    got = _sample(_tex(t, filt=L.FILTER_NEAREST), [(0.26, 0.1), (0.49, 0.9)])
    np.testing.assert_allclose(got[0], t[0, 1] / 255.0, rtol=1e-12)
    np.testing.assert_allclose(got[1], t[1, 1] / 255.0, rtol=1e-12)


def test_srgb_decode():
    t = np.zeros((1, 4, 4), np.uint8)
    t[0, :, 0] = (0, 10, 128, 255)
    t[0, :, 3] = 255
    got = _sample(_tex(t, fmt=L.TEX_RGBA8_SRGB, filt=L.FILTER_NEAREST), [((x + 0.5) / 4, 0.5) for x in range(4)])
    c = 128 / 255.0
    np.testing.assert_allclose(got[:, 0], [0.0, 10 / 255.0 / 12.92, ((c + 0.055) / 1.055) ** 2.4, 1.0], rtol=1e-12)
    assert np.all(got[:, 3] == 1.0)  # alpha is linear


def test_select_uv_rotation_offset_scale():
    t = _ramp()
    # rotation by 90 degrees maps (u, v) to (-v, u); then offset
    got = _sample(_tex(t, filt=L.FILTER_NEAREST), [(0.25, 0.125)], rotation=math.pi / 2, offset=(0.5, 0.0))
    # (-0.125 + 0.5, 0.25) -> texel x = floor(0.375 * 4) = 1, y = floor(0.25 * 2) = 0
    np.testing.assert_allclose(got[0], t[0, 1] / 255.0, rtol=1e-12)
    got = _sample(_tex(t, filt=L.FILTER_NEAREST), [(0.3, 0.3)], scale=(2.0, 2.0))  # (0.6, 0.6)
    np.testing.assert_allclose(got[0], t[1, 2] / 255.0, rtol=1e-12)


def test_flat_normal_map_keeps_the_geometry_normal():
    glb, srf, mats, mtex = _scene()
    mats["flags"] = L.FLAG_HAS_NORMAL_MAP
    mtex["normal"]["texture_index"] = 0
    flat = np.zeros((2, 2, 4), np.float32)
    flat[...] = (0.5, 0.5, 1.0, 1.0)
    srf["world_normal"] = (0.3, 0.8, -0.2)
    srf["world_tangent"] = (1.0, 0.2, 0.0)
    v, _, _ = _run(glb, srf, mats, mtex, [_tex(flat, fmt=L.TEX_RGBA32F)])
    n = np.array([0.3, 0.8, -0.2]) / np.linalg.norm([0.3, 0.8, -0.2])
    np.testing.assert_allclose(v[0, 0, 4:7], n, atol=1e-7)


def test_normal_map_tilts_along_the_tangent_frame():
    glb, srf, mats, mtex = _scene()
    mats["flags"] = L.FLAG_HAS_NORMAL_MAP
    mtex["normal"]["texture_index"] = 0
    mtex["params"] = (1.0, 1.0, 0.5, 0.0)
    tilt = np.zeros((1, 1, 4), np.float32)
    tilt[...] = (1.0, 0.5, 0.5, 1.0)  # tangent-space (1, 0, 0)
    srf["world_normal"] = (0.0, 0.0, 1.0)
    srf["world_tangent"] = (1.0, 0.0, 0.5)  # not orthogonal: Gram-Schmidt against N
    v, _, _ = _run(glb, srf, mats, mtex, [_tex(tilt, fmt=L.TEX_RGBA32F)])
    np.testing.assert_allclose(v[0, 0, 4:7], [1.0, 0.0, 0.0], atol=1e-7)


@pytest.mark.parametrize("debug", [1, 2, 3])
def test_debug_modes(debug):
    glb, srf, mats, mtex = _scene(debug=debug)
    mats["base_color"] = (0.6, 0.4, 0.2, 0.1)  # would be discarded outside the debug modes
    v, wr, _ = _run(glb, srf, mats, mtex)
    assert wr[0, 0]
    o = v[0, 0]
    if debug == 1:
        np.testing.assert_allclose(o[0:8], [0.25, 0.75, 0, 1, 0, 0, 1, 0])
    elif debug == 2:
        np.testing.assert_allclose(o[0:8], [1, 1, 1, 1, 0, 0, 1, 0])  # fallback texture value
    else:
        np.testing.assert_allclose(o[0:4], [0.6, 0.4, 0.2, 0.1], rtol=1e-7)
        np.testing.assert_allclose(o[4:12], [0, 1, 0, 0, 1, 0.5, 0.25, 0], atol=1e-7)
    assert np.all(o[12:18] == 0)
