"""Known-answer tests of the shadow term of the oracle (oracle/shadow_factor.h, the
checker of hl_shade_shadowed): fully lit and fully occluded atlases, lights that cast
no shadow, and layer indices beyond the atlas. CPU only."""
import numpy as np

import oracle
from helio_gb300 import layouts as L
from helio_gb300 import synthetic as S

from scenes import point_light


def _scene(W=96, H=64, layout=S.LAYOUT_F32):
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, layout, seed=21)
    lt = point_light((0.0, 0.0, -12.0), 40.0, intensity=4.0)
    tx, _ = L.tile_grid(W, H)
    glb = L.make_globals(tx, 1, ambient_color=(0.3, 0.3, 0.3), ambient_intensity=0.5)
    lists, counts = oracle.bin_tiles_ref(cam.record, lt, W, H)
    return cam, gb, lt, glb, ("tiles", lists, counts)


def _shadows(sc, fill, size=64):
    n = len(sc.kinds)
    atlas = np.full((n, size, size), fill, np.float32)
    return dict(dynamic=atlas, static=atlas.copy(), matrices=sc.matrices, config=sc.config,
                max_lights=sc.max_lights)


def test_lit_atlas_leaves_radiance_unchanged():
    cam, gb, lt, glb, grid = _scene()
    sc = S.shadow_scene(cam, lt, 1)
    plain = oracle.shade(cam.record, glb, gb, sc.lights, grid)
    shad, _, bounds = oracle.shade_shadowed(cam.record, glb, gb, sc.lights, grid, _shadows(sc, 1.0))
    assert not bounds
    np.testing.assert_array_equal(shad, plain)


def test_occluded_atlas_removes_the_light():
    cam, gb, lt, glb, grid = _scene()
    sc = S.shadow_scene(cam, lt, 1)
    shad, _, _ = oracle.shade_shadowed(cam.record, glb, gb, sc.lights, grid, _shadows(sc, 0.0))
    ambient_only = oracle.shade(cam.record, glb, gb, sc.lights[:0], grid)
    plain = oracle.shade(cam.record, glb, gb, sc.lights, grid)
    sky = np.isnan(plain[..., 0])
    assert (plain[~sky] != ambient_only[~sky]).any()  # the light does light the scene
    np.testing.assert_allclose(shad[~sky], ambient_only[~sky], rtol=1e-12, atol=0)


def test_lights_that_cast_no_shadow():
    cam, gb, lt, glb, grid = _scene()
    sc = S.shadow_scene(cam, lt, 1)
    plain = oracle.shade(cam.record, glb, gb, sc.lights, grid)
    sh = _shadows(sc, 0.0)
    sh["max_lights"] = 0  # light index >= MAX_SHADOW_LIGHTS
    np.testing.assert_array_equal(oracle.shade_shadowed(cam.record, glb, gb, sc.lights, grid, sh)[0], plain)
    lt2 = sc.lights.copy()
    lt2["shadow_index"] = L.NO_SHADOW
    np.testing.assert_array_equal(oracle.shade_shadowed(cam.record, glb, gb, lt2, grid, _shadows(sc, 0.0))[0],
                                  oracle.shade(cam.record, glb, gb, lt2, grid))


def test_layer_beyond_the_atlas_is_lit_and_reported():
    cam, gb, lt, glb, grid = _scene()
    sc = S.shadow_scene(cam, lt, 1)
    lt2 = sc.lights.copy()
    lt2["shadow_index"] = 600
    shad, _, bounds = oracle.shade_shadowed(cam.record, glb, gb, lt2, grid, _shadows(sc, 0.0))
    assert bounds
    np.testing.assert_array_equal(shad, oracle.shade(cam.record, glb, gb, lt2, grid))


def test_partial_occlusion_is_between():
    cam, gb, lt, glb, grid = _scene()
    sc = S.shadow_scene(cam, lt, 1)
    dyn, sta = S.shadow_atlases(sc.kinds, 64, seed=3)
    sh = dict(dynamic=dyn, static=sta, matrices=sc.matrices, config=sc.config, max_lights=sc.max_lights)
    shad, _, _ = oracle.shade_shadowed(cam.record, glb, gb, sc.lights, grid, sh)
    lit = oracle.shade(cam.record, glb, gb, sc.lights, grid)
    dark = oracle.shade(cam.record, glb, gb, sc.lights[:0], grid)
    sky = np.isnan(lit[..., 0])
    s, l, d = shad[~sky][:, :3], lit[~sky][:, :3], dark[~sky][:, :3]
    assert np.all(s <= l * (1 + 1e-12)) and np.all(s >= d * (1 - 1e-12))
    frac = ((s < l * (1 - 1e-9)) & (s > d * (1 + 1e-9))).any(-1).mean()
    assert frac > 0.05, frac  # filtered penumbrae exist


# ---- radiance-cascade GI (oracle/rc_gi.h) ----

def test_rc_with_zero_probes_is_the_hemisphere():
    cam, gb, lt, glb, grid = _scene()
    g = S.rc_globals(glb, (-60, -40, -110), (60, 40, 0))
    zero = np.zeros((1024, 64, 4), np.float16)
    rc, _, _ = oracle.shade_ex(cam.record, g, gb, lt, grid, rc=zero)
    np.testing.assert_array_equal(rc, oracle.shade(cam.record, glb, gb, lt, grid))
    g0 = g.copy()
    g0["has_rc_gi"] = 0  # probes bound but GI off
    np.testing.assert_array_equal(oracle.shade_ex(cam.record, g0, gb, lt, grid, rc=S.rc_probes(1))[0],
                                  oracle.shade(cam.record, glb, gb, lt, grid))


def test_rc_with_uniform_probes_inside_the_volume():
    """Uniform probes c with |c| >= 1/4: the ambient term is kD_ibl c albedo (RC weight 1)
    wherever the volume weight is 1; checked against a numpy evaluation, no lights."""
    cam, gb, lt, glb, grid = _scene(W=64, H=48)
    g = S.rc_globals(glb, (-500, -500, -500), (500, 500, 500))
    c = np.array([0.3, 0.5, 0.2])
    probes = np.zeros((1024, 64, 4), np.float16)
    probes[..., :3] = c.astype(np.float16)
    c = probes[0, 0, :3].astype(np.float64)
    got, _, _ = oracle.shade_ex(cam.record, g, gb, lt[:0], grid, rc=probes)
    W, H = gb.width, gb.height
    a = gb.planes[0].astype(np.float64)
    n = gb.planes[1].astype(np.float64)
    depth = gb.planes[2].astype(np.float64)
    inv = np.array(cam.record["inv_view_proj"][0], np.float64).reshape(4, 4).T
    for (x, y) in ((5, 7), (30, 20), (60, 44)):
        ndc = np.array([(x + 0.5) / W * 2 - 1, 1 - (y + 0.5) / H * 2, depth[y, x], 1.0])
        h = inv @ ndc
        P = h[:3] / h[3]
        N = n[y, x, :3] / np.linalg.norm(n[y, x, :3])
        V = cam.eye - P
        V /= np.linalg.norm(V)
        ndv = max(N @ V, 0.0)
        rough, metal, alb = a[y, x, 3], n[y, x, 3], a[y, x, :3]
        f0 = np.clip(0.04 * (1 - metal) + alb * metal, 0, 0.999)
        F = f0 + (np.maximum(1 - rough, f0) - f0) * (1 - ndv) ** 5
        want = (1 - F) * (1 - metal) * c * alb
        np.testing.assert_allclose(got[y, x, :3], want, rtol=1e-9)
