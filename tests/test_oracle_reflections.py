"""The oracle's reflection draw (fs_reflection, deferred_lighting.wgsl:1265-1341) against
known answers: an independent numpy restatement of the SSR and planar blends, the debug
modes, the switches and the radiance-cascade rough-specular fallback."""
import numpy as np
import pytest

import oracle
from helio_gb300 import layouts as L
from helio_gb300 import synthetic as S

RC_MIN, RC_MAX = (-60.0, -40.0, -110.0), (60.0, 40.0, 0.0)


def _frame(layout=S.LAYOUT_REFERENCE, W=48, H=32, seed=5, **glb_kw):
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, layout, seed=seed)
    tx, _ = L.tile_grid(W, H)
    glb = L.make_globals(tx, 0)
    for k, v in glb_kw.items():
        glb[k] = v
    base = np.random.default_rng(seed).uniform(0.0, 3.0, (H, W, 4))
    return cam, gb, glb, base


def _numpy_reflections(cam, gb, glb, base, ssr, planar, lm):
    """fs_reflection without RC, restated over whole images in float64."""
    H, W = base.shape[:2]
    if gb.layout == S.LAYOUT_REFERENCE:
        nr = gb.planes[1].astype(np.float64)
        orm = gb.planes[2].astype(np.float64) / 255.0
        em = gb.planes[3].astype(np.float64)
        n_raw, ao, rough = nr[..., :3], orm[..., 0], orm[..., 1]
        f0 = np.stack([nr[..., 3], orm[..., 3], em[..., 3]], -1)
        depth = gb.planes[4].astype(np.float64)
    elif gb.layout == S.LAYOUT_F32:  # ao 1, F0 = clamp(mix(0.04, albedo, metallic)) (gbuffer.wgsl:323-328)
        p0, p1 = gb.planes[0].astype(np.float64), gb.planes[1].astype(np.float64)
        n_raw, rough, metal = p1[..., :3], p0[..., 3], p1[..., 3]
        ao = np.ones_like(rough)
        f0 = 0.04 * (1 - metal[..., None]) + p0[..., :3] * metal[..., None]
        depth = gb.planes[2].astype(np.float64)
    else:  # F16: octahedral normal (Cigolle et al. 2014, z-up, signNotZero), metallic F0, ao 1
        p0 = gb.planes[0].astype(np.float64)
        o = gb.planes[1].astype(np.float64)
        metal = gb.planes[2].astype(np.float64).reshape(p0.shape[:2])
        u, v = o[..., 0], o[..., 1]
        z = 1 - np.abs(u) - np.abs(v)
        sx, sy = np.where(u >= 0, 1.0, -1.0), np.where(v >= 0, 1.0, -1.0)
        x = np.where(z < 0, (1 - np.abs(v)) * sx, u)
        y = np.where(z < 0, (1 - np.abs(u)) * sy, v)
        n_raw, rough = np.stack([x, y, z], -1), p0[..., 3]
        ao = np.ones_like(rough)
        f0 = 0.04 * (1 - metal[..., None]) + p0[..., :3] * metal[..., None]
        depth = gb.planes[3].astype(np.float64)
    N = n_raw / np.linalg.norm(n_raw, axis=-1, keepdims=True)
    f0 = np.clip(f0, 0.0, 0.999)
    xs, ys = np.meshgrid(np.arange(W) + 0.5, np.arange(H) + 0.5)
    ndc = np.stack([xs / W * 2 - 1, 1 - ys / H * 2, depth, np.ones_like(depth)], -1)
    inv = np.asarray(cam.record["inv_view_proj"], np.float64).reshape(4, 4)  # column major: rows of M^T
    h = ndc @ inv
    P = h[..., :3] / h[..., 3:4]
    eye = np.asarray(cam.record["position_near"], np.float64).reshape(-1)[:3]
    V = eye - P
    V /= np.linalg.norm(V, axis=-1, keepdims=True)
    ndv = np.maximum((N * V).sum(-1), 0.0)
    p5 = np.clip(1 - ndv, 0, 1) ** 5
    F = f0 + (np.maximum((1 - rough)[..., None], f0) - f0) * p5[..., None]
    spec = np.zeros((H, W, 3))
    s = ssr.astype(np.float64)
    pl = planar.astype(np.float64)
    if glb["enable_reflections"][0]:
        a = s[..., 3:4]
        spec = np.where(a > 0, spec * (1 - a) + s[..., :3] * F * a, spec)
        a = pl[..., 3:4]
        spec = np.where(a > 0, spec * (1 - a) + pl[..., :3] * F * a, spec)
    u = lm[..., 0].astype(np.float64) if lm is not None else np.full((H, W), -1.0)
    has_lm = ~(u < -1.5) & (u >= 0)
    out = base.copy()
    out[..., :3] += spec * np.where(has_lm, 1.0, ao)[..., None]
    sky = ~(depth < 1)
    out[sky] = base[sky]
    return out


def test_no_inputs_leave_the_target():
    for layout in (S.LAYOUT_REFERENCE, S.LAYOUT_F32, S.LAYOUT_F16):
        cam, gb, glb, base = _frame(layout)
        out, unsupported = oracle.reflections(cam.record, glb, gb, base)
        assert not unsupported
        np.testing.assert_array_equal(out, base)


@pytest.mark.parametrize("layout", [S.LAYOUT_REFERENCE, S.LAYOUT_F32, S.LAYOUT_F16])
@pytest.mark.parametrize("with_lightmap", [False, True])
def test_ssr_and_planar_match_numpy(with_lightmap, layout):
    cam, gb, glb, base = _frame(layout)
    ssr, planar, lm = S.reflection_images(gb.width, gb.height, 3)
    lm = lm if with_lightmap else None
    out, unsupported = oracle.reflections(cam.record, glb, gb, base, ssr=ssr, planar=planar, lightmap_uv=lm)
    assert not unsupported
    ref = _numpy_reflections(cam, gb, glb, base, ssr, planar, lm)
    np.testing.assert_allclose(out, ref, rtol=1e-12, atol=1e-12)
    covered = gb.planes[-1] < 1
    assert (np.abs(out - base)[covered][:, :3] > 0).any(-1).mean() > 0.5
    np.testing.assert_array_equal(out[..., 3], base[..., 3])  # alpha kept


def test_reflections_switched_off():
    cam, gb, glb, base = _frame(enable_reflections=0)
    ssr, planar, lm = S.reflection_images(gb.width, gb.height, 4)
    out, _ = oracle.reflections(cam.record, glb, gb, base, ssr=ssr, planar=planar, lightmap_uv=lm)
    np.testing.assert_array_equal(out, base)


def test_full_confidence_ssr_is_fresnel_times_hit():
    """With confidence 1 the SSR term replaces the environment term: spec = hit * F_ibl,
    so doubling the hit colour doubles the added light."""
    cam, gb, glb, base = _frame()
    ssr, _, _ = S.reflection_images(gb.width, gb.height, 6)
    ssr[..., 3] = 1.0
    ssr[..., :3] = np.float16(0.5)
    a, _ = oracle.reflections(cam.record, glb, gb, base, ssr=ssr)
    ssr[..., :3] = np.float16(1.0)
    b, _ = oracle.reflections(cam.record, glb, gb, base, ssr=ssr)
    np.testing.assert_allclose(b - base, 2 * (a - base), rtol=1e-12, atol=1e-14)


@pytest.mark.parametrize("mode", [30, 31])
def test_ssr_debug_modes_replace(mode):
    cam, gb, glb, base = _frame(debug_mode=mode)
    ssr, planar, _ = S.reflection_images(gb.width, gb.height, 8)
    out, _ = oracle.reflections(cam.record, glb, gb, base, ssr=ssr, planar=planar)
    covered = gb.planes[4] < 1
    s = ssr.astype(np.float64)
    want = np.concatenate([np.repeat(s[..., 3:4], 3, -1) if mode == 30 else s[..., :3], np.ones_like(s[..., :1])], -1)
    np.testing.assert_array_equal(out[covered], want[covered])
    np.testing.assert_array_equal(out[~covered], base[~covered])


@pytest.mark.parametrize("mode", [1, 2, 4, 5, 10, 11, 20, 21])
def test_lighting_debug_modes_add_nothing(mode):
    cam, gb, glb, base = _frame(debug_mode=mode)
    ssr, planar, _ = S.reflection_images(gb.width, gb.height, 9)
    out, _ = oracle.reflections(cam.record, glb, gb, base, ssr=ssr, planar=planar)
    np.testing.assert_array_equal(out, base)


def test_rc_specular_only_on_rough_pixels():
    cam, gb, glb, base = _frame(W=64, H=40)
    g = S.rc_globals(glb, RC_MIN, RC_MAX)
    probes = S.rc_probes(5)
    with_rc, unsupported = oracle.reflections(cam.record, g, gb, base, rc=probes)
    assert not unsupported
    rough = gb.planes[2][..., 1].astype(np.float64) / 255.0
    covered = gb.planes[4] < 1
    changed = (with_rc != base).any(-1)
    assert not changed[covered & (rough <= 0.6)].any()
    assert changed[covered & (rough > 0.6)].mean() > 0.9
    # blend weight smoothstep(0.6, 0.9, r) * 0.4 of a non-negative irradiance
    assert (with_rc[..., :3] >= base[..., :3]).all()
    # has_rc_gi without probes: the pixels that need them are reported
    _, unsupported = oracle.reflections(cam.record, g, gb, base)
    assert unsupported


def _env_scene(layout=S.LAYOUT_F32, W=64, H=40, seed=8):
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, layout, seed=seed)
    glb = L.make_globals(L.tile_grid(W, H)[0], 0)
    glb["enable_reflections"] = 1
    glb["enable_env_reflections"] = 1
    return cam, gb, glb


def test_environment_term_of_a_uniform_sky_is_the_split_sum():
    """Layer 0 only (no capture) holding one colour c at every texel: the environment
    sample is c at any direction and level, so the draw adds
    c (F0 env_brdf.x + env_brdf.y) ao (env_brdf_approx, pbr_eval.wgsl:70-76)."""
    cam, gb, glb = _env_scene()
    env = S.reflection_env(3, face_size=8, mip_levels=4, layers=1, n_captures=0)
    c = np.array([0.75, 1.5, 2.25])
    env["texels"][:, :3] = c.astype(np.float16)
    glb["reflection_capture_count"] = 0
    base = np.zeros((gb.height, gb.width, 4))
    out, flag = oracle.reflections(cam.record, glb, gb, base, env=env)
    assert not flag
    metal, dep = gb.planes[1][..., 3].astype(np.float64), gb.planes[2]
    # the three channels differ only through F0 and c: check their ratios
    m = dep < 1.0
    got = out[m][:, :3]
    assert np.all(got >= 0.0) and (got > 0).any(-1).mean() > 0.99
    ratio = got / c
    # for metallic == 0 every channel shares F0 = 0.04: the three ratios agree
    die = metal[m] == 0.0
    np.testing.assert_allclose(ratio[die][:, 0], ratio[die][:, 1], rtol=1e-12)
    np.testing.assert_allclose(ratio[die][:, 1], ratio[die][:, 2], rtol=1e-12)


def test_environment_capture_weight_and_brightness():
    """One sphere capture of uniform colour c1 (brightness b) well inside which every
    point lies, over a sky of colour c0: weight 1 everywhere inside the inner 90 % of
    the radius, so the sample is c1 b there; outside the sphere it is the sky c0."""
    cam, gb, glb = _env_scene(W=48, H=32)
    env = S.reflection_env(4, face_size=4, mip_levels=3, layers=2, n_captures=1)
    face = 6 * sum(max(1, 4 >> m) ** 2 for m in range(3))
    env["texels"][:face, :3] = np.float16(0.5)   # layer 0, the sky
    env["texels"][face:, :3] = np.float16(2.0)   # layer 1
    caps = env["captures"]
    caps[0]["position_radius"] = (0.0, 0.0, -10.0, 12.0)
    caps[0]["shape"] = L.CAPTURE_SPHERE
    caps[0]["cubemap_index"] = 1
    caps[0]["brightness"] = 1.25
    glb["reflection_capture_count"] = 1
    base = np.zeros((gb.height, gb.width, 4))
    out, _ = oracle.reflections(cam.record, glb, gb, base, env=env)
    env0 = dict(env, captures=caps[:0])
    glb0 = glb.copy()
    glb0["reflection_capture_count"] = 0
    sky, _ = oracle.reflections(cam.record, glb0, gb, base, env=env0)
    # world positions of the pixels (depth linear in NDC is not needed: use the ratio)
    m = gb.planes[2] < 1.0
    ratio = out[m][:, 0] / np.maximum(sky[m][:, 0], 1e-30)
    # inside: 2.0 * 1.25 / 0.5 = 5 times the sky; outside: 1; the fade band in between
    assert np.isclose(ratio, 5.0).any() and np.isclose(ratio, 1.0).any()
    assert np.all((ratio > 1.0 - 1e-9) & (ratio < 5.0 + 1e-9))
