"""hl_shade_reflections (the reflection draw, deferred_lighting.wgsl:1265-1341) against
the oracle: SSR and planar blends with and without lightmap UVs, the radiance-cascade
rough-specular fallback, the SSR debug modes, both target formats and argument errors."""
import numpy as np
import pytest

import oracle
from helio_gb300 import frame as FR
from helio_gb300 import layouts as L
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

RC_MIN, RC_MAX = (-60.0, -40.0, -110.0), (60.0, 40.0, 0.0)
# f32 arithmetic on values of order 1 (the world position and V in double-float):
# relative error of the added light ~1e-6; an RGBA16F target rounds the sum once.
TOL = {N.TARGET_RGBA32F: 1e-5, N.TARGET_RGBA16F: 1e-3}


def _frame(layout, W=320, H=192, seed=23, rc=False, **glb_kw):
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, layout, seed=seed)
    tx, _ = L.tile_grid(W, H)
    glb = L.make_globals(tx, 0)
    if rc:
        glb = S.rc_globals(glb, RC_MIN, RC_MAX)
    for k, v in glb_kw.items():
        glb[k] = v
    base = np.random.default_rng(seed).uniform(0.0, 3.0, (H, W, 4)).astype(np.float32)
    return cam, gb, glb, base


def _run(ctx, cam, gb, glb, base, fmt=N.TARGET_RGBA32F, ssr=None, planar=None, lm=None, probes=None):
    import torch

    df = FR.upload(cam.record, glb, np.zeros(0, L.GPU_LIGHT), gb)
    dt = torch.float32 if fmt == N.TARGET_RGBA32F else torch.float16
    out = torch.from_numpy(base).to(dt).cuda()
    dev = {k: torch.from_numpy(v).cuda() if v is not None else None
           for k, v in (("ssr", ssr), ("planar", planar), ("lm", lm))}
    rc = None
    if probes is not None:
        dev["rc"] = torch.from_numpy(probes).cuda()
        rc = N.rc_cascade_struct(dev["rc"])
    ctx.shade_reflections(df.camera, df.globals_, df.gbuffer, N.target_struct(out, fmt), ssr=dev["ssr"],
                          planar=dev["planar"], lightmap_uv=dev["lm"], rc=rc)
    ctx.sync_status()
    start = base.astype(np.float64) if fmt == N.TARGET_RGBA32F else base.astype(np.float16).astype(np.float64)
    return out.float().cpu().numpy().astype(np.float64), start


def _check(img, ref, start, fmt):
    added = np.abs(ref[..., :3] - start[..., :3])
    assert (added > 0).any(-1).mean() > 0.3  # the draw adds light to most pixels
    tol = TOL[fmt]
    err = np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3)
    assert float(err.max()) <= tol, (float(err.max()), np.unravel_index(err.argmax(), err.shape))
    np.testing.assert_array_equal(img[..., 3], start[..., 3])  # alpha kept


@pytest.mark.parametrize("with_rc", [False, True])
@pytest.mark.parametrize("layout", [S.LAYOUT_REFERENCE, S.LAYOUT_F32, S.LAYOUT_F16])
def test_reflections_match_oracle(ctx, layout, with_rc):
    cam, gb, glb, base = _frame(layout, rc=with_rc)
    ssr, planar, lm = S.reflection_images(gb.width, gb.height, 11)
    probes = S.rc_probes(7) if with_rc else None
    img, start = _run(ctx, cam, gb, glb, base, ssr=ssr, planar=planar, lm=lm, probes=probes)
    ref, unsupported = oracle.reflections(cam.record, glb, gb, start, ssr=ssr, planar=planar, lightmap_uv=lm,
                                          rc=probes)
    assert not unsupported
    _check(img, ref, start, N.TARGET_RGBA32F)


def test_reflections_rgba16f_target(ctx):
    cam, gb, glb, base = _frame(S.LAYOUT_REFERENCE, rc=True)
    ssr, planar, lm = S.reflection_images(gb.width, gb.height, 12)
    probes = S.rc_probes(2)
    img, start = _run(ctx, cam, gb, glb, base, fmt=N.TARGET_RGBA16F, ssr=ssr, planar=planar, lm=lm,
                      probes=probes)
    ref, _ = oracle.reflections(cam.record, glb, gb, start, ssr=ssr, planar=planar, lightmap_uv=lm, rc=probes)
    _check(img, ref, start, N.TARGET_RGBA16F)


def test_no_inputs_leave_the_target(ctx):
    cam, gb, glb, base = _frame(S.LAYOUT_F32, W=96, H=64)
    img, start = _run(ctx, cam, gb, glb, base)
    np.testing.assert_array_equal(img, start)


@pytest.mark.parametrize("mode", [30, 31, 5])
def test_debug_modes(ctx, mode):
    cam, gb, glb, base = _frame(S.LAYOUT_REFERENCE, W=96, H=64, debug_mode=mode)
    ssr, planar, _ = S.reflection_images(gb.width, gb.height, 13)
    img, start = _run(ctx, cam, gb, glb, base, ssr=ssr, planar=planar)
    ref, _ = oracle.reflections(cam.record, glb, gb, start, ssr=ssr, planar=planar)
    np.testing.assert_array_equal(img, ref)


def test_reflection_argument_errors(ctx):
    import torch

    cam, gb, glb, base = _frame(S.LAYOUT_REFERENCE, W=96, H=64, rc=True)
    df = FR.upload(cam.record, glb, np.zeros(0, L.GPU_LIGHT), gb)
    out = torch.zeros((gb.height, gb.width, 4), dtype=torch.float32, device="cuda")
    # has_rc_gi with rough pixels and no probes: reported as not supported
    ctx.shade_reflections(df.camera, df.globals_, df.gbuffer, N.target_struct(out))
    with pytest.raises(N.HelioError) as e:
        ctx.sync_status()
    assert e.value.status == N.HL_ERR_NOT_SUPPORTED
    # an SSR image narrower than the G-buffer
    narrow = torch.zeros((gb.height, gb.width - 8, 4), dtype=torch.float16, device="cuda")
    with pytest.raises(N.HelioError) as e:
        ctx.shade_reflections(df.camera, df.globals_, df.gbuffer, N.target_struct(out), ssr=narrow)
    assert e.value.status == N.HL_ERR_LAYOUT
    # a probe texture smaller than 64 x 1024
    probes = torch.from_numpy(S.rc_probes(1)).cuda()
    with pytest.raises(N.HelioError) as e:
        ctx.shade_reflections(df.camera, df.globals_, df.gbuffer, N.target_struct(out),
                              rc=N.rc_cascade_struct(probes[:512]))
    assert e.value.status == N.HL_ERR_SIZE


def test_rc_globals_without_probes_report_and_keep_the_other_pixels(ctx):
    """has_rc_gi set with no probe texture bound: the draw reports HL_ERR_NOT_SUPPORTED,
    leaves the pixels that need the radiance-cascade fallback (roughness > 0.6) as they
    were, and still lights every other pixel as the oracle does."""
    import torch

    cam, gb, glb, base = _frame(S.LAYOUT_REFERENCE, rc=True)
    ssr, planar, lm = S.reflection_images(gb.width, gb.height, 14)
    df = FR.upload(cam.record, glb, np.zeros(0, L.GPU_LIGHT), gb)
    out = torch.from_numpy(base).cuda()
    dssr, dpl, dlm = (torch.from_numpy(a).cuda() for a in (ssr, planar, lm))
    ctx.shade_reflections(df.camera, df.globals_, df.gbuffer, N.target_struct(out), ssr=dssr, planar=dpl,
                          lightmap_uv=dlm)
    with pytest.raises(N.HelioError) as e:
        ctx.sync_status()
    assert e.value.status == N.HL_ERR_NOT_SUPPORTED
    img = out.cpu().numpy().astype(np.float64)
    start = base.astype(np.float64)
    ref, unsupported = oracle.reflections(cam.record, glb, gb, start, ssr=ssr, planar=planar, lightmap_uv=lm)
    assert unsupported
    rough = gb.planes[2][..., 1].astype(np.float32) / np.float32(255.0) > 0.6  # ORM green, unorm8
    assert 0.1 < rough.mean() < 0.9
    np.testing.assert_array_equal(img[rough], start[rough])
    _check(img, ref, start, N.TARGET_RGBA32F)
    assert (np.abs(img - start)[~rough].max(-1) > 0).mean() > 0.3  # the smooth pixels were lit


@pytest.mark.parametrize("layout", [S.LAYOUT_REFERENCE, S.LAYOUT_F32, S.LAYOUT_F16])
@pytest.mark.parametrize("fmt", [N.TARGET_RGBA32F, N.TARGET_RGBA16F])
def test_environment_term_matches_oracle(ctx, layout, fmt):
    """The environment term (sample_reflection_environment, deferred_lighting.wgsl:646-694)
    with sphere and box captures over a cube-map array with mip chains, with SSR and
    planar hits blended over it. A pixel whose reflection direction lies within f32
    rounding of a cube face edge may sample the other face (the faces are filtered
    separately): such pixels must be rare."""
    import torch

    cam, gb, glb, base = _frame(layout, seed=41)
    glb["enable_reflections"] = 1
    glb["enable_env_reflections"] = 1
    env = S.reflection_env(41)
    glb["reflection_capture_count"] = len(env["captures"])
    ssr, planar, lm = S.reflection_images(gb.width, gb.height, 41)
    dcap = torch.from_numpy(env["captures"].view(np.uint8).copy()).cuda()
    dtex = torch.from_numpy(env["texels"]).cuda()
    es = N.reflection_env_struct(dcap, len(env["captures"]), dtex, env["face_size"], env["mip_levels"],
                                 env["layers"])
    df = FR.upload(cam.record, glb, np.zeros(0, L.GPU_LIGHT), gb)
    dt = torch.float32 if fmt == N.TARGET_RGBA32F else torch.float16
    out = torch.from_numpy(base).to(dt).cuda()
    dssr, dpl, dlm = (torch.from_numpy(a).cuda() for a in (ssr, planar, lm))
    ctx.shade_reflections(df.camera, df.globals_, df.gbuffer, N.target_struct(out, fmt), ssr=dssr, planar=dpl,
                          lightmap_uv=dlm, env=es)
    ctx.sync_status()
    img = out.float().cpu().numpy().astype(np.float64)
    start = base.astype(np.float64) if fmt == N.TARGET_RGBA32F else base.astype(np.float16).astype(np.float64)
    ref, flag = oracle.reflections(cam.record, glb, gb, start, ssr=ssr, planar=planar, lightmap_uv=lm, env=env)
    assert not flag
    m = gb.planes[-1] < 1.0
    added = np.abs(ref[m][:, :3] - start[m][:, :3])
    assert (added > 0).any(-1).mean() > 0.9  # the environment lights almost every pixel
    err = (np.abs(img - ref) / np.maximum(np.abs(ref), 1e-3))[m].max(-1)
    bad = err > TOL[fmt]
    assert bad.sum() <= max(2, 2e-4 * m.sum()), (int(bad.sum()), float(err.max()))
    np.testing.assert_array_equal(img[..., 3], start[..., 3])  # alpha kept


def test_environment_rejects_bad_inputs(ctx):
    import torch

    cam, gb, glb, base = _frame(S.LAYOUT_F32, W=64, H=32)
    env = S.reflection_env(2)
    df = FR.upload(cam.record, glb, np.zeros(0, L.GPU_LIGHT), gb)
    out = torch.from_numpy(base).cuda()
    dcap = torch.from_numpy(env["captures"].view(np.uint8).copy()).cuda()
    dtex = torch.from_numpy(env["texels"]).cuda()
    for kw, status in ((dict(face_size=0), N.HL_ERR_SIZE), (dict(mip_levels=16), N.HL_ERR_SIZE),
                       (dict(layers=0), N.HL_ERR_SIZE)):
        args = dict(face_size=env["face_size"], mip_levels=env["mip_levels"], layers=env["layers"])
        args.update(kw)
        es = N.reflection_env_struct(dcap, len(env["captures"]), dtex, **args)
        with pytest.raises(N.HelioError) as e:
            ctx.shade_reflections(df.camera, df.globals_, df.gbuffer, N.target_struct(out), env=es)
        assert e.value.status == status
