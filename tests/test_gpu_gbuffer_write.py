"""GPU parity of hl_write_gbuffer (the G-buffer pass's fragment stage, gbuffer.wgsl
fs_main) against the float64 oracle (oracle/gbuffer_write.cpp).

Tolerances, per channel of every written pixel:
  RGBA8 unorm targets (albedo, orm): the stored byte is a correct rounding of the
      oracle's value, |byte - 255 clamp(v)| <= 0.5 + 1e-3;
  RGBA16F / RG16F targets (normal, emissive, lightmap_uv, velocity): within half an
      f16 ulp of the oracle's value plus 1e-5 relative (f32 against f64 arithmetic),
      plus 2e-6 absolute for the unit normal's components.
Written / discarded pixels must agree exactly; discarded and uncovered pixels keep
every byte of their previous contents."""
import numpy as np
import pytest

import oracle
from helio_gb300 import frame as FR
from helio_gb300 import layouts as L
from helio_gb300 import metrics
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

from gpu_util import gpu_bin_froxels, gpu_shade
from scenes import mixed_lights

pytestmark = pytest.mark.gpu

FILL = 0xAB


def _run(ctx, scene, optional=True, n_materials=None, n_textures=None):
    d = FR.upload_material_scene(scene)
    planes, tg = FR.gbuffer_targets(d.width, d.height, optional=optional, fill=FILL)
    nm = d.n_materials if n_materials is None else n_materials
    table = d.texture_table if n_textures is None else d.texture_table[:n_textures]
    ctx.write_gbuffer(d.globals_, d.surfaces, d.surfaces_pitch, d.materials, d.material_textures, nm, table, tg)
    status = N.HL_OK
    try:
        ctx.sync_status()
    except N.HelioError as e:
        status = e.status
    host = [None if p is None else p.cpu().numpy() for p in planes]
    return host, status, d, planes


def _raw(p):
    return p.view(np.uint8).reshape(p.shape[0], p.shape[1], -1)


def _written(host):
    return np.any(np.concatenate([_raw(host[i]) for i in range(4)], -1) != FILL, axis=-1)


def _half_tol(v, floor=0.0):
    """Half an f16 ulp of v, plus 1e-5 relative and ``floor`` absolute for the f32
    evaluation (``floor`` 2e-6 for unit-normal components, whose f32 error is absolute)."""
    return 2.0 ** -11 * np.maximum(np.abs(v), 2.0 ** -14) + 1e-5 * np.abs(v) + floor


def _check(host, want, written, optional=True):
    got_w = _written(host)
    np.testing.assert_array_equal(got_w, written, err_msg="written/discarded pixels differ from the oracle")
    for i in range(len(host)):
        if host[i] is not None:
            assert np.all(_raw(host[i])[~written] == FILL), f"target {i} touched at a discarded/uncovered pixel"
    w = want[written]
    for plane, sl in ((0, slice(0, 4)), (2, slice(8, 12))):
        got = host[plane][written].astype(np.float64)
        exp = np.clip(w[:, sl], 0.0, 1.0) * 255.0
        err = np.abs(got - exp).max() if len(got) else 0.0
        assert err <= 0.5 + 1e-3, f"unorm8 target {plane}: max |byte - 255 v| = {err}"
    unit = np.array([2e-6, 2e-6, 2e-6, 0.0])
    halves = [(1, slice(4, 8), unit), (3, slice(12, 16), 0.0)]
    if optional:
        halves += [(4, slice(16, 18), 0.0), (7, slice(18, 20), 0.0)]
    for plane, sl, floor in halves:
        got = host[plane][written].astype(np.float64)
        exp = w[:, sl]
        bad = np.abs(got - exp) > _half_tol(exp, floor)
        assert not bad.any(), f"f16 target {plane}: {int(bad.sum())} values off, e.g. got {got[bad][:4]} want {exp[bad][:4]}"
    if optional:
        for plane in (5, 6):  # sss and extra: zero in the default template
            assert np.all(host[plane][written] == 0)


def _oracle(scene, n_materials=None, n_textures=None):
    mats = scene.materials if n_materials is None else scene.materials[:n_materials]
    mtex = scene.material_textures if n_materials is None else scene.material_textures[:n_materials]
    tex = scene.textures if n_textures is None else scene.textures[:n_textures]
    return oracle.write_gbuffer(scene.globals_, scene.surfaces, mats, mtex, tex)


@pytest.mark.parametrize("seed,size", [(5, (480, 270)), (11, (333, 187))])
def test_gbuffer_write_matches_oracle(ctx, seed, size):
    scene = S.material_scene(S.default_camera(*size), seed)
    host, status, _, _ = _run(ctx, scene)
    assert status == N.HL_OK
    want, written, bounds = _oracle(scene)
    assert not bounds
    assert 0.5 < written.mean() < 0.99  # discards and uncovered pixels are exercised
    _check(host, want, written)


@pytest.mark.parametrize("debug", [1, 2, 3])
def test_gbuffer_write_debug_modes(ctx, debug):
    scene = S.material_scene(S.default_camera(256, 144), 3, debug_mode=debug)
    host, status, _, _ = _run(ctx, scene)
    assert status == N.HL_OK
    want, written, _ = _oracle(scene)
    assert np.array_equal(written, scene.covered)  # no discard in the debug modes
    _check(host, want, written)


def test_gbuffer_write_required_targets_only(ctx):
    scene = S.material_scene(S.default_camera(200, 120), 8)
    full, _, _, _ = _run(ctx, scene)
    req, status, _, _ = _run(ctx, scene, optional=False)
    assert status == N.HL_OK
    for i in range(4):
        np.testing.assert_array_equal(_raw(req[i]), _raw(full[i]))


def test_gbuffer_write_out_of_range_indices(ctx):
    scene = S.material_scene(S.default_camera(256, 144), 5)
    nm, nt = 20, 7
    host, status, _, _ = _run(ctx, scene, n_materials=nm, n_textures=nt)
    assert status == N.HL_ERR_DEVICE_BOUNDS
    want, written, bounds = _oracle(scene, n_materials=nm, n_textures=nt)
    assert bounds
    mids = scene.surfaces["material_id"]
    assert not written[(mids != L.NO_FRAGMENT) & (mids >= nm)].any()
    _check(host, want, written)


def test_gbuffer_write_address_modes_and_filters(ctx):
    """One 5x3 texture of distinct texels under every (address mode, filter) pair, UVs
    sweeping [-2.3, 2.7] in both axes."""
    W, H = 64, 48
    cam = S.default_camera(W, H)
    base = S.material_scene(cam, 1, n_materials=1, n_textures=1)
    tex = (np.arange(5 * 3 * 4, dtype=np.float64).reshape(3, 5, 4) * 4 + 3).astype(np.uint8)
    for mode in (L.ADDRESS_REPEAT, L.ADDRESS_CLAMP_TO_EDGE, L.ADDRESS_MIRROR_REPEAT):
        for filt in (L.FILTER_NEAREST, L.FILTER_LINEAR):
            for fmt in (L.TEX_RGBA8_UNORM, L.TEX_RGBA8_SRGB):
                sc = S.material_scene(cam, 1, n_materials=1, n_textures=1)
                sc.textures = [(tex, fmt, mode, (mode + 1) % 3, filt)]
                mt = L.missing_material_textures(1)
                mt["base_color"]["texture_index"] = 0
                mt["params"] = (1.0, 1.0, 0.0, 0.0)
                sc.material_textures = mt
                sc.materials = base.materials.copy()
                sc.materials["base_color"] = (1.0, 1.0, 1.0, 1.0)
                srf = sc.surfaces.copy()
                ys, xs = np.mgrid[0:H, 0:W]
                srf["material_id"] = 0
                srf["tex_coords"] = np.stack([-2.3 + 5.0 * xs / W, -2.3 + 5.0 * ys / H], -1)
                sc.surfaces = srf
                host, status, _, _ = _run(ctx, sc)
                assert status == N.HL_OK
                want, written, _ = _oracle(sc)
                assert written.all()
                _check(host, want, written)


def test_gbuffer_write_argument_errors(ctx):
    import torch

    scene = S.material_scene(S.default_camera(64, 32), 2)
    d = FR.upload_material_scene(scene)
    planes, tg = FR.gbuffer_targets(64, 32)

    def call(**kw):
        args = dict(globals_=d.globals_, surfaces=d.surfaces, surfaces_pitch=d.surfaces_pitch, materials=d.materials,
                    material_textures=d.material_textures, n_materials=d.n_materials, textures=d.texture_table,
                    targets=tg)
        args.update(kw)
        with pytest.raises(N.HelioError) as e:
            ctx.write_gbuffer(**args)
        return e.value.status

    assert call(surfaces_pitch=64 * 64 - 16) == N.HL_ERR_LAYOUT
    assert call(textures=d.texture_table * 40) == N.HL_ERR_SIZE  # 24 x 40 > 256
    bad = N.texture_struct(d.textures[0], 9)
    assert call(textures=[bad]) == N.HL_ERR_INVALID_ARGUMENT
    _, tg2 = FR.gbuffer_targets(64, 32)
    tg2.planes[2] = None
    assert call(targets=tg2) == N.HL_ERR_INVALID_ARGUMENT
    _, tg3 = FR.gbuffer_targets(64, 32)
    tg3.pitch[1] = 64 * 8 - 8
    assert call(targets=tg3) == N.HL_ERR_LAYOUT
    ctx.sync_status()


def test_reference_layout_frame_end_to_end(ctx):
    """G-buffer write -> froxel binning -> shading of the written reference-layout
    G-buffer, against the f64 oracle's shading of the same G-buffer bytes."""
    import torch

    W, H = 480, 270
    cam = S.default_camera(W, H)
    scene = S.material_scene(cam, 9)
    # a fragment the G-buffer pass discards writes no depth either: those pixels keep
    # the depth clear value 1.0, like the uncovered ones
    _, written, _ = _oracle(scene)
    scene.depth = np.where(written, scene.depth, np.float32(1.0)).astype(np.float32)
    d = FR.upload_material_scene(scene)
    planes, tg = FR.gbuffer_targets(W, H, optional=False, fill=0)
    d.write(ctx, tg)
    lights = mixed_lights(cam, 4, 200, 60, n_dir=1)
    tx, _ = L.tile_grid(W, H)
    glb = L.make_globals(tx, len(lights), ambient_color=(0.5, 0.5, 0.6), ambient_intensity=0.3)
    p = L.froxel_params(16, 9, 24, W, H, cam.far)
    off, idx, keep = gpu_bin_froxels(ctx, cam.record, lights, p)
    gbs = FR.reference_gbuffer(planes, d.depth)
    df = FR.DeviceFrame(W, H, N.GBUF_REFERENCE, FR.bytes_tensor(cam.record), FR.bytes_tensor(glb),
                        FR.bytes_tensor(lights), len(lights), [planes[0], planes[1], planes[2], planes[3], d.depth])
    assert df.gbuffer.layout == gbs.layout
    grid = N.froxel_grid_struct(keep[3], keep[2], keep[4], keep[5])
    img = gpu_shade(ctx, df, grid)
    st = gpu_shade(ctx, df, grid, stats=True)
    host_gb = S.GBuffer(S.LAYOUT_REFERENCE, W, H, [planes[i].cpu().numpy() for i in range(4)] + [scene.depth])
    ref, pc = oracle.shade(cam.record, glb, host_gb, lights, ("froxels", idx, off, p), pair_counts=True)
    e = metrics.radiance_error(img, ref, st[..., 2], pc[..., 2])
    assert e["flips"] <= max(2, 1e-4 * e["n"]), e
    assert e["p9999"] <= 1e-5 and e["max"] <= 1e-3, e
    sky = np.isnan(ref[..., 0])  # uncovered, discarded, or covered at a depth that rounds to 1.0
    assert np.array_equal(sky, ~written | (scene.depth >= 1.0))
