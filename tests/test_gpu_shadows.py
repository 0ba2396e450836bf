"""GPU parity of the deferred pass's optional bindings against the f64 oracle:
hl_shade_shadowed / hl_shade_ex with shadow maps (the shadow term of the light loop) and
with radiance-cascade probes (indirect diffuse light).

Tolerances as for hl_shade (relative per pixel, floor 1e-6 of the image maximum):
FP32 / reference G-buffers 1e-5, FP16 G-buffer 2e-3. A pixel may exceed them when one
of its shadow taps compares a receiver depth that the kernel's f32 biased position and
the oracle's f64 one put on different sides of a texel depth (a "shadow flip"): such
pixels must be rare (at most 5e-4 of the lit pixels) and their error bounded by one
tap's weight in the filter."""
import numpy as np
import pytest

import oracle
from helio_gb300 import frame as FR
from helio_gb300 import layouts as L
from helio_gb300 import metrics
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

from gpu_util import gpu_shade
from scenes import directional_light, mixed_lights, point_light, spot_light

pytestmark = pytest.mark.gpu

TOL = {S.LAYOUT_F32: 1e-5, S.LAYOUT_REFERENCE: 1e-5, S.LAYOUT_F16: 2e-3}


def _lights(cam, seed):
    """Shadow casters first: a directional light, spots and points, then a mix."""
    casters = np.concatenate([
        directional_light((0.3, -1.0, 0.25), intensity=2.0),
        spot_light((0.0, 3.0, -8.0), 30.0, (0.0, -0.4, -1.0), 40.0, 30.0, intensity=6.0),
        spot_light((-4.0, 1.0, -20.0), 40.0, (0.3, 0.0, -1.0), 35.0, 20.0, intensity=6.0),
        point_light((2.0, 1.0, -15.0), 40.0, intensity=5.0),
        point_light((-3.0, -1.0, -30.0), 50.0, intensity=5.0),
        point_light((0.0, 0.0, -60.0), 60.0, intensity=8.0),
    ])
    return np.concatenate([casters, mixed_lights(cam, seed, 60, 20, n_dir=1)])


def _setup(layout, quality, W=320, H=192, size=256, seed=31):
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, layout, seed=seed)
    sc = S.shadow_scene(cam, _lights(cam, seed), 6, quality=quality)
    dyn, sta = S.shadow_atlases(sc.kinds, size, seed=seed)
    tx, _ = L.tile_grid(W, H)
    glb = L.make_globals(tx, len(sc.lights), ambient_color=(0.4, 0.45, 0.5), ambient_intensity=0.3)
    return cam, gb, sc, dyn, sta, glb


def _device_shadows(sc, dyn, sta):
    import torch

    d = dict(dyn=torch.from_numpy(dyn).cuda(), sta=torch.from_numpy(sta).cuda(),
             mats=torch.from_numpy(sc.matrices).cuda(), cfg=FR.bytes_tensor(sc.config))
    return d, N.shadow_maps_struct(d["dyn"], d["sta"], d["mats"], d["cfg"], sc.max_lights)


def _shade_shadowed(ctx, df, grid, maps, fill=7.0):
    import torch

    out = torch.full((df.height, df.width, 4), fill, dtype=torch.float32, device="cuda")
    ctx.shade_shadowed(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, maps, N.target_struct(out))
    ctx.sync_status()
    return out.cpu().numpy().astype(np.float64)


def _froxel_grid(cam, lights, W, H):
    import torch

    p = L.froxel_params(16, 9, 24, W, H, cam.far)
    off, idx = oracle.bin_froxels(cam.record, lights, p, capacity=1 << 24)
    doff = torch.from_numpy(off.view(np.int32).copy()).cuda()
    didx = torch.from_numpy(idx.view(np.int32).copy()).cuda()
    return ("froxels", idx, off, p), N.froxel_grid_struct(didx, doff, N.froxel_params_from_numpy(p), didx.numel()), \
        (didx, doff)


@pytest.mark.parametrize("quality", ["medium", "high"])
@pytest.mark.parametrize("layout", [S.LAYOUT_F32, S.LAYOUT_REFERENCE, S.LAYOUT_F16])
def test_shadowed_matches_oracle(ctx, layout, quality):
    cam, gb, sc, dyn, sta, glb = _setup(layout, quality)
    W, H = gb.width, gb.height
    df = FR.upload(cam.record, glb, sc.lights, gb)
    ogrid, dgrid, keep = _froxel_grid(cam, sc.lights, W, H)
    dsh, maps = _device_shadows(sc, dyn, sta)
    img = _shade_shadowed(ctx, df, dgrid, maps)
    shadows = dict(dynamic=dyn, static=sta, matrices=sc.matrices, config=sc.config, max_lights=sc.max_lights)
    ref, pc, bounds = oracle.shade_shadowed(cam.record, glb, gb, sc.lights, ogrid, shadows, pair_counts=True)
    assert not bounds
    st = gpu_shade(ctx, df, dgrid, stats=True)
    e = metrics.radiance_error(img, ref, st[..., 2], pc[..., 2])
    assert e["flips"] <= max(2, 1e-4 * e["n"]), e
    sky = np.isnan(ref[..., 0])
    assert np.all(img[sky] == 7.0)
    # the shadows are exercised: many pixels darker than without them
    plain = oracle.shade(cam.record, glb, gb, sc.lights, ogrid)
    darker = (ref[~sky][:, :3] < plain[~sky][:, :3] * (1 - 1e-6)).any(-1).mean()
    assert darker > 0.05, darker
    tol = TOL[layout]
    k, o = img[..., :3], ref[..., :3]
    valid = ~sky & (st[..., 2] == pc[..., 2])
    mx = np.abs(o[valid]).max()
    rel = (np.abs(k - o) / np.maximum(np.abs(o), 1e-6 * mx)).max(-1)[valid]
    n_over = int((rel > tol).sum())
    assert n_over <= max(3, 5e-4 * rel.size), (n_over, float(rel.max()), e)
    assert float(np.quantile(rel, 0.9999)) <= tol, e


def test_shadows_off_equal_hl_shade(ctx):
    cam, gb, sc, dyn, sta, glb = _setup(S.LAYOUT_F32, "medium", W=160, H=96, size=64)
    df = FR.upload(cam.record, glb, sc.lights, gb)
    _, dgrid, keep = _froxel_grid(cam, sc.lights, gb.width, gb.height)
    dsh, maps = _device_shadows(sc, dyn, sta)
    maps.max_shadow_lights = 0  # no light casts a shadow
    np.testing.assert_array_equal(_shade_shadowed(ctx, df, dgrid, maps), gpu_shade(ctx, df, dgrid))
    np.testing.assert_array_equal(_shade_shadowed(ctx, df, dgrid, None), gpu_shade(ctx, df, dgrid))


def test_shadow_layer_beyond_atlas_is_reported(ctx):
    import torch

    cam, gb, sc, dyn, sta, glb = _setup(S.LAYOUT_F32, "medium", W=160, H=96, size=64)
    lt = sc.lights.copy()
    lt["shadow_index"][:6] = 10_000
    df = FR.upload(cam.record, glb, lt, gb)
    _, dgrid, keep = _froxel_grid(cam, lt, gb.width, gb.height)
    dsh, maps = _device_shadows(sc, dyn, sta)
    out = torch.zeros((gb.height, gb.width, 4), dtype=torch.float32, device="cuda")
    ctx.shade_shadowed(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, dgrid, maps, N.target_struct(out))
    with pytest.raises(N.HelioError) as e:
        ctx.sync_status()
    assert e.value.status == N.HL_ERR_DEVICE_BOUNDS
    # skipped layers are lit: the result is the unshadowed one
    np.testing.assert_array_equal(out.cpu().numpy().astype(np.float64), gpu_shade(ctx, df, dgrid))


def test_shadow_argument_errors(ctx):
    cam, gb, sc, dyn, sta, glb = _setup(S.LAYOUT_F32, "medium", W=64, H=48, size=32)
    df = FR.upload(cam.record, glb, sc.lights, gb)
    _, dgrid, keep = _froxel_grid(cam, sc.lights, gb.width, gb.height)
    dsh, maps = _device_shadows(sc, dyn, sta)
    import torch

    out = torch.zeros((gb.height, gb.width, 4), dtype=torch.float32, device="cuda")
    for field, value, status in (("static_atlas", None, N.HL_ERR_INVALID_ARGUMENT), ("size", 0, N.HL_ERR_SIZE),
                                 ("reserved", 1, N.HL_ERR_INVALID_ARGUMENT),
                                 ("matrices", dsh["mats"].data_ptr() + 4, N.HL_ERR_LAYOUT)):
        _, m = _device_shadows(sc, dyn, sta)
        setattr(m, field, value)
        with pytest.raises(N.HelioError) as e:
            ctx.shade_shadowed(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, dgrid, m,
                               N.target_struct(out))
        assert e.value.status == status, field
    ctx.sync_status()


# ---- radiance-cascade GI (hl_shade_ex) ----

RC_MIN, RC_MAX = (-60.0, -40.0, -110.0), (60.0, 40.0, 0.0)


def _rc_device(probes):
    import torch

    t = torch.from_numpy(probes).cuda()
    return t, N.rc_cascade_struct(t)


def _shade_ex(ctx, df, grid, shadows=None, rc=None, fill=7.0):
    import torch

    out = torch.full((df.height, df.width, 4), fill, dtype=torch.float32, device="cuda")
    ctx.shade_ex(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, N.target_struct(out),
                 shadows=shadows, rc=rc)
    ctx.sync_status()
    return out.cpu().numpy().astype(np.float64)


# Radiance-cascade GI blends the hemisphere ambient h towards kD_ibl * irradiance * albedo
# by w = clamp(4 |irradiance|, 0, 1) (deferred_lighting.wgsl:1202-1209): where the blend
# nearly replaces a much larger h, the f32 error of w (~1e-6 relative, from the
# irradiance's sums) shows up as h * dw relative to a small result (measured up to
# 3.3e-4), so FP32 layouts are held to 5e-4 for these cases.
TOL_RC = {S.LAYOUT_F32: 5e-4, S.LAYOUT_REFERENCE: 5e-4, S.LAYOUT_F16: 2e-3}


def _check_tol(img, ref, st, pc, layout, tols=TOL_RC):
    e = metrics.radiance_error(img, ref, st[..., 2], pc[..., 2])
    assert e["flips"] <= max(2, 1e-4 * e["n"]), e
    sky = np.isnan(ref[..., 0])
    k, o = img[..., :3], ref[..., :3]
    valid = ~sky & (st[..., 2] == pc[..., 2])
    mx = np.abs(o[valid]).max()
    rel = (np.abs(k - o) / np.maximum(np.abs(o), 1e-6 * mx)).max(-1)[valid]
    tol = tols[layout]
    assert int((rel > tol).sum()) <= max(3, 5e-4 * rel.size), (int((rel > tol).sum()), float(rel.max()), e)
    assert float(np.quantile(rel, 0.9999)) <= tol, e
    return e


@pytest.mark.parametrize("with_shadows", [False, True])
@pytest.mark.parametrize("layout", [S.LAYOUT_F32, S.LAYOUT_REFERENCE, S.LAYOUT_F16])
def test_rc_gi_matches_oracle(ctx, layout, with_shadows):
    cam, gb, sc, dyn, sta, glb = _setup(layout, "high")
    glb = S.rc_globals(glb, RC_MIN, RC_MAX)
    probes = S.rc_probes(7)
    df = FR.upload(cam.record, glb, sc.lights, gb)
    ogrid, dgrid, keep = _froxel_grid(cam, sc.lights, gb.width, gb.height)
    dsh, maps = _device_shadows(sc, dyn, sta)
    drc, rcs = _rc_device(probes)
    img = _shade_ex(ctx, df, dgrid, shadows=maps if with_shadows else None, rc=rcs)
    shadows = dict(dynamic=dyn, static=sta, matrices=sc.matrices, config=sc.config, max_lights=sc.max_lights)
    ref, pc, _ = oracle.shade_ex(cam.record, glb, gb, sc.lights, ogrid, shadows=shadows if with_shadows else None,
                                 rc=probes, pair_counts=True)
    st = gpu_shade(ctx, df, dgrid, stats=True)
    _check_tol(img, ref, st, pc, layout)
    # the GI term is exercised: the radiance differs from the hemisphere-only one
    plain = oracle.shade_ex(cam.record, glb, gb, sc.lights, ogrid, shadows=shadows if with_shadows else None)[0]
    sky = np.isnan(ref[..., 0])
    changed = (np.abs(ref[~sky][:, :3] - plain[~sky][:, :3]) > 1e-6 * np.abs(plain[~sky][:, :3])).any(-1).mean()
    assert changed > 0.3, changed


def test_rc_gi_off_or_unbound(ctx):
    cam, gb, sc, dyn, sta, glb = _setup(S.LAYOUT_F32, "medium", W=160, H=96, size=64)
    df = FR.upload(cam.record, glb, sc.lights, gb)
    _, dgrid, keep = _froxel_grid(cam, sc.lights, gb.width, gb.height)
    drc, rcs = _rc_device(S.rc_probes(3))
    # probes bound, has_rc_gi == 0: the hemisphere ambient, as hl_shade
    np.testing.assert_array_equal(_shade_ex(ctx, df, dgrid, rc=rcs), gpu_shade(ctx, df, dgrid))
    # has_rc_gi != 0 without probes: reported as not supported
    dfo = FR.upload(cam.record, S.rc_globals(glb, RC_MIN, RC_MAX), sc.lights, gb)
    import torch

    out = torch.zeros((gb.height, gb.width, 4), dtype=torch.float32, device="cuda")
    ctx.shade_ex(dfo.camera, dfo.globals_, dfo.gbuffer, dfo.lights, dfo.n_lights, dgrid, N.target_struct(out))
    with pytest.raises(N.HelioError) as e:
        ctx.sync_status()
    assert e.value.status == N.HL_ERR_NOT_SUPPORTED
    # a probe texture smaller than 64 x 1024 is rejected
    small = N.rc_cascade_struct(drc[:512])
    with pytest.raises(N.HelioError) as e:
        ctx.shade_ex(dfo.camera, dfo.globals_, dfo.gbuffer, dfo.lights, dfo.n_lights, dgrid, N.target_struct(out),
                     rc=small)
    assert e.value.status == N.HL_ERR_SIZE


@pytest.mark.parametrize("layout", [S.LAYOUT_F32, S.LAYOUT_REFERENCE, S.LAYOUT_F16])
def test_shadow_debug_modes(ctx, layout):
    """Debug mode 10 (the mean shadow factor of the first light_count lights) and mode
    11 (the light-space projection by the first shadow matrix) of fs_main
    (deferred_lighting.wgsl:1049-1080), with shadow maps bound. Mode 11 is computed in
    f32 with the shader's operations in order: bit-exact against the f32 restatement.
    Mode 10 sums per-light shadow factors: exact except where a shadow tap flips."""
    cam, gb, sc, dyn, sta, glb0 = _setup(layout, "medium")
    W, H = gb.width, gb.height
    ogrid, dgrid, keep = _froxel_grid(cam, sc.lights, W, H)
    dsh, maps = _device_shadows(sc, dyn, sta)
    shadows = dict(dynamic=dyn, static=sta, matrices=sc.matrices, config=sc.config, max_lights=sc.max_lights)
    for mode in (10, 11):
        glb = L.make_globals(L.tile_grid(W, H)[0], len(sc.lights), debug_mode=mode)
        df = FR.upload(cam.record, glb, sc.lights, gb)
        img = _shade_shadowed(ctx, df, dgrid, maps)
        ref, _, _ = oracle.shade_shadowed(cam.record, glb, gb, sc.lights, ogrid, shadows)
        m = ~np.isnan(ref[..., 0])
        if mode == 11:
            assert np.array_equal(img[m], ref[m])
            inside = img[m][:, 2] == 0.0
            assert inside.any() and not inside.all(), "the first shadow frustum should cover part of the view"
        else:
            assert np.all(img[m][:, 3] == 1.0) and np.all(img[m][:, 0] == img[m][:, 1])
            d = np.abs(img[m][:, 0] - ref[m][:, 0])
            assert (d > 1e-6).mean() <= 5e-3, (d > 1e-6).mean()
            assert d.max() <= 1.0 / len(sc.lights) + 1e-6  # at most one light's factor apart
            assert (ref[m][:, 0] < 1.0).mean() > 0.1, "some pixels should be in shadow"


def test_shadow_debug_modes_without_shadow_maps(ctx):
    """hl_shade binds no shadow maps: every light's shadow factor is 1, so mode 10 is
    white (black with no light); mode 11 has no shadow matrix to project with and is
    reported as not supported."""
    W, H = 160, 96
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, S.LAYOUT_F16, seed=5)
    lt = mixed_lights(cam, 5, 30, 10)
    ogrid, dgrid, keep = _froxel_grid(cam, lt, W, H)
    for n, want in ((len(lt), 1.0), (0, 0.0)):
        glb = L.make_globals(L.tile_grid(W, H)[0], n, debug_mode=10)
        df = FR.upload(cam.record, glb, lt, gb)
        img = gpu_shade(ctx, df, dgrid)
        m = gb.planes[-1] < 1.0
        assert np.all(img[m][:, :3] == want) and np.all(img[m][:, 3] == 1.0)
    glb = L.make_globals(L.tile_grid(W, H)[0], len(lt), debug_mode=11)
    df = FR.upload(cam.record, glb, lt, gb)
    with pytest.raises(N.HelioError) as e:
        gpu_shade(ctx, df, dgrid)
    assert e.value.status == N.HL_ERR_NOT_SUPPORTED
