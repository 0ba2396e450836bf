"""GPU parity of hl_shade against the float64 oracle of fs_main / pbr_direct_light.

Tolerances (relative, per pixel, floor 1e-6 of the image maximum; see
helio_gb300/metrics.py):
  FP32 / reference G-buffers: max <= 1e-5
  FP16 G-buffer:              max <= 2e-3
The float64 reference is evaluated with the kernel's own branch decisions at the cuts
of pbr_direct_light (range, NdL == 0, radiance < 0.002), recorded by the timed
kernel itself (hl_set_pair_log), so every lit pixel is compared, including those where
f32 and f64 fall on different sides of a cut ("flips", counted)."""
import numpy as np
import pytest

import oracle
from helio_gb300 import frame as FR
from helio_gb300 import layouts as L
from helio_gb300 import metrics
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

from gpu_util import assert_tile_lists_equal, gpu_bin_froxels, gpu_bin_tiles, gpu_shade, gpu_shade_logged
from scenes import mixed_lights

pytestmark = pytest.mark.gpu

TOL = {S.LAYOUT_F32: (1e-5, 1e-5), S.LAYOUT_REFERENCE: (1e-5, 1e-5), S.LAYOUT_F16: (2e-3, 2e-3)}


def _grids(ctx, w_cam_rec, lights, gb, grid_shape, kind):
    import torch

    W, H = gb.width, gb.height
    if kind == "tiles":
        lists, counts = oracle.bin_tiles_ref(w_cam_rec, lights, W, H)
        dl = torch.from_numpy(lists.reshape(-1).view(np.int32).copy()).cuda()
        dc = torch.from_numpy(counts.view(np.int32).copy()).cuda()
        return ("tiles", lists, counts), N.tile_grid_struct(dl, dc), (dl, dc)
    p = L.froxel_params(*grid_shape, W, H, 100.0)
    off, idx = oracle.bin_froxels(w_cam_rec, lights, p, capacity=1 << 26)
    doff = torch.from_numpy(off.view(np.int32).copy()).cuda()
    didx = torch.from_numpy((idx if idx.size else np.zeros(1, np.uint32)).view(np.int32).copy()).cuda()
    return ("froxels", idx, off, p), N.froxel_grid_struct(didx, doff, N.froxel_params_from_numpy(p), didx.numel()), (didx, doff)


def _check(ctx, cam_rec, glb, lights, gb, grid_shape, kind, tol, counts=False):
    df = FR.upload(cam_rec, glb, lights, gb)
    ogrid, dgrid, keep = _grids(ctx, cam_rec, lights, gb, grid_shape, kind)
    img, pairs = gpu_shade_logged(ctx, df, dgrid)
    assert np.array_equal(gpu_shade(ctx, df, dgrid), img), "recording the lit pairs changed the image"
    ref, flips, unlisted = oracle.shade_forced(cam_rec, glb, gb, lights, ogrid, pairs)
    assert unlisted.sum() == 0, "the kernel lit a light that is not in the pixel's list"
    e = metrics.radiance_error(img, ref, flip_pixels=flips)
    sky = np.isnan(ref[..., 0])
    assert np.all(img[sky] == 7.0), "sky pixels must be left untouched"
    assert e["flips"] <= max(8, 1e-3 * e["n"]), e
    p_tol, max_tol = tol
    assert e["p9999"] <= p_tol and e["max"] <= max_tol, e
    # alpha channel
    assert np.allclose(img[~sky][:, 3], ref[~sky][:, 3])
    if not counts:
        return e, None, None
    _, pc = oracle.shade(cam_rec, glb, gb, lights, ogrid, pair_counts=True)
    st = gpu_shade(ctx, df, dgrid, stats=True)
    return e, st, pc


@pytest.mark.parametrize("wi", [0, 1, 4])
@pytest.mark.parametrize("kind", ["froxels", "tiles"])
def test_shade_workloads(ctx, wi, kind):
    w = S.workload(wi)
    _check(ctx, w.camera.record, w.globals_, w.lights, w.gbuffer, w.froxel_grid, kind, TOL[w.gbuffer.layout])


def test_shade_tiles_truncated_at_the_cap(ctx):
    """The reference's tile lists keep at most 64 lights per 16x16 tile
    (light_cull.wgsl:123-180). With 4096 clumped lights on a 960x540 view most tiles
    overflow: the GPU tile culling keeps the same first 64 lights as the oracle, and
    the shading over those truncated lists matches the oracle over the same lists."""
    w = S.workload(2, 0.25)
    W, H = w.gbuffer.width, w.gbuffer.height
    lists, counts = oracle.bin_tiles_ref(w.camera.record, w.lights, W, H)
    assert (counts == 64).mean() > 0.5
    assert_tile_lists_equal(gpu_bin_tiles(ctx, w.camera.record, w.lights, W, H), (lists, counts))
    _check(ctx, w.camera.record, w.globals_, w.lights, w.gbuffer, w.froxel_grid, "tiles", TOL[S.LAYOUT_F32])


def test_shade_4k_clumped(ctx):
    w = S.workload(2)
    _check(ctx, w.camera.record, w.globals_, w.lights, w.gbuffer, w.froxel_grid, "froxels", TOL[S.LAYOUT_F32])


def test_shade_fp16_clumped_long_lists(ctx):
    """The FP16 kernel over froxel lists of hundreds of entries (the clumped 4096-light
    workload's lights and grid at 1920x1080 on an FP16 G-buffer): several 32-entry chunks
    per froxel, culls and pair flushes under load; FP64 oracle with the kernel's own
    branch decisions."""
    w = S.workload(2, scale=0.5)
    gb = S.make_gbuffer(w.camera, S.LAYOUT_F16, seed=2000)
    p = L.froxel_params(*w.froxel_grid, gb.width, gb.height, w.camera.far)
    off, _ = oracle.bin_froxels(w.camera.record, w.lights, p, capacity=1 << 26)
    assert np.diff(off.astype(np.int64)).max() > 96
    _check(ctx, w.camera.record, w.globals_, w.lights, gb, w.froxel_grid, "froxels", TOL[S.LAYOUT_F16])


@pytest.mark.parametrize("layout", [S.LAYOUT_REFERENCE, S.LAYOUT_F32, S.LAYOUT_F16])
def test_shade_mixed_lights_with_ambient(ctx, layout):
    W, H = 480, 272
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, layout, seed=77)
    lt = mixed_lights(cam, 5, 150, 60, n_dir=2)
    tx, _ = L.tile_grid(W, H)
    glb = L.make_globals(tx, len(lt), ambient_color=(0.5, 0.5, 0.6), ambient_intensity=1.0)
    for kind in ("tiles", "froxels"):
        _check(ctx, cam.record, glb, lt, gb, (12, 8, 16), kind, TOL[layout])


def test_shade_pair_counts_match_oracle(ctx):
    w = S.workload(1)
    _, st, pc = _check(ctx, w.camera.record, w.globals_, w.lights, w.gbuffer, w.froxel_grid, "froxels",
                       TOL[w.gbuffer.layout], counts=True)
    mism = (st != pc).any(-1).mean()
    assert mism < 1e-4, mism


def test_shade_debug_modes(ctx):
    W, H = 128, 96
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, S.LAYOUT_F32, seed=3)
    lt = mixed_lights(cam, 9, 20, 5)
    tx, _ = L.tile_grid(W, H)
    for mode in (1, 5):
        glb = L.make_globals(tx, len(lt), debug_mode=mode)
        df = FR.upload(cam.record, glb, lt, gb)
        ogrid, dgrid, keep = _grids(ctx, cam.record, lt, gb, None, "tiles")
        img = gpu_shade(ctx, df, dgrid)
        ref = oracle.shade(cam.record, glb, gb, lt, ogrid)
        m = ~np.isnan(ref[..., 0])
        np.testing.assert_allclose(img[m], ref[m], rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("wi", [0, 1])  # FP32 G-buffer (shade_kernel), FP16 G-buffer (shade_f16_kernel)
def test_shade_rgba16f_target(ctx, wi):
    """The reference's own output format (RGBA16F, like pre_aa): each texel is the
    RGBA32F result rounded once to half precision, after an RGBA32F launch of the same
    kernel (both target instantiations launched in one process)."""
    w = S.workload(wi, scale=0.5)
    df = FR.upload_workload(w)
    ogrid, dgrid, keep = _grids(ctx, w.camera.record, w.lights, w.gbuffer, w.froxel_grid, "froxels")
    img32, pairs = gpu_shade_logged(ctx, df, dgrid)
    img = gpu_shade(ctx, df, dgrid, target_format=N.TARGET_RGBA16F)
    np.testing.assert_array_equal(img, img32.astype(np.float32).astype(np.float16).astype(np.float64))
    ref, flips, _ = oracle.shade_forced(w.camera.record, w.globals_, w.gbuffer, w.lights, ogrid, pairs)
    m = ~np.isnan(ref[..., 0])
    # the kernel's tolerance plus one rounding to half: 2^-11 relative for normal halves,
    # half of the subnormal spacing (2^-25) below 2^-14
    r = np.abs(ref[m][:, :3])
    tol = (TOL[w.gbuffer.layout][1] + 2.0 ** -11) * np.maximum(r, 1e-6 * r.max()) + 2.0 ** -25  # floor as metrics
    assert (np.abs(img[m][:, :3] - ref[m][:, :3]) <= tol).all()


def test_shade_uses_gpu_lists(ctx):
    """The whole path: lists from the GPU binning feed the GPU shading."""
    w = S.workload(1)
    p = L.froxel_params(*w.froxel_grid, w.gbuffer.width, w.gbuffer.height, w.camera.far)
    off, idx, keep = gpu_bin_froxels(ctx, w.camera.record, w.lights, p, capacity=1 << 20)
    cam_t, lt_t, d_off, d_idx, fp, cap = keep
    df = FR.upload_workload(w)
    grid = N.froxel_grid_struct(d_idx, d_off, fp, cap)
    img, pairs = gpu_shade_logged(ctx, df, grid)
    ref, flips, unlisted = oracle.shade_forced(w.camera.record, w.globals_, w.gbuffer, w.lights,
                                               ("froxels", idx, off, p), pairs)
    assert unlisted.sum() == 0
    e = metrics.radiance_error(img, ref, flip_pixels=flips)
    assert e["max"] <= 2e-3, e


def test_shade_rejects_bad_arguments(ctx):
    w = S.workload(0, scale=0.25)
    df = FR.upload_workload(w)
    ogrid, dgrid, keep = _grids(ctx, w.camera.record, w.lights, w.gbuffer, w.froxel_grid, "froxels")
    import torch

    out = torch.zeros((df.height, df.width, 4), dtype=torch.float32, device="cuda")
    bad = df.gbuffer
    bad.layout = 9
    with pytest.raises(N.HelioError) as e:
        ctx.shade(df.camera, df.globals_, bad, df.lights, df.n_lights, dgrid, N.target_struct(out))
    assert e.value.status == N.HL_ERR_INVALID_ARGUMENT
    gbm = df.gbuffer
    gbm.planes[0] = gbm.planes[0] + 4  # misaligned float4 plane
    with pytest.raises(N.HelioError) as e:
        ctx.shade(df.camera, df.globals_, gbm, df.lights, df.n_lights, dgrid, N.target_struct(out))
    assert e.value.status == N.HL_ERR_LAYOUT
    with pytest.raises(N.HelioError) as e:
        ctx.shade(df.camera, df.globals_, df.gbuffer, 0, df.n_lights, dgrid, N.target_struct(out))
    assert e.value.status == N.HL_ERR_INVALID_ARGUMENT


def test_fp16_froxel_out_of_range_light_index_is_reported(ctx):
    """FP16 G-buffer over froxel lists: an entry beyond n_lights, in a list of at most four
    entries (walked without the box cull) and in a long one, is skipped and reported
    (HL_ERR_DEVICE_BOUNDS), never read; the other pixels are unaffected."""
    import torch

    w = S.workload(1, scale=0.25)
    gb, cam = w.gbuffer, w.camera
    p = L.froxel_params(*w.froxel_grid, gb.width, gb.height, cam.far)
    off, idx = oracle.bin_froxels(cam.record, w.lights, p, capacity=1 << 24)
    lens = np.diff(off.astype(np.int64))
    short = int(np.flatnonzero((lens >= 1) & (lens <= 4))[0])
    long_ = int(np.argmax(lens))
    assert lens[long_] > 4
    bad = idx.copy()
    bad[off[short]] = 10_000_000
    bad[off[long_] + lens[long_] // 2] = 10_000_000
    df = FR.upload(cam.record, w.globals_, w.lights, gb)
    doff = torch.from_numpy(off.view(np.int32).copy()).cuda()
    didx = torch.from_numpy(bad.view(np.int32).copy()).cuda()
    grid = N.froxel_grid_struct(didx, doff, N.froxel_params_from_numpy(p), didx.numel())
    out = torch.zeros((gb.height, gb.width, 4), dtype=torch.float32, device="cuda")
    ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, N.target_struct(out))
    with pytest.raises(N.HelioError) as e:
        ctx.sync_status()
    assert e.value.status == N.HL_ERR_DEVICE_BOUNDS
    ctx.sync_status()  # cleared
    assert np.isfinite(out.cpu().numpy()).all()


def test_shade_out_of_range_light_index_is_reported(ctx):
    """A list entry beyond n_lights is skipped and reported, never read."""
    import torch

    w = S.workload(0, scale=0.25)
    df = FR.upload_workload(w)
    lists, counts = oracle.bin_tiles_ref(w.camera.record, w.lights, df.width, df.height)
    lists = lists.copy()
    counts = counts.copy()
    lists[0, 0] = 10_000_000
    counts[0] = max(int(counts[0]), 1)
    dl = torch.from_numpy(lists.reshape(-1).view(np.int32).copy()).cuda()
    dc = torch.from_numpy(counts.view(np.int32).copy()).cuda()
    out = torch.zeros((df.height, df.width, 4), dtype=torch.float32, device="cuda")
    ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, N.tile_grid_struct(dl, dc), N.target_struct(out))
    with pytest.raises(N.HelioError) as e:
        ctx.sync_status()
    assert e.value.status == N.HL_ERR_DEVICE_BOUNDS
    ctx.sync_status()  # cleared
