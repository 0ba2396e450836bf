"""GPU parity of the binning kernels: bit-exact against the f32 oracle.

Reference behaviour covered (light_cull.wgsl:123-180, light-cull/src/lib.rs:264-362):
ordered lists, the 64-light cap, directional lights always listed, clamped NDC at
the right/bottom edge tiles, zero lights clearing both buffers. Froxel lists: every
workload grid, capacity overflow, zero lights."""
import numpy as np
import pytest

import oracle
from helio_gb300 import layouts as L
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

from gpu_util import assert_tile_lists_equal, gpu_bin_froxels, gpu_bin_tiles
from scenes import mixed_lights, overlapping_lights

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("wi", [0, 1, 2, 4])
def test_tile_lists_workloads(ctx, wi):
    w = S.workload(wi)
    W, H = w.gbuffer.width, w.gbuffer.height
    got = gpu_bin_tiles(ctx, w.camera.record, w.lights, W, H)
    want = oracle.bin_tiles_ref(w.camera.record, w.lights, W, H)
    assert_tile_lists_equal(got, want)


@pytest.mark.parametrize("size", [(1000, 500), (17, 17), (1, 1), (1283, 719), (16, 4096)])
def test_tile_lists_ragged_viewports(ctx, size):
    W, H = size
    cam = S.default_camera(W, H)
    lt = mixed_lights(cam, 7, 120, 40)
    assert_tile_lists_equal(gpu_bin_tiles(ctx, cam.record, lt, W, H), oracle.bin_tiles_ref(cam.record, lt, W, H))


def test_tile_cap_drops_65th_light(ctx):
    W, H = 320, 180
    cam = S.default_camera(W, H)
    lt = overlapping_lights(70)
    lists, counts = gpu_bin_tiles(ctx, cam.record, lt, W, H)
    assert (counts == 64).all()
    assert (lists == np.arange(64, dtype=np.uint32)[None, :]).all()
    assert_tile_lists_equal((lists, counts), oracle.bin_tiles_ref(cam.record, lt, W, H))


def test_tile_directional_always_listed(ctx):
    W, H = 256, 128
    cam = S.default_camera(W, H)
    lt = mixed_lights(cam, 3, 10, 0, n_dir=3)
    lists, counts = gpu_bin_tiles(ctx, cam.record, lt, W, H)
    dirs = np.nonzero(lt["light_type"] == L.LIGHT_DIRECTIONAL)[0]
    for t in range(len(counts)):
        assert set(dirs.tolist()) <= set(lists[t, : counts[t]].tolist())


def test_tile_zero_lights_clears(ctx):
    W, H = 200, 100
    cam = S.default_camera(W, H)
    lists, counts = gpu_bin_tiles(ctx, cam.record, np.zeros(0, L.GPU_LIGHT), W, H)
    assert (counts == 0).all() and (lists == 0).all()


@pytest.mark.parametrize("wi", [0, 1, 2, 4])
def test_froxel_lists_workloads(ctx, wi):
    w = S.workload(wi)
    p = L.froxel_params(*w.froxel_grid, w.gbuffer.width, w.gbuffer.height, w.camera.far)
    off_w, idx_w = oracle.bin_froxels(w.camera.record, w.lights, p, capacity=1 << 26)
    off, idx, _ = gpu_bin_froxels(ctx, w.camera.record, w.lights, p, capacity=int(off_w[-1]) + 16)
    np.testing.assert_array_equal(off, off_w)
    np.testing.assert_array_equal(idx, idx_w)


@pytest.mark.parametrize("grid", [(1, 1, 1), (7, 5, 3), (16, 9, 24), (40, 23, 128)])
def test_froxel_lists_mixed_lights(ctx, grid):
    W, H = 640, 368
    cam = S.default_camera(W, H)
    lt = mixed_lights(cam, 11, 200, 80, n_dir=2)
    p = L.froxel_params(*grid, W, H, cam.far)
    off_w, idx_w = oracle.bin_froxels(cam.record, lt, p, capacity=1 << 26)
    off, idx, _ = gpu_bin_froxels(ctx, cam.record, lt, p, capacity=int(off_w[-1]) + 1)
    np.testing.assert_array_equal(off, off_w)
    np.testing.assert_array_equal(idx, idx_w)


def test_froxel_capacity_overflow(ctx):
    w = S.workload(0)
    p = L.froxel_params(*w.froxel_grid, w.gbuffer.width, w.gbuffer.height, w.camera.far)
    off_w, idx_w = oracle.bin_froxels(w.camera.record, w.lights, p, capacity=1 << 24)
    cap = int(off_w[-1]) // 2
    off, idx, _ = gpu_bin_froxels(ctx, w.camera.record, w.lights, p, capacity=cap, expect_status=N.HL_ERR_CAPACITY)
    np.testing.assert_array_equal(off, off_w)
    np.testing.assert_array_equal(idx[:cap], idx_w[:cap])


def test_froxel_zero_lights(ctx):
    cam = S.default_camera(320, 180)
    p = L.froxel_params(8, 4, 6, 320, 180, cam.far)
    off, idx, _ = gpu_bin_froxels(ctx, cam.record, np.zeros(0, L.GPU_LIGHT), p, capacity=16)
    assert (off == 0).all() and idx.size == 0


def test_froxel_lists_large_light_count(ctx):
    """More lights than one shared-memory round of the column list holds."""
    W, H = 256, 144
    cam = S.default_camera(W, H)
    lt = S.make_lights(cam, 21, 9000, 1000, radius=(5.0, 30.0))
    p = L.froxel_params(4, 2, 8, W, H, cam.far)
    off_w, idx_w = oracle.bin_froxels(cam.record, lt, p, capacity=1 << 26)
    off, idx, _ = gpu_bin_froxels(ctx, cam.record, lt, p, capacity=int(off_w[-1]))
    np.testing.assert_array_equal(off, off_w)
    np.testing.assert_array_equal(idx, idx_w)


def test_froxel_lists_many_columns(ctx):
    """32400 columns: far more CTAs than the GPU holds at once, so the single-pass
    binning's chained scan runs across many waves of CTAs."""
    W, H = 1920, 1080
    cam = S.default_camera(W, H)
    lt = mixed_lights(cam, 12, 300, 100, n_dir=1)
    p = L.froxel_params(240, 135, 4, W, H, cam.far)
    off_w, idx_w = oracle.bin_froxels(cam.record, lt, p, capacity=1 << 26)
    off, idx, _ = gpu_bin_froxels(ctx, cam.record, lt, p, capacity=int(off_w[-1]) + 8)
    np.testing.assert_array_equal(off, off_w)
    np.testing.assert_array_equal(idx, idx_w)


def test_froxel_binning_replays_in_a_cuda_graph(ctx):
    """hl_bin_froxels keeps its launch-to-launch state on the device, so a launch
    recorded in a CUDA graph gives the same lists on every replay, alternating with
    direct calls on other grids."""
    import torch

    from helio_gb300 import frame as FR

    w = S.workload(0, 0.5)
    W, H = w.gbuffer.width, w.gbuffer.height
    p_np = L.froxel_params(*w.froxel_grid, W, H, w.camera.far)
    off_w, idx_w = oracle.bin_froxels(w.camera.record, w.lights, p_np, capacity=1 << 24)
    p = N.froxel_params_from_numpy(p_np)
    F = p.grid_x * p.grid_y * p.grid_z
    cam, lt = FR.bytes_tensor(w.camera.record), FR.bytes_tensor(w.lights)
    cap = int(off_w[-1]) + 64
    off = torch.zeros(F + 1, dtype=torch.int32, device="cuda")
    idx = torch.zeros(cap, dtype=torch.int32, device="cuda")
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        ctx.bin_froxels(cam, lt, len(w.lights), p, off, idx, cap, s.cuda_stream)  # scratch allocated here
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        ctx.bin_froxels(cam, lt, len(w.lights), p, off, idx, cap, s.cuda_stream)
    other = L.froxel_params(5, 3, 7, W, H, w.camera.far)
    for _ in range(3):
        off.fill_(-1)
        idx.fill_(-1)
        g.replay()
        torch.cuda.synchronize()
        ctx.sync_status()
        np.testing.assert_array_equal(off.cpu().numpy().view(np.uint32), off_w)
        np.testing.assert_array_equal(idx.cpu().numpy().view(np.uint32)[: off_w[-1]], idx_w)
        o2, i2, _ = gpu_bin_froxels(ctx, w.camera.record, w.lights, other)  # a direct call in between
        o2w, i2w = oracle.bin_froxels(w.camera.record, w.lights, other, capacity=1 << 24)
        np.testing.assert_array_equal(o2, o2w)


def test_froxel_bounded_wait_times_out_and_the_context_recovers(ctx):
    """Failure detection of the single-launch binning: every work item finds where its
    lists start by polling the running totals earlier items publish, and each poll
    loop is bounded. With one item withholding its total (hl_inject_binning_stall),
    the later items give up after the given number of polls: the call reports
    HL_ERR_TIMEOUT through hl_sync_status instead of hanging, and the next call on the
    same context bins normally, bit-exact."""
    w = S.workload(1)
    p = L.froxel_params(*w.froxel_grid, w.gbuffer.width, w.gbuffer.height, w.camera.far)
    off_w, idx_w = oracle.bin_froxels(w.camera.record, w.lights, p, capacity=1 << 26)
    cap = int(off_w[-1]) + 16
    ctx.inject_binning_stall(item=5, spins=1024)
    gpu_bin_froxels(ctx, w.camera.record, w.lights, p, capacity=cap, expect_status=N.HL_ERR_TIMEOUT)
    for _ in range(2):
        off, idx, _ = gpu_bin_froxels(ctx, w.camera.record, w.lights, p, capacity=cap)
        np.testing.assert_array_equal(off, off_w)
        np.testing.assert_array_equal(idx, idx_w)
    with pytest.raises(N.HelioError) as e:
        ctx.inject_binning_stall(item=0, spins=0)
    assert e.value.status == N.HL_ERR_INVALID_ARGUMENT
