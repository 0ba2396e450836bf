"""hl_bin_froxels_noalloc: the froxel clustering entry point for callers that cannot
allocate device memory (frame code inside a CUDA stream capture, or engines whose pool
owns all device memory). Its scratch is a static device array shared by every call, so
this test calls it twice in a row with different scenes and checks each result against
hl_bin_froxels (which takes its scratch from a context): the lists are integers and
must match exactly. Named to be collected last."""
import numpy as np
import pytest

from helio_gb300 import frame as FR
from helio_gb300 import layouts as L
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _with_context(ctx, w, p, cap):
    off, idx = _buffers(p, cap)
    df = FR.upload_workload(w)
    ctx.bin_froxels(df.camera, df.lights, df.n_lights, N.froxel_params_from_numpy(p), off, idx, cap)
    ctx.sync_status()
    return _host(off, idx)


def _buffers(p, cap):
    import torch

    F = int(p["grid_x"][0] * p["grid_y"][0] * p["grid_z"][0])
    off = torch.full((F + 1,), -1, dtype=torch.int32, device="cuda")
    idx = torch.full((cap,), -1, dtype=torch.int32, device="cuda")
    return off, idx


def _host(off, idx):
    import torch

    torch.cuda.synchronize()
    o = off.cpu().numpy().view(np.uint32)
    return o, idx.cpu().numpy().view(np.uint32)[: int(o[-1])]


def test_noalloc_matches_context_entry_point_twice(ctx):
    import torch

    cases = [S.workload(1), S.workload(0)]  # 1080p x 1024 lights, then 720p x 64 lights
    for w in cases:
        p = L.froxel_params(*w.froxel_grid, w.gbuffer.width, w.gbuffer.height, w.camera.far)
        cap = 1 << 20
        want_off, want_idx = _with_context(ctx, w, p, cap)
        off, idx = _buffers(p, cap)
        df = FR.upload_workload(w)
        N.bin_froxels_noalloc(df.camera, df.lights, df.n_lights, N.froxel_params_from_numpy(p), off, idx, cap)
        got_off, got_idx = _host(off, idx)
        np.testing.assert_array_equal(got_off, want_off)
        np.testing.assert_array_equal(got_idx, want_idx)
    torch.cuda.synchronize()


def test_noalloc_rejects_sizes_beyond_its_limit(built_library):
    cam = S.default_camera(64, 64)
    p = N.froxel_params(16, 9, 24, 64, 64, 100.0)
    # the limits are checked before any device work: plain host pointers suffice here
    with pytest.raises(N.HelioError) as e:
        N.bin_froxels_noalloc(16, 16, N.NOALLOC_MAX_LIGHTS + 1, p, 16, 16, 16)
    assert e.value.status == N.HL_ERR_SIZE
    big = N.froxel_params(64, 64, 16, 640, 640, 100.0)  # 65536 froxels
    with pytest.raises(N.HelioError) as e:
        N.bin_froxels_noalloc(16, 16, 8, big, 16, 16, 16)
    assert e.value.status == N.HL_ERR_SIZE
    del cam


def test_noalloc_replays_in_a_cuda_graph_after_warm_up(ctx):
    """The use the entry point exists for: one warm-up call on the device (the scratch
    address is looked up there), then the call recorded inside a stream capture, where
    nothing may allocate. Every replay gives the lists of the oracle."""
    import torch

    import oracle

    w = S.workload(0, 0.5)
    W, H = w.gbuffer.width, w.gbuffer.height
    p_np = L.froxel_params(*w.froxel_grid, W, H, w.camera.far)
    off_w, idx_w = oracle.bin_froxels(w.camera.record, w.lights, p_np, capacity=1 << 24)
    p = N.froxel_params_from_numpy(p_np)
    cap = int(off_w[-1]) + 64
    off, idx = _buffers(p_np, cap)
    df = FR.upload_workload(w)
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        N.bin_froxels_noalloc(df.camera, df.lights, df.n_lights, p, off, idx, cap, s.cuda_stream)  # warm-up
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        N.bin_froxels_noalloc(df.camera, df.lights, df.n_lights, p, off, idx, cap, s.cuda_stream)
    for _ in range(3):
        off.fill_(-1)
        idx.fill_(-1)
        g.replay()
        got_off, got_idx = _host(off, idx)
        np.testing.assert_array_equal(got_off, off_w)
        np.testing.assert_array_equal(got_idx, idx_w)


def test_noalloc_overflow_shows_in_the_total_and_keeps_the_prefix(ctx):
    """With no device status word, a total above the capacity shows as
    offsets[F] > capacity: the offsets are all written, and the entries below the
    capacity are the true lists' first entries, nothing is written beyond it."""
    import torch

    import oracle

    w = S.workload(1, 0.5)
    W, H = w.gbuffer.width, w.gbuffer.height
    p_np = L.froxel_params(*w.froxel_grid, W, H, w.camera.far)
    off_w, idx_w = oracle.bin_froxels(w.camera.record, w.lights, p_np, capacity=1 << 24)
    total = int(off_w[-1])
    cap = total // 3
    assert cap > 0
    off, idx_full = _buffers(p_np, cap + 256)
    idx = idx_full[:cap]
    df = FR.upload_workload(w)
    N.bin_froxels_noalloc(df.camera, df.lights, df.n_lights, N.froxel_params_from_numpy(p_np), off, idx, cap)
    torch.cuda.synchronize()
    got_off = off.cpu().numpy().view(np.uint32)
    got = idx_full.cpu().numpy().view(np.uint32)
    assert got_off[-1] == total > cap
    np.testing.assert_array_equal(got_off, off_w)
    np.testing.assert_array_equal(got[:cap], idx_w[:cap])
    assert (got[cap:] == 0xFFFFFFFF).all()  # the guard words past the capacity are untouched
