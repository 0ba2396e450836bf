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
