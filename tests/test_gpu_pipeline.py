"""HostFramePipeline (frames from pinned host memory, copies overlapping kernels on
three streams) must return exactly the radiance of the device-resident path, for every
frame, with frames alternating between two different scenes."""
import numpy as np
import pytest

from helio_gb300 import frame as FR
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _device_radiance(ctx, w):
    import torch

    df = FR.upload_workload(w)
    W, H = w.gbuffer.width, w.gbuffer.height
    p = N.froxel_params(*w.froxel_grid, W, H, w.camera.far)
    F = p.grid_x * p.grid_y * p.grid_z
    cap = F * 64
    off = torch.zeros(F + 1, dtype=torch.int32, device="cuda")
    idx = torch.zeros(cap, dtype=torch.int32, device="cuda")
    out = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    ctx.bin_froxels(df.camera, df.lights, df.n_lights, p, off, idx, cap)
    ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, N.froxel_grid_struct(idx, off, p, cap),
              N.target_struct(out))
    ctx.sync_status()
    return out.cpu().numpy()


def test_pipeline_matches_device_path(ctx):
    import torch

    a = S.workload(1, 0.25)
    b = S.workload(1, 0.25)
    b.lights["color_intensity"][:, 3] *= 0.5  # a second scene of the same shape
    want = [_device_radiance(ctx, a), _device_radiance(ctx, b)]
    frames = [FR.PackedFrame(a.camera.record, a.globals_, a.lights, a.gbuffer),
              FR.PackedFrame(b.camera.record, b.globals_, b.lights, b.gbuffer)]
    W, H = a.gbuffer.width, a.gbuffer.height
    cap = a.froxel_grid[0] * a.froxel_grid[1] * a.froxel_grid[2] * 64
    pipe = FR.HostFramePipeline(ctx, frames[0], a.froxel_grid, a.camera.far, capacity=cap)
    outs = [torch.full((H, W, 4), -1.0, dtype=torch.float32).pin_memory() for _ in range(6)]
    for k in range(6):
        pipe.submit(frames[k % 2], outs[k])
    pipe.synchronize()
    ctx.sync_status()
    for k in range(6):
        assert np.array_equal(outs[k].numpy(), want[k % 2]), f"frame {k}"
