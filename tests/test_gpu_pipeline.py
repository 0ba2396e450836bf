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


def test_dependent_launch_orders(ctx):
    """The binning, light-table and shading launches start while their predecessor runs
    (programmatic dependent launches) and wait before reading its outputs. Back-to-back
    calls in any order on one stream, with no synchronisation between them, must give
    the results of the same calls synchronised one by one: binning after binning with
    and without lights, shading twice in a row, shading right after a binning without
    lights, and a second scene binned into the same buffers in between."""
    import torch

    a = S.workload(1, 0.5)
    b = S.workload(1, 0.5)
    b.lights["position_range"][:, 0] += 1.5  # a second light set of the same shape
    W, H = a.gbuffer.width, a.gbuffer.height
    p = N.froxel_params(*a.froxel_grid, W, H, a.camera.far)
    F = p.grid_x * p.grid_y * p.grid_z
    cap = F * 256
    da, db = FR.upload_workload(a), FR.upload_workload(b)
    off = torch.zeros(F + 1, dtype=torch.int32, device="cuda")
    idx = torch.zeros(cap, dtype=torch.int32, device="cuda")
    grid = N.froxel_grid_struct(idx, off, p, cap)
    outs = [torch.zeros((H, W, 4), dtype=torch.float32, device="cuda") for _ in range(4)]

    def run(sync):
        for o in outs:
            o.zero_()
        steps = [
            lambda: ctx.bin_froxels(da.camera, da.lights, 0, p, off, idx, cap),
            lambda: ctx.bin_froxels(da.camera, da.lights, 0, p, off, idx, cap),
            lambda: ctx.shade(da.camera, da.globals_, da.gbuffer, da.lights, 0, grid, N.target_struct(outs[0])),
            lambda: ctx.bin_froxels(db.camera, db.lights, db.n_lights, p, off, idx, cap),
            lambda: ctx.shade(db.camera, db.globals_, db.gbuffer, db.lights, db.n_lights, grid,
                              N.target_struct(outs[1])),
            lambda: ctx.bin_froxels(da.camera, da.lights, da.n_lights, p, off, idx, cap),
            lambda: ctx.shade(da.camera, da.globals_, da.gbuffer, da.lights, da.n_lights, grid,
                              N.target_struct(outs[2])),
            lambda: ctx.shade(da.camera, da.globals_, da.gbuffer, da.lights, da.n_lights, grid,
                              N.target_struct(outs[3])),
        ]
        for f in steps:
            f()
            if sync:
                torch.cuda.synchronize()
        ctx.sync_status()
        return [o.cpu().numpy() for o in outs] + [off.cpu().numpy(), idx[: int(off[-1])].cpu().numpy()]

    want = run(True)
    assert np.any(want[1] != want[2]), "the two scenes must differ"
    assert np.array_equal(want[2], want[3])
    for _ in range(5):
        got = run(False)
        for g, w in zip(got, want):
            assert np.array_equal(g, w)


def test_frame_replays_in_a_cuda_graph(ctx):
    """A whole frame (hl_bin_froxels + hl_shade, whose kernels are chained as dependent
    launches) recorded in a CUDA graph gives the radiance of direct calls on every replay."""
    import torch

    w = S.workload(1, 0.5)
    want = _device_radiance(ctx, w)
    df = FR.upload_workload(w)
    W, H = w.gbuffer.width, w.gbuffer.height
    p = N.froxel_params(*w.froxel_grid, W, H, w.camera.far)
    F = p.grid_x * p.grid_y * p.grid_z
    cap = F * 64
    off = torch.zeros(F + 1, dtype=torch.int32, device="cuda")
    idx = torch.zeros(cap, dtype=torch.int32, device="cuda")
    out = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    grid, tgt = N.froxel_grid_struct(idx, off, p, cap), N.target_struct(out)
    s = torch.cuda.Stream()

    def frame():
        ctx.bin_froxels(df.camera, df.lights, df.n_lights, p, off, idx, cap, s.cuda_stream)
        ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, tgt, s.cuda_stream)

    with torch.cuda.stream(s):
        frame()  # scratch allocated outside the capture
    s.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        frame()
    for _ in range(3):
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        ctx.sync_status()
        assert np.array_equal(out.cpu().numpy(), want)
