"""GPU tests of the batched-views plan (hl_batch_plan_create / hl_batch_execute): one
graph of six launches lights every view against one light buffer. Each view's
radiance must be bit-identical to the single-view path (hl_bin_froxels + hl_shade with
the grid the plan chose), since both run the same binning and shading code; a few views
are also checked against the float64 oracle (FP16 G-buffer tolerance 2e-3)."""
import numpy as np
import pytest

import oracle
from helio_gb300 import frame as FR
from helio_gb300 import layouts as L
from helio_gb300 import metrics
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


class Batch:
    """Device buffers of a scaled batched-views workload."""

    def __init__(self, scale=0.125, layout=S.LAYOUT_F16, views=None):
        import torch

        vs, lights = S.batched_views(scale, layout)
        if views is not None:
            vs = [vs[i] for i in views]
        self.views, self.lights_np = vs, lights
        self.globals_np = L.make_globals(1, len(lights), ambient_color=(0.4, 0.45, 0.5), ambient_intensity=0.3)
        self.lights = FR.bytes_tensor(lights)
        self.globals_ = FR.bytes_tensor(self.globals_np)
        self.frames = [FR.upload(v.camera.record, self.globals_np, lights, v.gbuffer) for v in vs]
        self.out = [torch.full((v.gbuffer.height, v.gbuffer.width, 4), 7.0, dtype=torch.float32, device="cuda")
                    for v in vs]

    def structs(self):
        return [N.view_struct(f.camera, f.gbuffer, N.target_struct(o)) for f, o in zip(self.frames, self.out)]

    def single_view(self, ctx, v, grid):
        """hl_bin_froxels + hl_shade of view v with froxel grid `grid`."""
        import torch

        f = self.frames[v]
        cam = self.views[v].camera
        p = N.froxel_params(*grid, f.width, f.height, cam.far)
        F = grid[0] * grid[1] * grid[2]
        cap = F * len(self.lights_np)
        off = torch.zeros(F + 1, dtype=torch.int32, device="cuda")
        idx = torch.zeros(cap, dtype=torch.int32, device="cuda")
        ctx.bin_froxels(f.camera, self.lights, len(self.lights_np), p, off, idx, cap)
        out = torch.full((f.height, f.width, 4), 7.0, dtype=torch.float32, device="cuda")
        ctx.shade(f.camera, self.globals_, f.gbuffer, self.lights, len(self.lights_np),
                  N.froxel_grid_struct(idx, off, p, cap), N.target_struct(out))
        ctx.sync_status()
        return out.cpu().numpy(), (off.cpu().numpy().view(np.uint32), idx.cpu().numpy().view(np.uint32), p)


def test_batch_matches_single_view_path(ctx):
    b = Batch()
    with ctx.batch_plan(b.structs(), b.lights, len(b.lights_np), b.globals_, grid=(4, 4, 16)) as plan:
        plan.execute()
        ctx.sync_status()
        got = [o.cpu().numpy() for o in b.out]
        for v in range(len(b.views)):
            g = plan.view_grid(v)
            assert g == (min(4, b.views[v].gbuffer.width), min(4, b.views[v].gbuffer.height), 16)
            want, _ = b.single_view(ctx, v, g)
            assert np.array_equal(got[v], want), f"view {v}"


def test_batch_views_match_oracle(ctx):
    b = Batch(views=[0, 40, 95, 96])
    with ctx.batch_plan(b.structs(), b.lights, len(b.lights_np), b.globals_, grid=(4, 4, 16)) as plan:
        plan.execute()
        ctx.sync_status()
        for v in range(len(b.views)):
            img = b.out[v].cpu().numpy().astype(np.float64)
            vw = b.views[v]
            _, (off, idx, p) = b.single_view(ctx, v, plan.view_grid(v))
            pn = L.froxel_params(p.grid_x, p.grid_y, p.grid_z, p.width, p.height, p.slice_far, p.slice_near)
            ref = oracle.shade(vw.camera.record, b.globals_np, vw.gbuffer, b.lights_np,
                               ("froxels", idx[: off[-1]], off, pn))
            e = metrics.radiance_error(img, ref)
            assert e["max"] <= 2e-3, (v, e)


def test_batch_replays_read_live_light_buffer(ctx):
    """The graph reads the light buffer at each execution: change intensities in
    place, execute again, and the result follows the single-view path."""
    b = Batch(views=[3, 50, 96])
    with ctx.batch_plan(b.structs(), b.lights, len(b.lights_np), b.globals_, grid=(8, 4, 24)) as plan:
        plan.execute()
        ctx.sync_status()
        first = [o.cpu().numpy() for o in b.out]
        lt = b.lights_np.copy()
        lt["color_intensity"][:, 3] *= 1.5
        b.lights.copy_(FR.bytes_tensor(lt))
        b.lights_np = lt
        plan.execute()
        plan.execute()
        ctx.sync_status()
        for v in range(3):
            got = b.out[v].cpu().numpy()
            want, _ = b.single_view(ctx, v, plan.view_grid(v))
            assert np.array_equal(got, want)
            assert not np.array_equal(got, first[v])


def test_batch_autotune_writes_and_reads_cache(ctx, tmp_path):
    b = Batch(views=[0, 1, 40, 96])
    cache = tmp_path / "tune.txt"
    with ctx.batch_plan(b.structs(), b.lights, len(b.lights_np), b.globals_, autotune=True,
                        cache_path=str(cache)) as plan:
        grids = [plan.view_grid(v) for v in range(4)]
    assert grids[0] == grids[1], "views of one size share a grid"
    lines = [l for l in cache.read_text().splitlines() if not l.startswith("#")]
    assert len(lines) == 3, lines  # three view sizes
    # a cache entry is used as given
    w, h = b.views[3].gbuffer.width, b.views[3].gbuffer.height
    edited = []
    for l in lines:
        f = l.split()
        if int(f[0]) == w and int(f[1]) == h:
            f[-3:] = ["3", "2", "8"]
        edited.append(" ".join(f))
    cache.write_text("\n".join(edited) + "\n")
    with ctx.batch_plan(b.structs(), b.lights, len(b.lights_np), b.globals_, autotune=True,
                        cache_path=str(cache)) as plan:
        assert plan.view_grid(3) == (3, 2, 8)
        assert plan.view_grid(0) == grids[0]
        plan.execute()
        ctx.sync_status()
        want, _ = b.single_view(ctx, 3, (3, 2, 8))
        assert np.array_equal(b.out[3].cpu().numpy(), want)


def test_batch_rejects_mixed_layouts(ctx):
    b16 = Batch(views=[0])
    b32 = Batch(views=[1], layout=S.LAYOUT_F32)
    views = b16.structs() + b32.structs()
    with pytest.raises(N.HelioError) as e:
        ctx.batch_plan(views, b16.lights, len(b16.lights_np), b16.globals_, grid=(4, 4, 16))
    assert e.value.status == N.HL_ERR_NOT_SUPPORTED
    with pytest.raises(N.HelioError) as e:
        ctx.batch_plan(b16.structs(), b16.lights, len(b16.lights_np), b16.globals_, grid=(0, 4, 16))
    assert e.value.status == N.HL_ERR_INVALID_ARGUMENT
