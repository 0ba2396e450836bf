"""GPU parity of hl_shade_fragments (the Forward+ and transparent light loops over the
same tile / froxel lists) against the float64 oracle.

Tolerance per fragment, relative over RGB with a floor of 1e-6 x the largest value:
p99.99 <= 1e-5 and max <= 1e-3 (the precise FP32 path), except fragments where a cut
(range, NdL = 0, the transparent mode's 0.002) decides differently in f32 and f64, which
must be at most max(2, 1e-3 n). Discarded fragments (forward mode, alpha <= 0.001) keep
the output buffer's previous contents."""
import numpy as np
import pytest

import oracle
from helio_gb300 import layouts as L
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

from scenes import fragment_params, fragments, mixed_lights

pytestmark = pytest.mark.gpu


def _scene(seed, n=20000, W=320, H=180, n_point=120, n_spot=40):
    cam = S.make_camera((0.2, 0.1, 0.3), (0.0, 0.0, -8.0), (0, 1, 0), 60.0, W, H)
    lt = mixed_lights(cam, seed, n_point=n_point, n_spot=n_spot, n_dir=2)
    fr = fragments(cam, seed, n)
    return cam, lt, fr


def _grid(cam, lt, kind):
    import torch

    W, H = cam.width, cam.height
    if kind == "tiles":
        lists, counts = oracle.bin_tiles_ref(cam.record, lt, W, H)
        dl = torch.from_numpy(lists.reshape(-1).view(np.int32).copy()).cuda()
        dc = torch.from_numpy(counts.view(np.int32).copy()).cuda()
        g = N.tile_grid_struct(dl, dc)
        g.lists_capacity = dl.numel()
        return ("tiles", lists, counts), g, (dl, dc)
    p = L.froxel_params(8, 6, 16, W, H, cam.far)
    off, idx = oracle.bin_froxels(cam.record, lt, p, capacity=1 << 24)
    doff = torch.from_numpy(off.view(np.int32).copy()).cuda()
    didx = torch.from_numpy((idx if idx.size else np.zeros(1, np.uint32)).view(np.int32).copy()).cuda()
    return ("froxels", idx, off, p), N.froxel_grid_struct(didx, doff, N.froxel_params_from_numpy(p), didx.numel()), (
        didx, doff)


def _run(ctx, cam, lt, fr, prm, dgrid, entity=None, xf=None, expect=N.HL_OK):
    import torch

    from helio_gb300 import frame as FR

    d_cam, d_lt = FR.bytes_tensor(cam.record), FR.bytes_tensor(lt)
    d_fr = FR.bytes_tensor(fr)
    out = torch.full((len(fr), 4), 7.0, dtype=torch.float32, device="cuda")
    d_ent = torch.from_numpy(entity.view(np.int32).copy()).cuda() if entity is not None else None
    d_xf = FR.bytes_tensor(xf) if xf is not None else None
    p = N.FragmentParams(int(prm["mode"][0]), int(prm["num_tiles_x"][0]), float(prm["ambient_intensity"][0]),
                         (N.C.c_float * 3)(*[float(v) for v in prm["ambient_color"][0]]))
    ctx.shade_fragments(d_cam, p, d_fr, len(fr), d_lt, len(lt), dgrid, out, entity_indices=d_ent, transforms=d_xf,
                        n_transforms=len(xf) if xf is not None else 0)
    status = N.HL_OK
    try:
        ctx.sync_status()
    except N.HelioError as e:
        status = e.status
    assert status == expect
    return out.cpu().numpy().astype(np.float64)


def _check(got, want, alpha, mode):
    keep = ~np.isnan(want[:, 0])
    if mode == L.FRAGMENTS_FORWARD:
        assert np.array_equal(keep, alpha > 0.001)
        assert np.all(got[~keep] == 7.0), "discarded fragments keep the previous output"
    g, w = got[keep][:, :3], want[keep][:, :3]
    floor = 1e-6 * np.abs(w).max()
    rel = (np.abs(g - w) / np.maximum(np.abs(w), floor)).max(1)
    bad = rel > 1e-3
    assert bad.sum() <= max(2, 1e-3 * keep.sum()), (int(bad.sum()), float(rel.max()))
    ok = rel[~bad]
    assert np.quantile(ok, 0.9999) <= 1e-5 and ok.max() <= 1e-3, float(ok.max())
    np.testing.assert_array_equal(got[keep][:, 3], want[keep][:, 3])
    assert (w > 0).any(1).mean() > 0.5, "most fragments should be lit"


@pytest.mark.parametrize("kind", ["tiles", "froxels"])
@pytest.mark.parametrize("mode", [L.FRAGMENTS_FORWARD, L.FRAGMENTS_TRANSPARENT])
def test_fragments_match_oracle(ctx, kind, mode):
    cam, lt, fr = _scene(31 + mode)
    ogrid, dgrid, keep = _grid(cam, lt, kind)
    prm = fragment_params(mode, L.tile_grid(cam.width, cam.height)[0])
    got = _run(ctx, cam, lt, fr, prm, dgrid)
    want = oracle.shade_fragments(cam.record, prm, fr, lt, ogrid)
    _check(got, want, fr["alpha"], mode)


def test_forward_fragments_read_light_transforms(ctx):
    """Forward+ reads light positions and directions from the scene transforms through
    the entity indices (forward_lit.wgsl:470-480); an index past the transforms drops
    its light and is reported."""
    cam, lt, fr = _scene(41)
    n = len(lt)
    rng = np.random.default_rng(41)
    rot = rng.uniform(-180, 180, (n, 3)).astype(np.float32)
    perm = rng.permutation(n).astype(np.uint32)
    xf = np.zeros(n, L.TRANSFORM)
    xf["position"][perm] = lt["position_range"][:, :3]
    xf["rotation"][perm] = rot
    lt_stale = lt.copy()
    lt_stale["position_range"][:, :3] = 0.0  # the records' own xyz are stale in this pass
    lt_stale["direction_outer"][:, :3] = (0.0, -1.0, 0.0)
    ogrid, dgrid, keep = _grid(cam, lt, "tiles")  # lists binned from the live positions
    prm = fragment_params(L.FRAGMENTS_FORWARD, L.tile_grid(cam.width, cam.height)[0])
    got = _run(ctx, cam, lt_stale, fr, prm, dgrid, entity=perm, xf=xf)
    want = oracle.shade_fragments(cam.record, prm, fr, lt_stale, ogrid, entity_indices=perm, transforms=xf)
    _check(got, want, fr["alpha"], L.FRAGMENTS_FORWARD)
    bad = perm.copy()
    bad[int(np.flatnonzero(lt["light_type"] == L.LIGHT_DIRECTIONAL)[0])] = n + 3
    got = _run(ctx, cam, lt_stale, fr, prm, dgrid, entity=bad, xf=xf, expect=N.HL_ERR_DEVICE_BOUNDS)
    want = oracle.shade_fragments(cam.record, prm, fr, lt_stale, ogrid, entity_indices=bad, transforms=xf)
    _check(got, want, fr["alpha"], L.FRAGMENTS_FORWARD)


def test_fragments_argument_errors(ctx):
    import torch

    cam, lt, fr = _scene(43, n=64)
    ogrid, dgrid, keep = _grid(cam, lt, "tiles")
    prm = fragment_params(7, 20)
    with pytest.raises(N.HelioError) as e:
        _run(ctx, cam, lt, fr, prm, dgrid)
    assert e.value.status == N.HL_ERR_INVALID_ARGUMENT
    dgrid.lists_capacity = 0
    with pytest.raises(N.HelioError) as e:
        _run(ctx, cam, lt, fr, fragment_params(L.FRAGMENTS_FORWARD, 20), dgrid)
    assert e.value.status == N.HL_ERR_INVALID_ARGUMENT
    del torch
