"""GPU parity of hl_shade_adjoint (the hand-written adjoint kernel) against the FP64
oracle adjoint, and of the torch.autograd wrapper against FP64 central finite
differences of the oracle's forward.

Tolerances:
  light gradients (f64 out, f32 per pair):  per component, max |gpu - oracle| <= 1e-4 x
      max |oracle| of that component;
  pixel gradients (f32): |gpu - oracle| <= 1e-3 (|oracle| + 1e-3 max |oracle|), except
      at most max(2, 1e-4 n) pixels where a cut decides differently in f32 and f64;
  autograd vs finite differences: |grad - fd| <= 1e-3 max(|grad|, |fd|) + 1e-7."""
import numpy as np
import pytest

import oracle
from helio_gb300 import frame as FR
from helio_gb300 import layouts as L
from helio_gb300 import native as N
from helio_gb300 import synthetic as S

pytestmark = pytest.mark.gpu


def _scene(seed, layout=S.LAYOUT_F32, W=96, H=64, n_point=40, n_spot=16, radius=(3.0, 9.0)):
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, layout, seed=seed)
    d = S.uniform(seed, 90, W * H, 2.0, 14.0).reshape(H, W)
    depth = ((cam.far / (cam.far - cam.near)) * (1.0 - cam.near / d)).astype(np.float32)
    sky = S.uniform(seed, 91, W * H, 0.0, 1.0).reshape(H, W) < 0.05
    depth[sky] = 1.0
    gb.planes[-1] = np.ascontiguousarray(depth)
    lt = S.make_lights(cam, seed, n_point, n_spot, radius=radius)
    lt["position_range"][:, 2] = np.clip(lt["position_range"][:, 2], -13.0, -2.0)
    d0 = L.make_lights(1)
    d0["light_type"] = L.LIGHT_DIRECTIONAL
    d0["direction_outer"] = (0.3, -0.8, -0.5, 0.0)
    d0["color_intensity"] = (0.9, 0.8, 0.7, 0.6)
    lt = np.concatenate([lt[:5], d0, lt[5:]])
    glb = L.make_globals(L.tile_grid(W, H)[0], len(lt), ambient_color=(0.5, 0.5, 0.6), ambient_intensity=0.7)
    return cam, glb, lt, gb


def _grid(cam, lt, W, H, kind, shape=(6, 4, 12)):
    import torch

    if kind == "tiles":
        lists, counts = oracle.bin_tiles_ref(cam.record, lt, W, H)
        dl = torch.from_numpy(lists.reshape(-1).view(np.int32).copy()).cuda()
        dc = torch.from_numpy(counts.view(np.int32).copy()).cuda()
        return ("tiles", lists, counts), N.tile_grid_struct(dl, dc), (dl, dc)
    p = L.froxel_params(*shape, W, H, cam.far)
    off, idx = oracle.bin_froxels(cam.record, lt, p, capacity=1 << 24)
    doff = torch.from_numpy(off.view(np.int32).copy()).cuda()
    didx = torch.from_numpy((idx if idx.size else np.zeros(1, np.uint32)).view(np.int32).copy()).cuda()
    return ("froxels", idx, off, p), N.froxel_grid_struct(didx, doff, N.froxel_params_from_numpy(p), didx.numel()), (
        didx, doff)


def _gpu_adjoint(ctx, cam, glb, lt, gb, dgrid, w, pitch_pad=0):
    import torch

    df = FR.upload(cam.record, glb, lt, gb)
    H, W = w.shape[:2]
    wt = torch.zeros(H, W + pitch_pad, 4, dtype=torch.float32, device="cuda")
    wt[:, :W] = torch.from_numpy(w.astype(np.float32)).cuda()
    d_lights = torch.full((max(len(lt), 1), 7), 7.0, dtype=torch.float64, device="cuda")
    d_pixels = torch.full((H, W, 5), 7.0, dtype=torch.float32, device="cuda")
    ctx.shade_adjoint(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, dgrid, wt,
                      wt.stride(0) * wt.element_size(), d_lights, d_pixels)
    ctx.sync_status()
    return d_lights.cpu().numpy()[: len(lt)], d_pixels.cpu().numpy().astype(np.float64)


def _check(dl, dp, odl, odp, sky):
    if len(odl):
        scale = np.abs(odl).max(0)
        err = np.abs(dl - odl).max(0)
        assert np.all(err <= 1e-4 * np.maximum(scale, 1e-30)), (err / np.maximum(scale, 1e-30)).tolist()
    assert np.all(dp[sky] == 0.0), "sky pixels get zero gradients"
    m = ~sky
    pscale = np.abs(odp[m]).max(0)
    bad = (np.abs(dp[m] - odp[m]) > 1e-3 * (np.abs(odp[m]) + 1e-3 * pscale)).any(-1)
    assert bad.sum() <= max(2, 1e-4 * m.sum()), int(bad.sum())


@pytest.mark.parametrize("kind", ["froxels", "tiles"])
@pytest.mark.parametrize("seed", [1, 2])
def test_adjoint_matches_oracle(ctx, kind, seed):
    cam, glb, lt, gb = _scene(seed)
    ogrid, dgrid, keep = _grid(cam, lt, gb.width, gb.height, kind)
    w = np.random.default_rng(seed).normal(size=(gb.height, gb.width, 4))
    dl, dp = _gpu_adjoint(ctx, cam, glb, lt, gb, dgrid, w)
    odl, odp = oracle.shade_adjoint(cam.record, glb, gb, lt, ogrid, w)
    sky = ~(gb.planes[-1] < 1.0)
    assert np.abs(odl).max() > 0 and np.abs(odp).max() > 0
    _check(dl, dp, odl, odp, sky)


@pytest.mark.parametrize("layout", [S.LAYOUT_REFERENCE, S.LAYOUT_F16])
def test_adjoint_other_layouts(ctx, layout):
    cam, glb, lt, gb = _scene(4, layout=layout)
    ogrid, dgrid, keep = _grid(cam, lt, gb.width, gb.height, "froxels")
    w = np.random.default_rng(4).normal(size=(gb.height, gb.width, 4))
    dl, dp = _gpu_adjoint(ctx, cam, glb, lt, gb, dgrid, w, pitch_pad=3)
    odl, odp = oracle.shade_adjoint(cam.record, glb, gb, lt, ogrid, w)
    _check(dl, dp, odl, odp, ~(gb.planes[-1] < 1.0))


def test_adjoint_more_lights_than_one_window(ctx):
    """700 lights: the kernel takes them in windows of 256."""
    cam, glb, lt, gb = _scene(5, n_point=560, n_spot=139, radius=(1.5, 5.0))
    pos = lt["position_range"]
    pos[:, 0] = S.uniform(5, 120, len(lt), -5.0, 5.0)  # in front of the surfaces
    pos[:, 1] = S.uniform(5, 121, len(lt), -3.5, 3.5)
    ogrid, dgrid, keep = _grid(cam, lt, gb.width, gb.height, "froxels")
    w = np.random.default_rng(5).normal(size=(gb.height, gb.width, 4))
    dl, dp = _gpu_adjoint(ctx, cam, glb, lt, gb, dgrid, w)
    odl, odp = oracle.shade_adjoint(cam.record, glb, gb, lt, ogrid, w)
    assert (np.abs(odl[256:]).max(1) > 0).sum() > 200
    _check(dl, dp, odl, odp, ~(gb.planes[-1] < 1.0))


def test_adjoint_is_deterministic(ctx):
    cam, glb, lt, gb = _scene(6, W=160, H=96)
    ogrid, dgrid, keep = _grid(cam, lt, gb.width, gb.height, "froxels")
    w = np.random.default_rng(6).normal(size=(gb.height, gb.width, 4))
    a = _gpu_adjoint(ctx, cam, glb, lt, gb, dgrid, w)
    b = _gpu_adjoint(ctx, cam, glb, lt, gb, dgrid, w)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_adjoint_without_lights(ctx):
    """No lights: only the hemisphere ambient term reaches the albedo gradient."""
    cam, glb, lt, gb = _scene(7)
    lt = lt[:0]
    ogrid, dgrid, keep = _grid(cam, lt, gb.width, gb.height, "froxels")
    w = np.random.default_rng(7).normal(size=(gb.height, gb.width, 4))
    dl, dp = _gpu_adjoint(ctx, cam, glb, lt, gb, dgrid, w)
    odl, odp = oracle.shade_adjoint(cam.record, glb, gb, lt, ogrid, w)
    assert dl.shape == (0, 7)
    _check(dl, dp, odl, odp, ~(gb.planes[-1] < 1.0))
    assert np.all(dp[..., 3:] == 0.0)


def test_adjoint_rejects_bad_arguments(ctx):
    import torch

    cam, glb, lt, gb = _scene(8, W=32, H=16, n_point=4, n_spot=0)
    ogrid, dgrid, keep = _grid(cam, lt, gb.width, gb.height, "froxels")
    df = FR.upload(cam.record, glb, lt, gb)
    wt = torch.zeros(16, 32, 4, dtype=torch.float32, device="cuda")
    dlt = torch.zeros(len(lt), 7, dtype=torch.float64, device="cuda")
    dpx = torch.zeros(16, 32, 5, dtype=torch.float32, device="cuda")
    with pytest.raises(N.HelioError) as e:
        ctx.shade_adjoint(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, dgrid, wt, 32 * 16 - 16, dlt, dpx)
    assert e.value.status == N.HL_ERR_LAYOUT
    with pytest.raises(N.HelioError) as e:
        ctx.shade_adjoint(df.camera, df.globals_, df.gbuffer, df.lights, 65537, dgrid, wt, 32 * 16, dlt, dpx)
    assert e.value.status == N.HL_ERR_SIZE


def test_autograd_wrapper_matches_finite_differences(ctx):
    """Loss = sum((radiance - target)^2), the target rendered with the lights moved by
    N(0, 0.5^2) per axis and intensities scaled by U[0.8, 1.2]. Gradients with respect
    to light position, intensity, colour and per-pixel albedo, roughness, metallic come
    from DeferredShade.backward (hl_shade_adjoint) and are checked on 32 random
    parameters against float64 central differences (h = 1e-3) of the oracle's forward."""
    import torch

    from helio_gb300 import autograd as AG

    cam, glb, lt, gb = _scene(9, W=48, H=32, n_point=10, n_spot=4)
    W, H = gb.width, gb.height
    df = FR.upload(cam.record, glb, lt, gb)
    normal = torch.from_numpy(gb.planes[1][..., :3].copy()).cuda()
    depth = torch.from_numpy(gb.planes[2].copy()).cuda()
    scene = AG.ShadeScene(ctx, df.camera, df.globals_, df.lights, normal, depth,
                          N.froxel_params(4, 2, 8, W, H, cam.far))
    lp0 = AG.light_params_of(lt)
    pp_np = np.concatenate([gb.planes[0], gb.planes[1][..., 3:4]], -1)
    rng = np.random.default_rng(9)
    moved = lp0.clone()
    is_local = torch.from_numpy(lt["light_type"] != L.LIGHT_DIRECTIONAL)
    moved[is_local, 0:3] += torch.from_numpy(rng.normal(0.0, 0.5, (int(is_local.sum()), 3)).astype(np.float32))
    moved[:, 3] *= torch.from_numpy(rng.uniform(0.8, 1.2, len(lt)).astype(np.float32))
    with torch.no_grad():
        target = AG.shade(moved.cuda(), torch.from_numpy(pp_np.copy()).cuda(), scene)
    lp = lp0.clone().cuda().requires_grad_(True)
    pp = torch.from_numpy(pp_np.copy()).cuda().requires_grad_(True)
    rad = AG.shade(lp, pp, scene)
    loss = ((rad[..., :3] - target[..., :3]) ** 2).sum()
    loss.backward()
    g_l = lp.grad.double().cpu().numpy()
    g_p = pp.grad.double().cpu().numpy()
    tgt = target.double().cpu().numpy()[..., :3]

    allp = L.froxel_params(1, 1, 1, W, H, cam.far)
    everything = ("froxels", np.arange(len(lt), dtype=np.uint32), np.array([0, len(lt)], np.uint32), allp)

    def f(lights, planes):
        r = oracle.shade(cam.record, glb, S.GBuffer(S.LAYOUT_F32, W, H, planes), lights, everything)
        r = np.nan_to_num(r)[..., :3]
        return float(((r - tgt) ** 2).sum())

    fields = [("position_range", 0), ("position_range", 1), ("position_range", 2), ("color_intensity", 3),
              ("color_intensity", 0), ("color_intensity", 1), ("color_intensity", 2)]
    pick_l = np.flatnonzero(np.abs(g_l).ravel() > 1e-3 * np.abs(g_l).max())
    pick_p = np.flatnonzero(np.abs(g_p).ravel() > 1e-3 * np.abs(g_p).max())
    pick_l = rng.choice(pick_l, 16, replace=False)
    pick_p = rng.choice(pick_p, 16, replace=False)
    h = 1e-3
    for flat in pick_l:
        li, q = np.unravel_index(flat, g_l.shape)
        field, comp = fields[q]
        v = float(lt[field][li, comp])
        lp_, lm_ = lt.copy(), lt.copy()
        lp_[field][li, comp] = np.float32(v + h)
        lm_[field][li, comp] = np.float32(v - h)
        hh = float(lp_[field][li, comp]) - float(lm_[field][li, comp])
        fd = (f(lp_, gb.planes) - f(lm_, gb.planes)) / hh
        assert abs(fd - g_l[li, q]) <= 1e-3 * max(abs(fd), abs(g_l[li, q])) + 1e-6, (li, q, fd, g_l[li, q])
    for flat in pick_p:
        y, x, q = np.unravel_index(flat, g_p.shape)
        plane, comp = (0, q) if q < 4 else (1, 3)
        v = float(gb.planes[plane][y, x, comp])
        pl_p = [p.copy() for p in gb.planes]
        pl_m = [p.copy() for p in gb.planes]
        pl_p[plane][y, x, comp] = np.float32(v + h)
        pl_m[plane][y, x, comp] = np.float32(v - h)
        hh = float(pl_p[plane][y, x, comp]) - float(pl_m[plane][y, x, comp])
        fd = (f(lt, pl_p) - f(lt, pl_m)) / hh
        assert abs(fd - g_p[y, x, q]) <= 1e-3 * max(abs(fd), abs(g_p[y, x, q])) + 1e-6, ((y, x, q), fd, g_p[y, x, q])


def test_autograd_matches_finite_differences_at_the_differentiation_workload():
    """The differentiation workload at its own shape: 1920x1080 FP32 G-buffer, 256 point
    lights, target rendered by the FP64 oracle with the lights moved by N(0, 0.5^2) per
    axis and intensities scaled by U[0.8, 1.2], loss = sum((radiance - target)^2).
    Gradients from DeferredShade.backward (hl_shade_adjoint) against FP64 central
    differences (h = 1e-3) on 32 random parameters (16 light, 16 pixel). The FP64
    forward holds the kernel's own branch decisions at the cuts of pbr_direct_light
    (recorded with hl_set_pair_log), as the adjoint does, and evaluates only the rows a
    parameter reaches. A parameter whose differences at h and h/2 disagree sits at a
    kink of a clamp (range falloff, NdL, spot cone) and is replaced by another."""
    import torch

    from helio_gb300 import autograd as AG

    w = S.workload(4)
    cam, gb, lt, glb = w.camera, w.gbuffer, w.lights, w.globals_
    W, H = gb.width, gb.height
    p_np = L.froxel_params(*w.froxel_grid, W, H, cam.far)
    moved = S.perturbed_lights(lt, 4500)
    off_t, idx_t = oracle.bin_froxels(cam.record, moved, p_np, capacity=1 << 26)
    tgt = np.nan_to_num(oracle.shade(cam.record, glb, gb, moved, ("froxels", idx_t, off_t, p_np)))[..., :3]

    with N.Context(0) as ctx:
        df = FR.upload(cam.record, glb, lt, gb)
        normal = torch.from_numpy(gb.planes[1][..., :3].copy()).cuda()
        depth = torch.from_numpy(gb.planes[2].copy()).cuda()
        scene = AG.ShadeScene(ctx, df.camera, df.globals_, df.lights, normal, depth,
                              N.froxel_params_from_numpy(p_np), capacity=1 << 24)
        pp_np = np.concatenate([gb.planes[0], gb.planes[1][..., 3:4]], -1)
        lp = AG.light_params_of(lt).cuda().requires_grad_(True)
        pp = torch.from_numpy(pp_np.copy()).cuda().requires_grad_(True)
        pairs_d = torch.zeros((W * H * 4, 2), dtype=torch.int32, device="cuda")
        count = torch.zeros(1, dtype=torch.int32, device="cuda")
        ctx.set_pair_log(pairs_d, count)
        rad = AG.shade(lp, pp, scene)
        ctx.set_pair_log(None)
        loss = ((rad[..., :3] - torch.from_numpy(tgt.astype(np.float32)).cuda()) ** 2).sum()
        loss.backward()
        ctx.sync_status()
        n = int(count.item())
        assert n <= pairs_d.shape[0]
        pairs = pairs_d[:n].cpu().numpy().view(np.uint32)
        g_l = lp.grad.double().cpu().numpy()
        g_p = pp.grad.double().cpu().numpy()

    off, idx = oracle.bin_froxels(cam.record, lt, p_np, capacity=1 << 26)
    grid = ("froxels", idx, off, p_np)
    csr = oracle.forced_csr(pairs, W * H)
    pix_of = pairs[:, 0].astype(np.int64)

    def loss_rows(lights, planes, r0, r1):
        r, _, unlisted = oracle.shade_forced(cam.record, glb, S.GBuffer(S.LAYOUT_F32, W, H, planes), lights, grid, csr,
                                             rows=(r0, r1))
        assert unlisted.sum() == 0
        r = np.nan_to_num(r[r0:r1])[..., :3]
        return float(((r - tgt[r0:r1]) ** 2).sum())

    fields = [("position_range", 0), ("position_range", 1), ("position_range", 2), ("color_intensity", 3),
              ("color_intensity", 0), ("color_intensity", 1), ("color_intensity", 2)]

    def fd_light(li, q, h):
        field, comp = fields[q]
        ys = pix_of[pairs[:, 1] == li] // W
        r0, r1 = int(ys.min()), int(ys.max()) + 1
        v = float(lt[field][li, comp])
        lp_, lm_ = lt.copy(), lt.copy()
        lp_[field][li, comp] = np.float32(v + h)
        lm_[field][li, comp] = np.float32(v - h)
        hh = float(lp_[field][li, comp]) - float(lm_[field][li, comp])
        return (loss_rows(lp_, gb.planes, r0, r1) - loss_rows(lm_, gb.planes, r0, r1)) / hh

    def fd_pixel(y, x, q, h):
        plane, comp = (0, q) if q < 4 else (1, 3)
        v = float(gb.planes[plane][y, x, comp])
        pl_p = [p.copy() for p in gb.planes]
        pl_m = [p.copy() for p in gb.planes]
        pl_p[plane][y, x, comp] = np.float32(v + h)
        pl_m[plane][y, x, comp] = np.float32(v - h)
        hh = float(pl_p[plane][y, x, comp]) - float(pl_m[plane][y, x, comp])
        return (loss_rows(lt, pl_p, y, y + 1) - loss_rows(lt, pl_m, y, y + 1)) / hh

    rng = np.random.default_rng(4)
    h = 1e-3
    lit_lights = np.unique(pairs[:, 1])
    cand_l = [int(f) for f in rng.permutation(np.flatnonzero(np.abs(g_l).ravel() > 1e-3 * np.abs(g_l).max()))
              if f // 7 in set(lit_lights.tolist())]
    cand_p = rng.permutation(np.flatnonzero(np.abs(g_p).ravel() > 1e-3 * np.abs(g_p).max()))
    checked = {"light": 0, "pixel": 0}
    kinks = 0
    for kind, cands in (("light", cand_l), ("pixel", cand_p)):
        for flat in cands:
            if checked[kind] == 16:
                break
            if kind == "light":
                li, q = divmod(int(flat), 7)
                fd, fd2, g = fd_light(li, q, h), fd_light(li, q, h / 2), g_l[li, q]
            else:
                y, x, q = np.unravel_index(int(flat), g_p.shape)
                fd, fd2, g = fd_pixel(y, x, q, h), fd_pixel(y, x, q, h / 2), g_p[y, x, q]
            if abs(fd - fd2) > 1e-4 * max(abs(fd), abs(fd2), 1e-12):
                kinks += 1
                continue
            assert abs(fd - g) <= 1e-3 * max(abs(fd), abs(g)) + 1e-7, (kind, int(flat), fd, g)
            checked[kind] += 1
    assert checked == {"light": 16, "pixel": 16}, (checked, kinks)
    assert kinks <= 16, kinks
