"""The CPU oracle, pinned: golden vectors from an independent 50-digit restatement,
closed-form known-answer cases of pbr_direct_light / fs_main and light_cull, the
conservativeness of froxel lists, and the FP64 adjoint against finite differences.
(The reference's own tests for this path pin no lighting value; see the oracle's
header.) CPU only."""
import math
from pathlib import Path

import numpy as np
import pytest

import oracle
from helio_gb300 import layouts as L
from helio_gb300 import synthetic as S

from scenes import (directional_light, fragment_params, fragments, mixed_lights, overlapping_lights,
                    point_light, spot_light)

GOLDEN = Path(__file__).resolve().parent / "golden" / "shade_golden.npz"
PI = 3.14159265359


# ----------------------------------------------------------------------------------
# golden vectors
# ----------------------------------------------------------------------------------


@pytest.mark.parametrize("k", [0, 1])
def test_shade_matches_golden_vectors(k):
    g = np.load(GOLDEN)
    planes = [g[f"s{k}_plane{i}"] for i in range(3)]
    H, W = planes[2].shape
    gb = S.GBuffer(S.LAYOUT_F32, W, H, planes)
    lt = g[f"s{k}_lights"]
    tiles = (np.arange(64, dtype=np.uint32)[None, :].repeat(L.tile_grid(W, H)[0] * L.tile_grid(W, H)[1], 0))
    counts = np.full(len(tiles), len(lt), np.uint32)
    assert len(lt) <= 64
    got = oracle.shade(g[f"s{k}_camera"], g[f"s{k}_globals"], gb, lt, ("tiles", tiles, counts))
    want = g[f"s{k}_radiance"]
    m = ~np.isnan(want[..., 0])
    assert m.sum() > 0.9 * m.size
    lit = (want[..., :3] > 0).any(-1)
    assert lit.mean() > 0.5, "golden scene should light most pixels"
    np.testing.assert_allclose(got[m], want[m], rtol=1e-11, atol=1e-14)


# ----------------------------------------------------------------------------------
# known-answer cases
# ----------------------------------------------------------------------------------


def _one_pixel(depth_view=10.0, normal=(0.0, 0.0, 1.0), albedo=(0.8, 0.6, 0.4), rough=0.5, metal=0.0):
    cam = S.default_camera(1, 1)
    gb = S.make_gbuffer(cam, S.LAYOUT_F32, seed=1)
    z = (cam.far / (cam.far - cam.near)) * (1.0 - cam.near / depth_view)
    gb.planes[2][:] = np.float32(z)
    gb.planes[0][0, 0] = (*albedo, rough)
    gb.planes[1][0, 0] = (*normal, metal)
    # exact world position of the pixel centre in float64 (ndc = (0, 0))
    m = cam.record[0]["inv_view_proj"].astype(np.float64).reshape(4, 4).T
    h = m @ np.array([0.0, 0.0, float(gb.planes[2][0, 0]), 1.0])
    return cam, gb, h[:3] / h[3]


def _shade_one(cam, gb, lights, ambient=0.0):
    glb = L.make_globals(1, len(lights), ambient_color=(0.5, 0.5, 0.6), ambient_intensity=ambient)
    tiles = np.zeros((1, 64), np.uint32)
    tiles[0, : len(lights)] = np.arange(len(lights))
    return oracle.shade(cam.record, glb, gb, lights, ("tiles", tiles, np.array([len(lights)], np.uint32)))[0, 0]


def _closed_form_on_axis(h, r, color, inten, albedo, rough, metal, spot=1.0):
    """Light straight along N = V: L = H = N, HdV = 1 so F = F0, NdH = 1."""
    a2 = rough ** 4
    D = a2 / (PI * a2 * a2 + 1e-4)
    k = (rough + 1) ** 2 / 8
    G = (1.0 / (1.0 * (1 - k) + k + 1e-4)) ** 2
    atten = 1.0 / (h * h + 1e-4) * max(0.0, 1 - (h / r) ** 4) * spot
    out = []
    for c, al in zip(color, albedo):
        F0 = min(max(0.04 * (1 - metal) + al * metal, 0.0), 0.999)
        spec = D * G * F0 / (4 * 1 * 1 + 1e-4)
        kd = (1 - F0) * (1 - metal)
        out.append((kd * al / PI + spec) * (c * inten * atten) * 1.0)
    return np.array(out)


def test_kat_point_light_on_normal():
    cam, gb, P = _one_pixel()
    r, color, inten = 5.0, (1.0, 0.5, 0.25), 3.0
    lt = point_light((P[0], P[1], P[2] + 2.0), r, color, inten)
    h = float(lt["position_range"][0, 2]) - P[2]
    got = _shade_one(cam, gb, lt)
    want = _closed_form_on_axis(h, r, color, inten, (0.8, 0.6, 0.4), 0.5, 0.0)
    np.testing.assert_allclose(got[:3], want, rtol=1e-6)  # gbuffer albedo is f32
    assert got[3] == 1.0


def test_kat_metallic_and_rough_extremes():
    for rough, metal in ((0.05, 1.0), (1.0, 0.0), (0.3, 1.0)):
        cam, gb, P = _one_pixel(rough=rough, metal=metal)
        lt = point_light((P[0], P[1], P[2] + 1.5), 4.0, (0.7, 0.7, 0.7), 2.0)
        h = float(lt["position_range"][0, 2]) - P[2]
        got = _shade_one(cam, gb, lt)
        alb = tuple(float(v) for v in gb.planes[0][0, 0, :3])
        want = _closed_form_on_axis(h, 4.0, (0.7, 0.7, 0.7), 2.0, alb, float(np.float32(rough)), metal)
        np.testing.assert_allclose(got[:3], want, rtol=1e-6)


def test_kat_light_at_range_gives_zero():
    cam, gb, P = _one_pixel()
    lt = point_light((P[0], P[1], P[2] + 3.0), 3.0)
    lt["position_range"][0, 3] = np.float32(float(lt["position_range"][0, 2]) - P[2])  # dist == range (to f32)
    got = _shade_one(cam, gb, lt)
    assert np.all(got[:3] == 0.0)


def test_kat_light_behind_surface_gives_zero():
    cam, gb, P = _one_pixel()
    lt = point_light((P[0], P[1], P[2] - 1.0), 5.0, intensity=10.0)
    assert np.all(_shade_one(cam, gb, lt)[:3] == 0.0)


def test_kat_radiance_cut_at_0002():
    cam, gb, P = _one_pixel()
    h, r = 2.0, 50.0
    lt = point_light((P[0], P[1], P[2] + h), r)
    hh = float(lt["position_range"][0, 2]) - P[2]
    atten = 1.0 / (hh * hh + 1e-4) * (1 - (hh / r) ** 4)
    for scale, lit in ((0.0019, False), (0.0021, True)):
        lt["color_intensity"][0] = (1.0, 1.0, 1.0, scale / atten)
        got = _shade_one(cam, gb, lt)
        assert (got[:3] > 0).all() == lit


def test_kat_spot_edges():
    cam, gb, P = _one_pixel()
    pos = (P[0], P[1], P[2] + 2.0)
    base = _shade_one(cam, gb, point_light(pos, 5.0, intensity=3.0))
    inside = spot_light(pos, 5.0, (0, 0, -1), 30.0, 20.0, intensity=3.0)  # axis on the pixel: cos_a = 1 >= inner
    np.testing.assert_allclose(_shade_one(cam, gb, inside)[:3], base[:3], rtol=1e-12)
    edge = spot_light(pos, 5.0, (0, 0, -1), 0.0, 0.0, intensity=3.0)
    edge["direction_outer"][0, 3] = 1.0  # cos_outer == cos_a: smoothstep gives 0
    edge["inner_angle"][0] = 1.5
    assert np.all(_shade_one(cam, gb, edge)[:3] == 0.0)


def test_kat_directional_light():
    cam, gb, P = _one_pixel()
    lt = directional_light((0.0, 0.0, -1.0), (0.5, 1.0, 0.25), 2.0)  # shines straight onto N = +z
    got = _shade_one(cam, gb, lt)
    # a directional light has no distance attenuation: the on-axis form at h = 1, r -> inf
    # carries atten = 1/(1 + 1e-4), which is undone here
    want = _closed_form_on_axis(1.0, 1e30, (0.5, 1.0, 0.25), 2.0, (0.8, 0.6, 0.4), 0.5, 0.0) * (1.0 + 1e-4)
    np.testing.assert_allclose(got[:3], want, rtol=1e-6)


def test_kat_ambient_hemisphere():
    cam, gb, P = _one_pixel(normal=(0.0, 1.0, 0.0))
    got = _shade_one(cam, gb, np.zeros(0, L.GPU_LIGHT), ambient=1.0)
    alb = gb.planes[0][0, 0, :3].astype(np.float64)
    sky = np.array([0.5, 0.5, 0.6], np.float32).astype(np.float64)
    np.testing.assert_allclose(got[:3], sky * alb, rtol=1e-7)  # N.y = 1: full sky term


def test_kat_sky_pixel_untouched():
    cam, gb, P = _one_pixel()
    gb.planes[2][:] = 1.0
    assert np.isnan(_shade_one(cam, gb, point_light((0, 0, -5), 10.0))).all()


# ----------------------------------------------------------------------------------
# tile culling (light_cull.wgsl:123-180)
# ----------------------------------------------------------------------------------


def test_tile_cap_and_order():
    cam = S.default_camera(64, 48)
    lists, counts = oracle.bin_tiles_ref(cam.record, overlapping_lights(70), 64, 48)
    assert (counts == 64).all() and (lists == np.arange(64)[None, :]).all()


def test_tile_zero_lights_cleared():
    cam = S.default_camera(40, 40)
    lists, counts = oracle.bin_tiles_ref(cam.record, np.zeros(0, L.GPU_LIGHT), 40, 40)
    assert (lists == 0).all() and (counts == 0).all()


def test_tile_directional_and_far_lights():
    cam = S.default_camera(96, 64)
    lt = np.concatenate([directional_light((0, -1, 0)), point_light((1000.0, 0.0, -10.0), 5.0)])
    lists, counts = oracle.bin_tiles_ref(cam.record, lt, 96, 64)
    assert (counts == 1).all() and (lists[:, 0] == 0).all()


def test_tile_lists_match_per_tile_brute_force_geometry():
    """A light far inside a tile's frustum is listed; one far outside every tile is not."""
    W, H = 160, 96
    cam = S.default_camera(W, H)
    lt = mixed_lights(cam, 2, 40, 10)
    lists, counts = oracle.bin_tiles_ref(cam.record, lt, W, H)
    lists64, counts64 = oracle.bin_tiles_ref(cam.record, lt, W, H, precision="f64")
    # f32 and f64 evaluations differ at most at boundary cases
    assert (counts != counts64).mean() < 0.05


# ----------------------------------------------------------------------------------
# froxel clustering
# ----------------------------------------------------------------------------------


@pytest.mark.parametrize("grid", [(4, 3, 8), (16, 9, 24), (7, 5, 3)])
def test_froxel_lists_are_conservative(grid):
    """Shading through the froxel lists equals shading every pixel over all lights (the
    exact semantics of the reference's light loop without a per-tile cap)."""
    W, H = 96, 64
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, S.LAYOUT_F32, seed=5)
    lt = mixed_lights(cam, 4, 120, 60, n_dir=2)
    glb = L.make_globals(L.tile_grid(W, H)[0], len(lt), ambient_color=(0.5, 0.5, 0.6), ambient_intensity=0.3)
    p = L.froxel_params(*grid, W, H, cam.far)
    off, idx = oracle.bin_froxels(cam.record, lt, p)
    got = oracle.shade(cam.record, glb, gb, lt, ("froxels", idx, off, p))
    allp = L.froxel_params(1, 1, 1, W, H, cam.far)
    everything = ("froxels", np.arange(len(lt), dtype=np.uint32), np.array([0, len(lt)], np.uint32), allp)
    want = oracle.shade(cam.record, glb, gb, lt, everything)
    np.testing.assert_array_equal(got, want)


def test_froxel_offsets_are_prefix_sums_and_sorted():
    cam = S.default_camera(128, 72)
    lt = mixed_lights(cam, 8, 200, 40)
    p = L.froxel_params(8, 4, 12, 128, 72, cam.far)
    off, idx = oracle.bin_froxels(cam.record, lt, p)
    assert off[0] == 0 and np.all(np.diff(off.astype(np.int64)) >= 0) and off[-1] == len(idx)
    for f in range(len(off) - 1):
        seg = idx[off[f]:off[f + 1]]
        assert np.all(np.diff(seg.astype(np.int64)) > 0)


def test_froxel_capacity_truncation_keeps_offsets():
    cam = S.default_camera(128, 72)
    lt = mixed_lights(cam, 8, 200, 40)
    p = L.froxel_params(8, 4, 12, 128, 72, cam.far)
    off, idx = oracle.bin_froxels(cam.record, lt, p)
    off2, idx2 = oracle.bin_froxels(cam.record, lt, p, capacity=len(idx) // 3)
    np.testing.assert_array_equal(off, off2)
    np.testing.assert_array_equal(idx[: len(idx) // 3], idx2)


def test_slice_table_convention():
    # prelude.wgsl:202-211: near 0.5, exponential up to max(far, 1)
    p = L.froxel_params(16, 9, 24, 1920, 1080, 100.0)
    t = oracle.froxel_slice_table(p).astype(np.float64)
    k = np.arange(1, 24)
    np.testing.assert_allclose(t[1:24], 0.5 * (100.0 / 0.5) ** (k / 24), rtol=1e-7)
    assert t[0] == 0.0 and t[24] == 100.0


# ----------------------------------------------------------------------------------
# FP64 adjoint against central finite differences
# ----------------------------------------------------------------------------------


def test_adjoint_matches_finite_differences():
    W, H = 24, 16
    cam = S.default_camera(W, H)
    gb = S.make_gbuffer(cam, S.LAYOUT_F32, seed=9)
    d = S.uniform(9, 90, W * H, 3.0, 9.0).reshape(H, W)
    gb.planes[2][:] = ((cam.far / (cam.far - cam.near)) * (1.0 - cam.near / d)).astype(np.float32)
    lt = S.make_lights(cam, 9, 12, 4, radius=(4.0, 9.0))
    lt["position_range"][:, 2] = np.clip(lt["position_range"][:, 2], -9.0, -3.0)
    glb = L.make_globals(L.tile_grid(W, H)[0], len(lt))
    allp = L.froxel_params(1, 1, 1, W, H, cam.far)
    grid = ("froxels", np.arange(len(lt), dtype=np.uint32), np.array([0, len(lt)], np.uint32), allp)
    rng = np.random.default_rng(3)
    w = rng.normal(size=(H, W, 4))
    dl, dp = oracle.shade_adjoint(cam.record, glb, gb, lt, grid, w)

    def loss(lights, gbuf):
        r = oracle.shade(cam.record, glb, gbuf, lights, grid)
        m = ~np.isnan(r[..., 0])
        return float((w[m][:, :3] * r[m][:, :3]).sum())

    # Finite differences need inputs perturbable in float64: rebuild the scene with the
    # oracle's double inputs by scaling with the f32 step exactly representable.
    checked = 0
    for li in range(len(lt)):
        for q, (field, comp) in enumerate([("position_range", 0), ("position_range", 1), ("position_range", 2),
                                           ("color_intensity", 3), ("color_intensity", 0),
                                           ("color_intensity", 1), ("color_intensity", 2)]):
            h = 1e-3 if q < 3 else 1e-3 * max(abs(float(lt[field][li, comp])), 1.0)
            lp, lm = lt.copy(), lt.copy()
            lp[field][li, comp] += np.float32(h)
            lm[field][li, comp] -= np.float32(h)
            hh = float(lp[field][li, comp]) - float(lm[field][li, comp])
            fd = (loss(lp, gb) - loss(lm, gb)) / hh
            if abs(dl[li, q]) > 1e-3 or abs(fd) > 1e-3:
                assert abs(fd - dl[li, q]) <= 2e-3 * max(abs(fd), abs(dl[li, q])) + 1e-6, (li, q, fd, dl[li, q])
                checked += 1
    assert checked >= 12
    # per-pixel albedo / roughness / metallic of a few lit pixels
    for (y, x) in [(4, 5), (8, 12), (10, 3)]:
        for c, (plane, comp) in enumerate([(0, 0), (0, 1), (0, 2), (0, 3), (1, 3)]):
            gp, gm = [p.copy() for p in gb.planes], [p.copy() for p in gb.planes]
            h = 1e-3
            gp[plane][y, x, comp] += np.float32(h)
            gm[plane][y, x, comp] -= np.float32(h)
            hh = float(gp[plane][y, x, comp]) - float(gm[plane][y, x, comp])
            fd = (loss(lt, S.GBuffer(1, W, H, gp)) - loss(lt, S.GBuffer(1, W, H, gm))) / hh
            assert abs(fd - dp[y, x, c]) <= 2e-3 * max(abs(fd), abs(dp[y, x, c])) + 1e-6, (y, x, c, fd, dp[y, x, c])


# ----------------------------------------------------------------------------------
# fragment lighting (Forward+ and transparent light loops)
# ----------------------------------------------------------------------------------


@pytest.mark.parametrize("rot,want", [((0, 0, 0), (0, 0, -1)), ((0, 90, 0), (-1, 0, 0)), ((90, 0, 0), (0, 1, 0)),
                                      ((0, 0, 90), (0, 0, -1)), ((0, 180, 0), (0, 0, 1)), ((-90, 0, 0), (0, -1, 0))])
def test_light_direction_from_rotation(rot, want):
    """Euler Y, X, Z (yaw, pitch, roll in degrees) applied to -Z (forward_lit.wgsl:374-383)."""
    np.testing.assert_allclose(oracle.light_dir_from_rotation(rot), want, atol=1e-12)


def _fragment_scene(seed=21, n=600, W=64, H=48):
    cam = S.make_camera((0.2, 0.1, 0.3), (0.0, 0.0, -8.0), (0, 1, 0), 60.0, W, H)
    lt = mixed_lights(cam, seed, n_point=20, n_spot=8, n_dir=1)
    fr = fragments(cam, seed, n)
    lists, counts = oracle.bin_tiles_ref(cam.record, lt, W, H)
    return cam, lt, fr, ("tiles", lists, counts)


def test_fragment_modes_agree_without_ambient_emission_or_cut():
    """With no ambient, no emission and every radiance above the 0.002 cut, the forward
    and transparent light loops are the same sum."""
    cam, lt, fr, grid = _fragment_scene()
    lt["color_intensity"][:, 3] = 1e4  # all radiances >> 0.002 inside the range
    fr["emissive"] = 0.0
    tx = L.tile_grid(cam.width, cam.height)[0]
    fwd = oracle.shade_fragments(cam.record, fragment_params(L.FRAGMENTS_FORWARD, tx, 0.0), fr, lt, grid)
    tra = oracle.shade_fragments(cam.record, fragment_params(L.FRAGMENTS_TRANSPARENT, tx, 0.0), fr, lt, grid)
    keep = fr["alpha"] > 0.001
    assert np.isnan(fwd[~keep]).all() and not np.isnan(tra).any()
    assert (fwd[keep][:, :3] > 0).any()
    np.testing.assert_allclose(fwd[keep], tra[keep], rtol=1e-12, atol=0)


def test_fragment_forward_ambient_and_emission():
    cam, lt, fr, grid = _fragment_scene()
    tx = L.tile_grid(cam.width, cam.height)[0]
    base = oracle.shade_fragments(cam.record, fragment_params(L.FRAGMENTS_FORWARD, tx, 0.0), fr, lt, grid)
    amb = oracle.shade_fragments(cam.record, fragment_params(L.FRAGMENTS_FORWARD, tx, 0.8, (0.2, 0.4, 0.6)), fr, lt,
                                 grid)
    keep = fr["alpha"] > 0.001
    want = (0.8 * np.array([0.2, 0.4, 0.6], np.float32).astype(np.float64) * fr["albedo"][keep] *
            fr["ao"][keep][:, None])
    np.testing.assert_allclose(amb[keep][:, :3] - base[keep][:, :3], want, rtol=1e-6, atol=1e-12)
    np.testing.assert_allclose(amb[keep][:, 3], fr["alpha"][keep])


def test_fragment_forward_reads_light_transforms():
    """Forward mode with entity indices reads positions and directions from the
    transforms; with transforms equal to the records' own values nothing changes."""
    cam, lt, fr, grid = _fragment_scene()
    n = len(lt)
    rng = np.random.default_rng(5)
    rot = rng.uniform(-180, 180, (n, 3)).astype(np.float32)
    dirs = np.stack([oracle.light_dir_from_rotation(r) for r in rot]).astype(np.float32)
    lt["direction_outer"][:, :3] = dirs
    perm = rng.permutation(n).astype(np.uint32)  # light i -> entity perm[i]
    xf = np.zeros(n, L.TRANSFORM)
    xf["position"][perm] = lt["position_range"][:, :3]
    xf["rotation"][perm] = rot
    tx = L.tile_grid(cam.width, cam.height)[0]
    prm = fragment_params(L.FRAGMENTS_FORWARD, tx)
    own = oracle.shade_fragments(cam.record, prm, fr, lt, grid)
    via = oracle.shade_fragments(cam.record, prm, fr, lt, grid, entity_indices=perm, transforms=xf)
    np.testing.assert_array_equal(np.isnan(own), np.isnan(via))
    k = ~np.isnan(own[:, 0])
    np.testing.assert_allclose(via[k], own[k], rtol=1e-12, atol=1e-300)
    # an entity index out of range drops that light (here the directional light)
    bad = perm.copy()
    bad[int(np.flatnonzero(lt["light_type"] == L.LIGHT_DIRECTIONAL)[0])] = n + 7
    dropped = oracle.shade_fragments(cam.record, prm, fr, lt, grid, entity_indices=bad, transforms=xf)
    assert not np.allclose(dropped[k], own[k])
