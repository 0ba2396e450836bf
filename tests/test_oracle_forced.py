"""The forced-branch form of the FP64 oracle (oracle.shade_forced), CPU only.

The GPU parity tests compare a kernel's radiance with the FP64 oracle evaluated with
the kernel's own branch decisions at the cuts of pbr_direct_light (range, NdL == 0,
radiance < 0.002; deferred_lighting.wgsl:725,779,781), as recorded by hl_set_pair_log.
Here the forced form is pinned against the plain oracle: given the oracle's own
decisions (restated below in numpy) it reproduces the plain radiance bit for bit with
no flips; a decision taken away or added moves exactly that pixel by exactly that
pair's term, and is counted; a lit pair whose light is not in the pixel's list is
reported."""
import numpy as np
import pytest

import oracle
from helio_gb300 import layouts as L
from helio_gb300 import synthetic as S



def _scene(w=96, h=54, layout=S.LAYOUT_F32):
    cam = S.default_camera(w, h)
    gb = S.make_gbuffer(cam, layout, seed=31)
    lights = S.make_lights(cam, 32, 450, 150)
    p = L.froxel_params(8, 6, 16, w, h, cam.far)
    off, idx = oracle.bin_froxels(cam.record, lights, p, capacity=1 << 22)
    glb = L.make_globals(L.tile_grid(w, h)[0], len(lights), ambient_color=(0.3, 0.35, 0.4), ambient_intensity=0.25)
    return cam, gb, lights, glb, ("froxels", idx, off, p)


def _own_lit_pairs(cam, gb, lights, grid):
    """The FP64 oracle's own lit (pixel, light) pairs of an F32 G-buffer, restated in
    numpy from pbr_direct_light's cuts (deferred_lighting.wgsl:719-733, 778-781)."""
    _, idx, off, p = grid
    W, H = gb.width, gb.height
    rec = cam.record[0]
    m = rec["inv_view_proj"].astype(np.float64).reshape(4, 4).T
    near, far = float(rec["position_near"][3]), float(rec["forward_far"][3])
    tab = oracle.froxel_slice_table(p).astype(np.float64)
    gx, gy, gz = int(p["grid_x"][0]), int(p["grid_y"][0]), int(p["grid_z"][0])
    depth = gb.planes[2].astype(np.float64)
    nrm = gb.planes[1][..., :3].astype(np.float64)
    pairs = []
    for y in range(H):
        for x in range(W):
            d = depth[y, x]
            if not d < 1.0:
                continue
            ndc = np.array([(x + 0.5) / W * 2 - 1, 1 - (y + 0.5) / H * 2, d, 1.0])
            hh = m @ ndc
            P = hh[:3] / hh[3]
            N = nrm[y, x] / np.linalg.norm(nrm[y, x])
            dv = near * far / (far - d * (far - near))
            s = max([k for k in range(gz) if tab[k] <= dv] + [0])
            f = ((y * gy // H) * gx + x * gx // W) * gz + s
            for li in idx[off[f]:off[f + 1]]:
                l = lights[li]
                col = l["color_intensity"][:3].astype(np.float64) * float(l["color_intensity"][3])
                if l["light_type"] == L.LIGHT_DIRECTIONAL:
                    dr = -l["direction_outer"][:3].astype(np.float64)
                    Ld = dr / np.linalg.norm(dr)
                    rad = col
                else:
                    t = l["position_range"][:3].astype(np.float64) - P
                    dist = np.linalg.norm(t)
                    r = float(l["position_range"][3])
                    if dist > r:
                        continue
                    Ld = t / dist
                    att = 1.0 / (dist * dist + 1e-4) * max(0.0, 1.0 - (dist / r) ** 4)
                    if l["light_type"] == L.LIGHT_SPOT:
                        lo, hi = float(l["direction_outer"][3]), float(l["inner_angle"])
                        c = float(-Ld @ l["direction_outer"][:3].astype(np.float64))
                        tt = min(max((c - lo) / (hi - lo), 0.0), 1.0)
                        att *= tt * tt * (3 - 2 * tt)
                    rad = col * att
                if max(N @ Ld, 0.0) == 0.0 or np.all(rad < 0.002):
                    continue
                pairs.append((y * W + x, int(li)))
    return np.array(pairs, np.uint32).reshape(-1, 2)


@pytest.fixture(scope="module")
def scene():
    cam, gb, lights, glb, grid = _scene()
    return cam, gb, lights, glb, grid, _own_lit_pairs(cam, gb, lights, grid)


def test_own_decisions_reproduce_the_plain_oracle(scene):
    cam, gb, lights, glb, grid, pairs = scene
    assert len(pairs) > 800
    plain, pc = oracle.shade(cam.record, glb, gb, lights, grid, pair_counts=True)
    assert int(pc[..., 2].sum()) == len(pairs)
    forced, flips, unlisted = oracle.shade_forced(cam.record, glb, gb, lights, grid, pairs[::-1])  # any order
    assert flips.sum() == 0 and unlisted.sum() == 0
    sky = np.isnan(plain[..., 0])
    assert np.array_equal(np.isnan(forced[..., 0]), sky)
    assert np.array_equal(forced[~sky], plain[~sky])


def test_a_changed_decision_moves_only_its_pixel_by_its_term(scene):
    cam, gb, lights, glb, grid, pairs = scene
    plain = oracle.shade(cam.record, glb, gb, lights, grid)
    drop = len(pairs) // 3
    pix, li = int(pairs[drop, 0]), int(pairs[drop, 1])
    forced, flips, unlisted = oracle.shade_forced(cam.record, glb, gb, lights, grid, np.delete(pairs, drop, 0))
    W = gb.width
    assert flips.reshape(-1)[pix] == 1 and flips.sum() == 1 and unlisted.sum() == 0
    diff = np.abs(forced - plain)[..., :3].reshape(-1, 3)
    diff[np.isnan(diff)] = 0
    assert np.count_nonzero(diff.max(-1)) == 1 and diff[pix].max() > 0
    # the dropped term, alone: the pixel's radiance with that one light lit
    only = oracle.shade_forced(cam.record, glb, gb, lights, grid, np.array([[pix, li]], np.uint32))[0]
    amb = oracle.shade_forced(cam.record, glb, gb, lights, grid, np.zeros((0, 2), np.uint32))[0]
    y, x = divmod(pix, W)
    term = only[y, x, :3] - amb[y, x, :3]
    np.testing.assert_allclose(plain[y, x, :3] - forced[y, x, :3], term, rtol=1e-12, atol=1e-15)


def test_forced_pair_across_a_cut_is_evaluated_without_it(scene):
    cam, gb, lights, glb, grid, pairs = scene
    _, idx, off, p = grid
    have = set(map(tuple, pairs.tolist()))
    # a listed pair the oracle cuts (out of range, below the horizon or under 0.002)
    forced_pairs = None
    plain = oracle.shade(cam.record, glb, gb, lights, grid)
    for pix, li in pairs[:50]:
        for other in idx[:200]:
            if (int(pix), int(other)) not in have:
                cand = np.vstack([pairs, [[pix, other]]]).astype(np.uint32)
                forced, flips, unlisted = oracle.shade_forced(cam.record, glb, gb, lights, grid, cand)
                if unlisted.sum() == 0:
                    forced_pairs = (int(pix), int(other), forced, flips)
                    break
        if forced_pairs:
            break
    assert forced_pairs is not None
    pix, other, forced, flips = forced_pairs
    assert flips.reshape(-1)[pix] == 1 and flips.sum() == 1
    y, x = divmod(pix, gb.width)
    # beyond the range or below the horizon the forced term is 0; under the radiance cut
    # it is the (small, non-negative) full BRDF value
    assert np.all(forced[y, x, :3] >= plain[y, x, :3])


def test_lit_pair_outside_the_list_is_reported(scene):
    cam, gb, lights, glb, grid, pairs = scene
    _, idx, off, p = grid
    pix = int(pairs[0, 0])
    y, x = divmod(pix, gb.width)
    # the pixel's own froxel list: any other light is not in it
    near, far = cam.near, cam.far
    d = float(gb.planes[2][y, x])
    dv = near * far / (far - d * (far - near))
    tab = oracle.froxel_slice_table(p)
    gx, gy, gz = int(p["grid_x"][0]), int(p["grid_y"][0]), int(p["grid_z"][0])
    s = max([k for k in range(gz) if tab[k] <= dv] + [0])
    f = ((y * gy // gb.height) * gx + x * gx // gb.width) * gz + s
    outside = sorted(set(range(len(lights))) - set(idx[off[f]:off[f + 1]].tolist()))
    cand = np.vstack([pairs, [[pix, outside[0]]]]).astype(np.uint32)
    _, flips, unlisted = oracle.shade_forced(cam.record, glb, gb, lights, grid, cand)
    assert unlisted.reshape(-1)[pix] == 1 and unlisted.sum() == 1 and flips.sum() == 0


def test_forced_csr_sorts_and_deduplicates():
    off, lts = oracle.forced_csr(np.array([[3, 9], [1, 4], [3, 2], [3, 9], [0, 7]], np.uint32), 5)
    assert off.tolist() == [0, 1, 2, 2, 4, 4]
    assert lts.tolist() == [7, 4, 2, 9]
    with pytest.raises(ValueError):
        oracle.forced_csr(np.array([[5, 0]], np.uint32), 5)
