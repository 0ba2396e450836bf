"""Small hand-built scenes for edge cases of binning and shading (shared by the CPU
oracle tests and the GPU parity tests)."""
from __future__ import annotations

import math

import numpy as np

from helio_gb300 import layouts as L
from helio_gb300 import synthetic as S


def point_light(pos, rng, color=(1.0, 1.0, 1.0), intensity=1.0):
    lt = L.make_lights(1)
    lt["position_range"][0] = (*pos, rng)
    lt["color_intensity"][0] = (*color, intensity)
    return lt


def spot_light(pos, rng, direction, outer_deg, inner_deg, color=(1.0, 1.0, 1.0), intensity=1.0):
    lt = point_light(pos, rng, color, intensity)
    d = np.asarray(direction, np.float64)
    d = d / np.linalg.norm(d)
    lt["light_type"] = L.LIGHT_SPOT
    lt["direction_outer"][0] = (*d, math.cos(math.radians(outer_deg)))
    lt["inner_angle"][0] = math.cos(math.radians(inner_deg))
    return lt


def directional_light(direction, color=(1.0, 1.0, 1.0), intensity=1.0):
    lt = L.make_lights(1)
    lt["light_type"] = L.LIGHT_DIRECTIONAL
    lt["direction_outer"][0] = (*direction, 0.0)
    lt["color_intensity"][0] = (*color, intensity)
    return lt


def overlapping_lights(n, centre=(0.0, 0.0, -10.0), rng=50.0):
    """``n`` point lights all covering the whole view (to exercise the 64 cap)."""
    return np.concatenate([point_light(centre, rng, intensity=1.0 + 0.01 * i) for i in range(n)])


def mixed_lights(cam, seed, n_point=40, n_spot=20, n_dir=2):
    """Point, spot (with well-formed and degenerate cones) and directional lights,
    some behind the camera and some far outside the frustum."""
    base = S.make_lights(cam, seed, n_point, n_spot)
    extra = [
        directional_light((0.3, -1.0, 0.2)),
        point_light((0.0, 0.0, 5.0), 2.0),        # behind the camera
        point_light((0.0, 0.0, 5.0), 20.0),       # behind, reaching into the frustum
        point_light((500.0, 0.0, -50.0), 10.0),   # far outside
        spot_light((0.0, 2.0, -10.0), 15.0, (0, -1, 0), 30.0, 40.0),   # inner > outer
        spot_light((1.0, 0.0, -8.0), 12.0, (0, 0, -1), 95.0, 60.0),    # obtuse cone
        spot_light((-1.0, 0.5, -12.0), 12.0, (1, 0, 0), 20.0, 20.0),   # inner == outer
    ]
    for _ in range(max(0, n_dir - 1)):
        extra.append(directional_light((-0.5, -0.7, 0.1)))
    lt = np.concatenate([base] + extra)
    order = np.argsort(S.uniform(seed, 99, len(lt)), kind="stable")
    return lt[order]


def fragments(cam, seed, n, discard_frac=0.05):
    """``n`` fragments at random pixels of ``cam``'s viewport, view depth U[2, 14], each
    the world point under its pixel centre (f32), with random normals facing the camera
    and random materials; about ``discard_frac`` of them have alpha <= 0.001."""
    W, H = cam.width, cam.height
    u = lambda k, lo=0.0, hi=1.0: S.uniform(seed, 300 + k, n, lo, hi)
    x = np.minimum((u(0) * W).astype(np.int64), W - 1)
    y = np.minimum((u(1) * H).astype(np.int64), H - 1)
    d = u(2, 2.0, 14.0)
    z = (cam.far / (cam.far - cam.near)) * (1.0 - cam.near / d)
    ndc = np.stack([(x + 0.5) / W * 2 - 1, 1 - (y + 0.5) / H * 2, z, np.ones(n)])
    h = cam.inv_view_proj @ ndc
    P = (h[:3] / h[3]).T
    V = np.asarray(cam.eye, np.float64)[None, :] - P
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    Nr = np.stack([u(3, -1, 1), u(4, -1, 1), u(5, -1, 1)], 1) + 1.2 * V
    Nr /= np.linalg.norm(Nr, axis=1, keepdims=True)
    fr = np.zeros(n, L.FRAGMENT)
    fr["position"] = P.astype(np.float32)
    fr["pixel"] = (x | (y << 16)).astype(np.uint32)
    fr["normal"] = Nr.astype(np.float32)
    fr["alpha"] = np.where(u(6) < discard_frac, 0.0005, u(7, 0.2, 1.0)).astype(np.float32)
    albedo = np.stack([u(8), u(9), u(10)], 1)
    metal = (u(11) < 0.3).astype(np.float64)
    fr["albedo"] = albedo.astype(np.float32)
    fr["roughness"] = u(12, 0.05, 1.0).astype(np.float32)
    fr["metallic"] = metal.astype(np.float32)
    fr["f0"] = np.clip(0.04 * (1 - metal[:, None]) + albedo * metal[:, None], 0, 0.999).astype(np.float32)
    fr["emissive"] = np.stack([u(13, 0, 0.2), u(14, 0, 0.2), u(15, 0, 0.2)], 1).astype(np.float32)
    fr["ao"] = u(16, 0.5, 1.0).astype(np.float32)
    return fr


def fragment_params(mode, num_tiles_x, ambient_intensity=0.4, ambient_color=(0.5, 0.55, 0.6)):
    p = np.zeros(1, L.FRAGMENT_PARAMS)
    p["mode"], p["num_tiles_x"] = mode, num_tiles_x
    p["ambient_intensity"], p["ambient_color"] = ambient_intensity, ambient_color
    return p
