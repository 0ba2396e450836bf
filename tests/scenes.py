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
    """``n`` fragments at random pixels of ``cam``'s viewport (synthetic.make_fragments)."""
    return S.make_fragments(cam, seed, n, discard_frac)


def fragment_params(mode, num_tiles_x, ambient_intensity=0.4, ambient_color=(0.5, 0.55, 0.6)):
    return S.fragment_params(mode, num_tiles_x, ambient_intensity, ambient_color)
