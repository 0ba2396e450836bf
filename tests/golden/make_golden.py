"""Generates tests/golden/shade_golden.npz: fs_main radiance of small scenes evaluated
at 50 significant digits by an independent Python restatement of the reference's WGSL
(deferred_lighting.wgsl:699-820 pbr_direct_light, :991-1259 fs_main under fallback
bindings; pbr_eval.wgsl:6-66), using mpmath. The C++ oracle's float64 evaluation is
checked against these vectors (tests/test_oracle.py).

Run: python tests/golden/make_golden.py   (writes the .npz next to this file)

Inputs are float32 exactly as the GPU receives them (camera matrices, G-buffer, lights);
every operation after that is carried out in 50-digit arithmetic.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

import mpmath as mp  # noqa: E402

from helio_gb300 import layouts as L  # noqa: E402
from helio_gb300 import synthetic as S  # noqa: E402

mp.mp.dps = 50
PI = mp.mpf("3.14159265359")  # pbr_eval.wgsl:6


def vec(a):
    return [mp.mpf(float(x)) for x in a]


def dot(a, b):
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]


def sub(a, b):
    return [a[i] - b[i] for i in range(3)]


def add(a, b):
    return [a[i] + b[i] for i in range(3)]


def scale(a, s):
    return [x * s for x in a]


def normalize(v):
    n = mp.sqrt(dot(v, v))
    return [x / n for x in v]


def clamp(x, lo, hi):
    return min(max(x, lo), hi)


def smoothstep(e0, e1, x):
    t = clamp((x - e0) / (e1 - e0), mp.mpf(0), mp.mpf(1))
    return t * t * (3 - 2 * t)


def pbr_direct_light(l, P, N, V, F0, albedo, rough, metal):
    color = vec(l["color_intensity"][:3])
    inten = mp.mpf(float(l["color_intensity"][3]))
    if int(l["light_type"]) == 0:
        Ld = normalize([-x for x in vec(l["direction_outer"][:3])])
        radiance = scale(color, inten)
    else:
        to_light = sub(vec(l["position_range"][:3]), P)
        dist = mp.sqrt(dot(to_light, to_light))
        rng = mp.mpf(float(l["position_range"][3]))
        if dist > rng:
            return [mp.mpf(0)] * 3
        Ld = scale(to_light, 1 / dist)
        atten = 1 / (dist * dist + mp.mpf("0.0001"))
        nd = dist / rng
        atten *= max(mp.mpf(0), 1 - nd ** 4)
        if int(l["light_type"]) == 2:
            cos_a = dot([-x for x in Ld], vec(l["direction_outer"][:3]))
            atten *= smoothstep(mp.mpf(float(l["direction_outer"][3])), mp.mpf(float(l["inner_angle"])), cos_a)
        radiance = scale(scale(color, inten), atten)
    NdL = max(dot(N, Ld), mp.mpf(0))
    if NdL == 0:
        return [mp.mpf(0)] * 3
    cut = mp.mpf(float(np.float64(np.float32(0.002))))  # the WGSL literal as f32
    if all(r < cut for r in radiance):
        return [mp.mpf(0)] * 3
    H = normalize(add(V, Ld))
    x = clamp(1 - max(dot(H, V), mp.mpf(0)), mp.mpf(0), mp.mpf(1))
    p5 = x ** 5
    F = [F0[i] + (1 - F0[i]) * p5 for i in range(3)]
    kD = [(1 - F[i]) * (1 - metal) for i in range(3)]
    NdV = max(dot(N, V), mp.mpf(0))
    a = rough * rough
    a2 = a * a
    NdH = max(dot(N, H), mp.mpf(0))
    den = NdH * NdH * (a2 - 1) + 1
    D = a2 / (PI * den * den + mp.mpf("0.0001"))
    k = (rough + 1) ** 2 / 8
    G = NdV / (NdV * (1 - k) + k + mp.mpf("0.0001")) * NdL / (NdL * (1 - k) + k + mp.mpf("0.0001"))
    spec = [D * G * F[i] / (4 * NdV * NdL + mp.mpf("0.0001")) for i in range(3)]
    return [(kD[i] * albedo[i] / PI + spec[i]) * radiance[i] * NdL for i in range(3)]


def shade_pixel(cam, gl, gb, lights, x, y):
    """fs_main for an F32-layout G-buffer; all lights in index order (one tile list)."""
    W, H = gb.width, gb.height
    a = gb.planes[0][y, x]
    n = gb.planes[1][y, x]
    depth = float(gb.planes[2][y, x])
    if not depth < 1.0:
        return [mp.nan] * 4
    albedo = vec(a[:3])
    rough = mp.mpf(float(a[3]))
    metal = mp.mpf(float(n[3]))
    N = normalize(vec(n[:3]))
    m = [mp.mpf(float(v)) for v in cam["inv_view_proj"]]
    u = (mp.mpf(x) + mp.mpf("0.5")) / W
    v = (mp.mpf(y) + mp.mpf("0.5")) / H
    ndc = [u * 2 - 1, 1 - v * 2, mp.mpf(depth), mp.mpf(1)]
    h = [sum(m[4 * c + r] * ndc[c] for c in range(4)) for r in range(4)]
    P = [h[0] / h[3], h[1] / h[3], h[2] / h[3]]
    F0 = [clamp(mp.mpf("0.04") * (1 - metal) + albedo[i] * metal, mp.mpf(0), mp.mpf("0.999")) for i in range(3)]
    V = normalize(sub(vec(cam["position_near"][:3]), P))
    Lo = [mp.mpf(0)] * 3
    for l in lights:
        if int(l["light_type"]) != 0:
            d = sub(vec(l["position_range"][:3]), P)
            if mp.sqrt(dot(d, d)) > mp.mpf(float(l["position_range"][3])):
                continue
        c = pbr_direct_light(l, P, N, V, F0, albedo, rough, metal)
        Lo = add(Lo, c)
    sky = [mp.mpf(float(gl["ambient_color"][i])) * mp.mpf(float(gl["ambient_intensity"])) for i in range(3)]
    t = N[1] * mp.mpf("0.5") + mp.mpf("0.5")
    hemi = [(sky[i] * mp.mpf("0.15") * (1 - t) + sky[i] * t) * albedo[i] for i in range(3)]
    return [Lo[i] + hemi[i] for i in range(3)] + [mp.mpf(1)]


def scene(seed: int, W=12, H=10, n_point=24, n_spot=10, ambient=0.7):
    cam = S.make_camera((0.3, -0.2, 0.5), (0.1, 0.2, -8.0), (0, 1, 0), 55.0, W, H, near=0.1, far=30.0)
    gb = S.make_gbuffer(cam, S.LAYOUT_F32, seed=seed)
    # pull depths into the lights' neighbourhood so most pixels are lit
    d = S.uniform(seed, 90, W * H, 2.0, 12.0).reshape(H, W)
    z = (cam.far / (cam.far - cam.near)) * (1.0 - cam.near / d)
    gb.planes[2] = np.ascontiguousarray(z.astype(np.float32))
    pts = np.stack([S.uniform(seed, 91 + k, n_point + n_spot, lo, hi) for k, (lo, hi) in
                    enumerate([(-3, 3), (-2.5, 2.5), (-11, -3)])], 1)
    lt = L.make_lights(n_point + n_spot)
    lt["position_range"][:, :3] = pts
    lt["position_range"][:, 3] = S.uniform(seed, 95, n_point + n_spot, 2.0, 8.0)
    lt["color_intensity"][:, :3] = np.stack([S.uniform(seed, 96 + k, n_point + n_spot) for k in range(3)], 1)
    lt["color_intensity"][:, 3] = S.uniform(seed, 99, n_point + n_spot, 0.5, 5.0)
    sp = np.arange(n_point, n_point + n_spot)
    dirs = S._unit_vectors(seed, 100, n_spot)
    outer = np.radians(S.uniform(seed, 102, n_spot, 20.0, 60.0))
    lt["light_type"][sp] = L.LIGHT_SPOT
    lt["direction_outer"][sp, :3] = dirs
    lt["direction_outer"][sp, 3] = np.cos(outer)
    lt["inner_angle"][sp] = np.cos(0.7 * outer)
    d0 = L.make_lights(1)
    d0["light_type"] = L.LIGHT_DIRECTIONAL
    d0["direction_outer"] = (0.3, -0.8, -0.5, 0.0)
    d0["color_intensity"] = (0.9, 0.8, 0.7, 0.6)
    lt = np.concatenate([lt[: n_point // 2], d0, lt[n_point // 2:]])
    tx, _ = L.tile_grid(W, H)
    glb = L.make_globals(tx, len(lt), ambient_color=(0.5, 0.5, 0.6), ambient_intensity=ambient)
    return cam, gb, lt, glb


def main():
    out = {}
    for k, seed in enumerate((11, 12)):
        cam, gb, lt, glb = scene(seed)
        rad = np.zeros((gb.height, gb.width, 4), np.float64)
        for y in range(gb.height):
            for x in range(gb.width):
                rad[y, x] = [float(v) for v in shade_pixel(cam.record[0], glb[0], gb, lt, x, y)]
        out[f"s{k}_camera"] = cam.record
        out[f"s{k}_globals"] = glb
        out[f"s{k}_lights"] = lt
        for i, p in enumerate(gb.planes):
            out[f"s{k}_plane{i}"] = p
        out[f"s{k}_radiance"] = rad
    np.savez_compressed(HERE / "shade_golden.npz", **out)
    print("wrote", HERE / "shade_golden.npz")


if __name__ == "__main__":
    main()
