"""Seeded synthetic scenes for the deferred-lighting path.

The reference benchmarks no public dataset for this path; its inputs are a G-buffer,
a camera and a light buffer. These generators build those inputs with the shapes and
value distributions of the five workloads this project measures:

  w0  1280x720  F32 G-buffer,   64 point lights,                      froxels 16x9x24
  w1  1920x1080 F16 G-buffer, 1024 lights (768 point / 256 spot),     froxels 16x9x24
  w2  3840x2160 F32 G-buffer, 4096 point lights in 8 Gaussian clumps, froxels 32x18x48
  w3  98 views (96 cube faces 128^2/256^2/512^2 + 1080p + 720p), F16, 2048 lights
  w4  1920x1080 F32 G-buffer,  256 point lights, adjoint against perturbed lights

Camera: glam's right-handed look-at and DirectX-convention perspective (NDC z in
[0,1], near -> 0), as Helio builds it (helio/src/scene/camera.rs:124-125); all
matrices are formed in float64 and stored as float32, column major.

G-buffer: linear view depth d ~ U[0.5, 100] stored as NDC depth; normal uniform on
the hemisphere facing the camera; albedo ~ U[0,1]^3; roughness ~ U[0.05, 1];
metallic in {0, 1} with P(1) = 0.3.

Random numbers come from a counter-based SplitMix64 hash of (seed, stream, index), so
every array is reproducible element by element on any machine.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import layouts as L

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix64(x: np.ndarray) -> np.ndarray:
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def uniform(seed: int, stream: int, n: int, lo: float = 0.0, hi: float = 1.0) -> np.ndarray:
    """``n`` float64 values in [lo, hi) from the hash of (seed, stream, index)."""
    with np.errstate(over="ignore"):
        base = _splitmix64(np.array([(seed * 0x100000001B3 + stream * 0x9E3779B1) & 0xFFFFFFFFFFFFFFFF], np.uint64))[0]
        idx = np.arange(n, dtype=np.uint64)
        h = _splitmix64(idx ^ base)
    u = (h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


# ----------------------------------------------------------------------------------
# Camera
# ----------------------------------------------------------------------------------


def look_at_rh(eye, target, up) -> np.ndarray:
    """glam ``look_at_rh`` as a 4x4 float64 matrix (row = math row)."""
    eye, target, up = (np.asarray(v, np.float64) for v in (eye, target, up))
    f = target - eye
    f = f / np.linalg.norm(f)
    s = np.cross(f, up)
    s = s / np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def perspective_rh_dx(fov_y: float, aspect: float, near: float, far: float) -> np.ndarray:
    """glam ``perspective_rh`` (DirectX depth range) as a 4x4 float64 matrix."""
    h = math.cos(0.5 * fov_y) / math.sin(0.5 * fov_y)
    w = h / aspect
    r = far / (near - far)
    m = np.zeros((4, 4))
    m[0, 0], m[1, 1], m[2, 2], m[2, 3], m[3, 2] = w, h, r, r * near, -1.0
    return m


@dataclass
class Camera:
    eye: np.ndarray
    view: np.ndarray  # float64 4x4
    proj: np.ndarray
    near: float
    far: float
    width: int
    height: int
    fov_y: float
    record: np.ndarray = field(repr=False)  # GPU_CAMERA, shape (1,)

    @property
    def inv_view_proj(self) -> np.ndarray:
        return np.linalg.inv(self.proj @ self.view)

    def bytes(self) -> bytes:
        return self.record.tobytes()


def _cols(m: np.ndarray) -> np.ndarray:
    return m.T.reshape(16).astype(np.float32)


def make_camera(eye, target, up, fov_y_deg, width, height, near=0.1, far=100.0) -> Camera:
    view = look_at_rh(eye, target, up)
    proj = perspective_rh_dx(math.radians(fov_y_deg), width / height, near, far)
    vp = proj @ view
    rec = np.zeros(1, L.GPU_CAMERA)
    rec["view"] = _cols(view)
    rec["proj"] = _cols(proj)
    rec["view_proj"] = _cols(vp)
    rec["inv_view_proj"] = _cols(np.linalg.inv(vp))
    eye = np.asarray(eye, np.float64)
    fwd = np.asarray(target, np.float64) - eye
    fwd = fwd / np.linalg.norm(fwd)
    rec["position_near"] = (*eye, near)
    rec["forward_far"] = (*fwd, far)
    rec["jitter_frame"] = (0.0, 0.0, 0.0, 0.0)
    rec["prev_view_proj"] = _cols(vp)
    return Camera(eye, view, proj, near, far, width, height, math.radians(fov_y_deg), rec)


def default_camera(width: int, height: int, fov_y_deg: float = 60.0) -> Camera:
    """Eye at the origin looking down -Z, up +Y, near 0.1, far 100."""
    return make_camera((0, 0, 0), (0, 0, -1), (0, 1, 0), fov_y_deg, width, height)


CUBE_FACES = (  # (forward, up) per face, +X -X +Y -Y +Z -Z
    ((1, 0, 0), (0, -1, 0)),
    ((-1, 0, 0), (0, -1, 0)),
    ((0, 1, 0), (0, 0, 1)),
    ((0, -1, 0), (0, 0, -1)),
    ((0, 0, 1), (0, -1, 0)),
    ((0, 0, -1), (0, -1, 0)),
)


def cube_face_camera(center, face: int, size: int) -> Camera:
    f, up = CUBE_FACES[face]
    c = np.asarray(center, np.float64)
    return make_camera(c, c + np.asarray(f, np.float64), up, 90.0, size, size)


# ----------------------------------------------------------------------------------
# Half floats, octahedral normals
# ----------------------------------------------------------------------------------


def oct_encode(n: np.ndarray) -> np.ndarray:
    """Octahedral encoding of unit vectors (Cigolle et al. 2014), z up; (..., 2)."""
    a = np.abs(n).sum(-1, keepdims=True)
    p = n[..., :2] / a
    neg = n[..., 2] < 0
    sgn = np.where(p >= 0, 1.0, -1.0)
    q = (1.0 - np.abs(p[..., ::-1])) * sgn
    return np.where(neg[..., None], q, p)


def oct_decode(e: np.ndarray) -> np.ndarray:
    x, y = e[..., 0].astype(np.float64), e[..., 1].astype(np.float64)
    z = 1.0 - np.abs(x) - np.abs(y)
    neg = z < 0
    ox = (1.0 - np.abs(y)) * np.where(x >= 0, 1.0, -1.0)
    oy = (1.0 - np.abs(x)) * np.where(y >= 0, 1.0, -1.0)
    x = np.where(neg, ox, x)
    y = np.where(neg, oy, y)
    n = np.stack([x, y, z], -1)
    return n / np.linalg.norm(n, axis=-1, keepdims=True)


# ----------------------------------------------------------------------------------
# G-buffers
# ----------------------------------------------------------------------------------


@dataclass
class GBuffer:
    layout: int  # 0 reference, 1 F32, 2 F16
    width: int
    height: int
    planes: list  # numpy arrays, each (H, W, C) or (H, W)
    # float64 ground truth of the generated surface (before storage rounding)
    truth: dict = field(default_factory=dict, repr=False)

    @property
    def bytes_per_pixel(self) -> int:
        return sum(p.dtype.itemsize * (p.shape[2] if p.ndim == 3 else 1) for p in self.planes)


LAYOUT_REFERENCE, LAYOUT_F32, LAYOUT_F16 = 0, 1, 2


def _surface(cam: Camera, seed: int):
    W, H = cam.width, cam.height
    n = W * H
    d = uniform(seed, 1, n, 0.5, 100.0)
    near, far = cam.near, cam.far
    z = (far / (far - near)) * (1.0 - near / d)
    depth = z.astype(np.float32)
    # view direction of each pixel centre (float64) to orient the hemisphere
    xs = (np.arange(W) + 0.5) / W * 2.0 - 1.0
    ys = 1.0 - (np.arange(H) + 0.5) / H * 2.0
    X, Y = np.meshgrid(xs, ys)
    inv = cam.inv_view_proj
    h = np.stack([X.ravel(), Y.ravel(), depth.astype(np.float64), np.ones(n)], 0)
    wp = inv @ h
    P = (wp[:3] / wp[3]).T
    V = cam.eye[None, :] - P
    V /= np.linalg.norm(V, axis=1, keepdims=True)
    u1 = uniform(seed, 2, n)
    u2 = uniform(seed, 3, n)
    zc = 1.0 - 2.0 * u1
    r = np.sqrt(np.maximum(0.0, 1.0 - zc * zc))
    phi = 2.0 * math.pi * u2
    N = np.stack([r * np.cos(phi), r * np.sin(phi), zc], 1)
    flip = (N * V).sum(1) < 0
    N[flip] *= -1.0
    albedo = np.stack([uniform(seed, 4, n), uniform(seed, 5, n), uniform(seed, 6, n)], 1)
    rough = uniform(seed, 7, n, 0.05, 1.0)
    metal = (uniform(seed, 8, n) < 0.3).astype(np.float64)
    return depth.reshape(H, W), N.reshape(H, W, 3), albedo.reshape(H, W, 3), rough.reshape(H, W), metal.reshape(H, W)


def make_gbuffer(cam: Camera, layout: int, seed: int) -> GBuffer:
    depth, N, albedo, rough, metal = _surface(cam, seed)
    W, H = cam.width, cam.height
    truth = dict(depth=depth, normal=N, albedo=albedo, roughness=rough, metallic=metal)
    if layout == LAYOUT_F32:
        p0 = np.concatenate([albedo, rough[..., None]], -1).astype(np.float32)
        p1 = np.concatenate([N, metal[..., None]], -1).astype(np.float32)
        planes = [np.ascontiguousarray(p0), np.ascontiguousarray(p1), np.ascontiguousarray(depth)]
    elif layout == LAYOUT_F16:
        p0 = np.concatenate([albedo, rough[..., None]], -1).astype(np.float16)
        p1 = oct_encode(N).astype(np.float16)
        p2 = metal.astype(np.float16)
        planes = [np.ascontiguousarray(p0), np.ascontiguousarray(p1), np.ascontiguousarray(p2), np.ascontiguousarray(depth)]
    elif layout == LAYOUT_REFERENCE:
        f0 = np.clip(0.04 * (1.0 - metal[..., None]) + albedo * metal[..., None], 0.0, 0.999)
        u8 = lambda v: np.clip(np.rint(v * 255.0), 0, 255).astype(np.uint8)
        a = np.concatenate([u8(albedo), np.full((H, W, 1), 255, np.uint8)], -1)
        nrm = np.concatenate([N, f0[..., :1]], -1).astype(np.float16)
        orm = np.stack([np.full((H, W), 255, np.uint8), u8(rough), u8(metal), u8(f0[..., 1])], -1)
        emi = np.concatenate([np.zeros((H, W, 3)), f0[..., 2:3]], -1).astype(np.float16)
        planes = [a, nrm, orm, emi, np.ascontiguousarray(depth)]
    else:
        raise ValueError(f"unknown layout {layout}")
    return GBuffer(layout, W, H, planes, truth)


# ----------------------------------------------------------------------------------
# Lights
# ----------------------------------------------------------------------------------


def _frustum_points(cam: Camera, seed: int, stream: int, n: int) -> np.ndarray:
    """``n`` world points uniform in the camera frustum volume (rejection sampling in
    the view-space bounding box)."""
    ty = math.tan(0.5 * cam.fov_y)
    tx = ty * cam.width / cam.height
    far, near = cam.far, cam.near
    out = []
    got, batch, k = 0, max(4 * n, 64), 0
    while got < n:
        u = uniform(seed, stream * 1000 + 3 * k, batch, -1.0, 1.0)
        v = uniform(seed, stream * 1000 + 3 * k + 1, batch, -1.0, 1.0)
        w = uniform(seed, stream * 1000 + 3 * k + 2, batch, near, far)
        x, y, zd = u * far * tx, v * far * ty, w
        ok = (np.abs(x) <= zd * tx) & (np.abs(y) <= zd * ty)
        pts = np.stack([x[ok], y[ok], -zd[ok], np.ones(ok.sum())], 1)
        out.append(pts)
        got += len(pts)
        k += 1
    vs = np.concatenate(out)[:n]
    inv_view = np.linalg.inv(cam.view)
    return (inv_view @ vs.T).T[:, :3]


def _unit_vectors(seed: int, stream: int, n: int) -> np.ndarray:
    zc = uniform(seed, stream, n, -1.0, 1.0)
    phi = uniform(seed, stream + 1, n, 0.0, 2.0 * math.pi)
    r = np.sqrt(np.maximum(0.0, 1.0 - zc * zc))
    return np.stack([r * np.cos(phi), r * np.sin(phi), zc], 1)


def make_lights(
    cam: Camera,
    seed: int,
    n_point: int,
    n_spot: int = 0,
    radius=(1.0, 10.0),
    intensity=(0.5, 5.0),
    clumps: int = 0,
    clump_sigma: float = 5.0,
) -> np.ndarray:
    """A ``GpuLight`` array: point and spot lights (spots spread through the index
    order by a seeded permutation), shadows off, no IES, no light function."""
    n = n_point + n_spot
    lt = L.make_lights(n)
    if clumps:
        centres = _frustum_points(cam, seed, 10, clumps)
        which = np.minimum((uniform(seed, 11, n) * clumps).astype(np.int64), clumps - 1)
        g = np.stack([uniform(seed, 12 + a, n) for a in range(6)], 1)
        # Box-Muller: three normals from six uniforms
        u1 = np.maximum(g[:, 0:3], 1e-300)
        u2 = g[:, 3:6]
        gauss = np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)
        pos = centres[which] + clump_sigma * gauss
    else:
        pos = _frustum_points(cam, seed, 20, n)
    rng = uniform(seed, 30, n, *radius)
    inten = uniform(seed, 31, n, *intensity)
    col = np.stack([uniform(seed, 32, n), uniform(seed, 33, n), uniform(seed, 34, n)], 1)
    types = np.full(n, L.LIGHT_POINT, np.uint32)
    if n_spot:
        order = np.argsort(uniform(seed, 35, n), kind="stable")
        types[order[:n_spot]] = L.LIGHT_SPOT
    dirs = _unit_vectors(seed, 36, n)
    outer = np.radians(uniform(seed, 38, n, 10.0, 45.0))
    inner = 0.75 * outer
    lt["position_range"][:, :3] = pos
    lt["position_range"][:, 3] = rng
    lt["color_intensity"][:, :3] = col
    lt["color_intensity"][:, 3] = inten
    lt["light_type"] = types
    spot = types == L.LIGHT_SPOT
    lt["direction_outer"][spot, :3] = dirs[spot]
    lt["direction_outer"][spot, 3] = np.cos(outer[spot])
    lt["inner_angle"][spot] = np.cos(inner[spot])
    return lt


# ----------------------------------------------------------------------------------
# Workloads
# ----------------------------------------------------------------------------------


@dataclass
class Workload:
    name: str
    camera: Camera
    gbuffer: GBuffer
    lights: np.ndarray
    globals_: np.ndarray
    froxel_grid: tuple


def workload(index: int, scale: float = 1.0) -> Workload:
    """The single-view workloads w0, w1, w2, w4 (w3 is ``batched_views``). ``scale``
    shrinks the resolution for quick tests while keeping every distribution."""
    specs = {
        0: dict(W=1280, H=720, layout=LAYOUT_F32, n_point=64, n_spot=0, grid=(16, 9, 24), radius=(1.0, 10.0), clumps=0),
        1: dict(W=1920, H=1080, layout=LAYOUT_F16, n_point=768, n_spot=256, grid=(16, 9, 24), radius=(1.0, 10.0), clumps=0),
        2: dict(W=3840, H=2160, layout=LAYOUT_F32, n_point=4096, n_spot=0, grid=(32, 18, 48), radius=(0.5, 20.0), clumps=8),
        4: dict(W=1920, H=1080, layout=LAYOUT_F32, n_point=256, n_spot=0, grid=(16, 9, 24), radius=(1.0, 10.0), clumps=0),
    }
    s = specs[index]
    W, H = max(16, int(round(s["W"] * scale))), max(16, int(round(s["H"] * scale)))
    cam = default_camera(W, H)
    gb = make_gbuffer(cam, s["layout"], seed=index * 1000)
    lights = make_lights(cam, index * 1000 + 500, s["n_point"], s["n_spot"], radius=s["radius"], clumps=s["clumps"])
    tx, _ = L.tile_grid(W, H)
    glb = L.make_globals(tx, len(lights))
    return Workload(f"w{index}", cam, gb, lights, glb, s["grid"])


def perturbed_lights(lights: np.ndarray, seed: int, sigma: float = 0.5, lo: float = 0.8, hi: float = 1.2) -> np.ndarray:
    """Target lights of the adjoint workload: position + N(0, sigma^2) per axis and
    intensity x U[lo, hi]."""
    n = len(lights)
    out = lights.copy()
    g = np.stack([uniform(seed, 60 + a, n) for a in range(6)], 1)
    gauss = np.sqrt(-2.0 * np.log(np.maximum(g[:, :3], 1e-300))) * np.cos(2.0 * math.pi * g[:, 3:])
    out["position_range"][:, :3] += (sigma * gauss).astype(np.float32)
    out["color_intensity"][:, 3] *= uniform(seed, 70, n, lo, hi).astype(np.float32)
    return out


@dataclass
class View:
    camera: Camera
    gbuffer: GBuffer


def batched_views(scale: float = 1.0, layout: int = LAYOUT_F16):
    """Workload w3: 16 probes x 6 cube faces (probes 0-5 at 128^2, 6-10 at 256^2,
    11-15 at 512^2) plus a 1920x1080 and a 1280x720 viewport, sharing 2048 lights
    (3 point : 1 spot) placed in the 1080p viewport's frustum. Probe centres are
    uniform in that frustum as well."""
    main = default_camera(max(16, int(1920 * scale)), max(16, int(1080 * scale)))
    lights = make_lights(main, 3500, 1536, 512)
    centres = _frustum_points(main, 3000, 40, 16)
    views = []
    vi = 0
    for p in range(16):
        size = 128 if p < 6 else (256 if p < 11 else 512)
        size = max(16, int(size * scale))
        for f in range(6):
            cam = cube_face_camera(centres[p], f, size)
            views.append(View(cam, make_gbuffer(cam, layout, seed=3000 + vi)))
            vi += 1
    for (w, h) in ((1920, 1080), (1280, 720)):
        cam = default_camera(max(16, int(w * scale)), max(16, int(h * scale)))
        views.append(View(cam, make_gbuffer(cam, layout, seed=3000 + vi)))
        vi += 1
    return views, lights


def make_fragments(cam: Camera, seed: int, n: int, discard_frac: float = 0.05, raster_order: bool = False) -> np.ndarray:
    """``n`` hl_fragment records (layouts.FRAGMENT) at random pixels of ``cam``'s viewport,
    view depth U[2, 14], each the world point under its pixel centre (f32), with random
    normals facing the camera and random materials; about ``discard_frac`` of them have
    alpha <= 0.001. ``raster_order`` sorts them by pixel, as a rasteriser emits them."""
    W, H = cam.width, cam.height
    u = lambda k, lo=0.0, hi=1.0: uniform(seed, 300 + k, n, lo, hi)
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
    if raster_order:
        fr = fr[np.argsort(y * W + x, kind="stable")]
    return fr


def fragment_params(mode: int, num_tiles_x: int, ambient_intensity: float = 0.4,
                    ambient_color=(0.5, 0.55, 0.6)) -> np.ndarray:
    """One layouts.FRAGMENT_PARAMS record."""
    p = np.zeros(1, L.FRAGMENT_PARAMS)
    p["mode"], p["num_tiles_x"] = mode, num_tiles_x
    p["ambient_intensity"], p["ambient_color"] = ambient_intensity, ambient_color
    return p


# ----------------------------------------------------------------------------------
# Material scenes: the inputs of the G-buffer pass's fragment stage
# ----------------------------------------------------------------------------------


@dataclass
class MaterialScene:
    """Inputs of hl_write_gbuffer for one view: per-pixel SURFACE records (the
    rasteriser's interpolated vertex outputs), GpuMaterial / GpuMaterialTextures tables,
    textures as (texels[h, w, 4], format, address_u, address_v, filter), the pass's
    GBufferGlobals and the depth the rasteriser wrote (1.0 where nothing is covered)."""
    camera: Camera
    surfaces: np.ndarray
    materials: np.ndarray
    material_textures: np.ndarray
    textures: list
    globals_: np.ndarray
    depth: np.ndarray

    @property
    def covered(self) -> np.ndarray:
        return self.surfaces["material_id"] != L.NO_FRAGMENT


def _texture(seed: int, stream: int, kind: str, size: int, fmt: int):
    n = size * size
    u = lambda k, lo=0.0, hi=1.0: uniform(seed, stream * 16 + k, n, lo, hi).reshape(size, size)
    yy, xx = np.meshgrid(np.arange(size) / size, np.arange(size) / size, indexing="ij")
    if kind == "normal":  # tangent-space normal map, z dominant, encoded n*0.5+0.5
        tx = 0.35 * np.sin(2 * math.pi * (3 * xx + u(0) * 0.1))
        ty = 0.35 * np.cos(2 * math.pi * (2 * yy + u(1) * 0.1))
        tz = np.sqrt(np.maximum(1.0 - tx * tx - ty * ty, 0.0))
        v = np.stack([tx * 0.5 + 0.5, ty * 0.5 + 0.5, tz * 0.5 + 0.5, np.ones_like(tx)], -1)
    else:  # smooth pattern plus noise, channels independent
        ch = [0.5 + 0.35 * np.sin(2 * math.pi * ((k + 1) * xx + (3 - k) * yy)) + 0.15 * (u(k) - 0.5) for k in range(4)]
        v = np.stack(ch, -1)
        if kind == "base" and stream % 2 == 0:  # opaque colour texture; the others are cut-outs
            v[..., 3] = 1.0
        if kind == "emissive":
            v = v * 2.0
    if fmt in (L.TEX_RGBA8_UNORM, L.TEX_RGBA8_SRGB):
        return np.clip(np.rint(np.clip(v, 0, 1) * 255.0), 0, 255).astype(np.uint8)
    return v.astype(np.float16 if fmt == L.TEX_RGBA16F else np.float32)


def material_scene(cam: Camera, seed: int, n_materials: int = 64, n_textures: int = 24, block: int = 48,
                   uncovered: float = 0.03, debug_mode: int = 0) -> MaterialScene:
    """A seeded scene for the G-buffer pass: pixels in ``block`` x ``block`` squares
    share a material; UVs vary smoothly (1 to 3 repeats across the view, so textures
    are magnified or 1:1); about ``uncovered`` of the pixels are not covered by any
    fragment. Textures: base colours sRGB RGBA8, normal maps and ORM maps RGBA8 unorm,
    emissive RGBA16F, some RGBA32F; sizes 128-512; mostly repeat and linear, some
    clamp-to-edge, mirrored-repeat and nearest. Materials: 80 % metallic workflow,
    60 % with a normal map, about a quarter with base alpha below 1 (some discarded by
    the 0.5 cutoff), some emissive."""
    W, H = cam.width, cam.height
    n = W * H
    depth, N, _, _, _ = _surface(cam, seed)
    r = lambda k, lo=0.0, hi=1.0, m=n: uniform(seed, 100 + k, m, lo, hi)

    # textures
    kinds = ["base", "normal", "orm", "emissive", "orm"]
    textures = []
    for t in range(n_textures):
        kind = kinds[t % len(kinds)]
        fmt = {"base": L.TEX_RGBA8_SRGB, "normal": L.TEX_RGBA8_UNORM, "orm": L.TEX_RGBA8_UNORM,
               "emissive": L.TEX_RGBA16F}[kind]
        if kind == "orm" and t % 3 == 0:
            fmt = L.TEX_RGBA32F
        size = (128, 256, 512)[t % 3]
        au = (L.ADDRESS_REPEAT, L.ADDRESS_REPEAT, L.ADDRESS_CLAMP_TO_EDGE, L.ADDRESS_MIRROR_REPEAT)[t % 4]
        av = (L.ADDRESS_REPEAT, L.ADDRESS_MIRROR_REPEAT, L.ADDRESS_REPEAT)[t % 3]
        filt = L.FILTER_NEAREST if t % 7 == 3 else L.FILTER_LINEAR
        textures.append((_texture(seed, 20 + t, kind, size, fmt), fmt, au, av, filt))
    by_kind = {k: [i for i in range(n_textures) if kinds[i % len(kinds)] == k] for k in set(kinds)}

    # materials
    M = n_materials
    mats = np.zeros(M, L.GPU_MATERIAL)
    alpha = np.where(r(1, m=M) < 0.25, r(2, 0.3, 1.0, M), 1.0)
    mats["base_color"] = np.stack([r(3, 0.2, 1.0, M), r(4, 0.2, 1.0, M), r(5, 0.2, 1.0, M), alpha], 1)
    emissive_w = np.where(r(6, m=M) < 0.2, r(7, 0.0, 4.0, M), 0.0)
    mats["emissive"] = np.stack([r(8, m=M), r(9, m=M), r(10, m=M), emissive_w], 1)
    mats["roughness_metallic"] = np.stack([r(11, 0.05, 1.0, M), (r(12, m=M) < 0.3) * r(13, 0.5, 1.0, M),
                                           r(14, 1.3, 1.8, M), r(15, m=M)], 1)
    for f in ("tex_base_color", "tex_normal", "tex_roughness", "tex_emissive", "tex_occlusion"):
        mats[f] = L.NO_TEXTURE
    mats["workflow"] = np.where(r(16, m=M) < 0.2, L.WORKFLOW_SPECULAR, L.WORKFLOW_METALLIC)
    mats["flags"] = np.where(r(17, m=M) < 0.6, L.FLAG_HAS_NORMAL_MAP, 0)
    mtex = L.missing_material_textures(M)
    pick = lambda k, pool, i: pool[int(r(30 + k, m=M)[i] * len(pool)) % len(pool)]
    for i in range(M):
        want = {"base_color": (0.8, "base"), "normal": (0.9 if mats["flags"][i] else 0.2, "normal"),
                "roughness_metallic": (0.7, "orm"), "emissive": (0.3, "emissive"), "occlusion": (0.5, "orm"),
                "specular_color": (0.6, "base"), "specular_weight": (0.6, "orm")}
        for k, (slot, (p, kind)) in enumerate(want.items()):
            if r(40 + k, m=M)[i] >= p or not by_kind.get(kind):
                continue
            s = mtex[slot][i]
            s["texture_index"] = pick(k, by_kind[kind], i)
            s["offset_scale"] = (r(50 + k, -1, 1, M)[i], r(60 + k, -1, 1, M)[i], r(70 + k, 0.5, 2, M)[i],
                                 r(80 + k, 0.5, 2, M)[i])
            ang = r(90 + k, 0, 2 * math.pi, M)[i] if r(97, m=M)[i] < 0.3 else 0.0
            s["rotation"] = (math.sin(ang), math.cos(ang), 0.0, 0.0)
            mtex[slot][i] = s
    mtex["params"] = np.stack([r(18, 0.5, 1.5, M), r(19, m=M), np.where(r(20, m=M) < 0.8, 0.5, 0.0), np.zeros(M)], 1)

    # per-pixel surfaces
    ys, xs = np.divmod(np.arange(n), W)
    bw = (W + block - 1) // block
    blk = (ys // block) * bw + xs // block
    nb = int(blk.max()) + 1
    mid = (uniform(seed, 200, nb) * M).astype(np.uint32)[blk]
    hole = r(21) < uncovered
    mid[hole] = L.NO_FRAGMENT
    srf = np.zeros(n, L.SURFACE)
    Nf = N.reshape(n, 3) * r(22, 0.8, 1.2)[:, None]  # interpolated normals are not unit length
    T0 = np.stack([r(23, -1, 1), r(24, -1, 1), r(25, -1, 1)], 1)
    srf["world_normal"] = Nf
    srf["bitangent_sign"] = np.where(r(26) < 0.5, -1.0, 1.0)
    srf["world_tangent"] = T0
    srf["material_id"] = mid
    rep = uniform(seed, 201, nb, 1.0, 3.0)[blk]
    off_u, off_v = uniform(seed, 202, nb, -1, 1)[blk], uniform(seed, 203, nb, -1, 1)[blk]
    srf["tex_coords"] = np.stack([(xs + 0.5) / W * rep + off_u, (ys + 0.5) / H * rep + off_v], 1)
    lm = np.where((mid % 2 == 0)[:, None], np.stack([r(27), r(28)], 1), -1.0)
    srf["lightmap_uv"] = lm
    d = depth.reshape(n).astype(np.float64)
    ndc_x = (xs + 0.5) / W * 2 - 1
    ndc_y = 1 - (ys + 0.5) / H * 2
    near, far = cam.near, cam.far
    w_clip = near * far / (far - d * (far - near))  # view depth of the stored NDC depth
    px, py = ndc_x + r(29, -0.01, 0.01), ndc_y + r(30, -0.01, 0.01)
    srf["prev_clip"] = np.stack([px * w_clip, py * w_clip, d * w_clip, w_clip], 1)
    depth = np.where(hole.reshape(H, W), np.float32(1.0), depth).astype(np.float32)

    glb = np.zeros(1, L.GBUFFER_GLOBALS)
    glb["ambient_color"] = (0.1, 0.1, 0.15, 1.0)
    glb["ambient_intensity"] = 0.1
    glb["rc_world_min"] = (-100.0,) * 4
    glb["rc_world_max"] = (100.0,) * 4
    glb["csm_splits"] = L.CSM_SPLITS
    glb["debug_mode"] = debug_mode
    glb["screen_width"], glb["screen_height"] = float(W), float(H)
    return MaterialScene(cam, srf.reshape(H, W), mats, mtex, textures, glb, depth)


# ----------------------------------------------------------------------------------
# Shadow maps: light-space matrices and depth atlases
# ----------------------------------------------------------------------------------


def orthographic_rh_dx(half_w: float, half_h: float, near: float, far: float) -> np.ndarray:
    """glam ``orthographic_rh`` (DirectX depth range [0, 1]) of a box centred on the axis."""
    m = np.eye(4)
    m[0, 0], m[1, 1] = 1.0 / half_w, 1.0 / half_h
    m[2, 2], m[2, 3] = 1.0 / (near - far), near / (near - far)
    return m


def _look(eye, d):
    d = np.asarray(d, np.float64)
    up = (1.0, 0.0, 0.0) if abs(d[1]) > 0.99 * np.linalg.norm(d) else (0.0, 1.0, 0.0)
    return look_at_rh(eye, np.asarray(eye, np.float64) + d, up)


SHADOW_CUBE_AXES = ((1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1))  # point_light_face order


@dataclass
class ShadowScene:
    """Shadow inputs for hl_shade_shadowed: ``lights`` with shadow_index set for the
    first ``n_shadowed`` lights (6 layers each, as GpuShadowMatrix lays them out),
    matrices (layers, 16) float32 column major, the config, and ``kinds[layer]`` =
    "persp" or "ortho" for the atlas generator."""
    lights: np.ndarray
    matrices: np.ndarray
    config: np.ndarray
    kinds: list
    max_lights: int


def shadow_scene(cam: Camera, lights: np.ndarray, n_shadowed: int, quality: str = "medium",
                 max_lights: int = L.MAX_SHADOW_LIGHTS) -> ShadowScene:
    """Light-space matrices for the first ``n_shadowed`` lights: six 90-degree cube faces
    for a point light, one perspective of the outer cone for a spot light, four
    orthographic cascades (half extents = the CSM splits) around the camera for a
    directional light; DirectX depth, near 0.05, far = the light's range (500 for
    cascades)."""
    lt = lights.copy()
    n_shadowed = min(n_shadowed, len(lt))
    mats = np.tile(np.eye(4).T.reshape(16).astype(np.float32), (6 * max(n_shadowed, 1), 1))
    kinds = ["persp"] * (6 * max(n_shadowed, 1))
    lt["shadow_index"] = L.NO_SHADOW
    for i in range(n_shadowed):
        base = 6 * i
        lt["shadow_index"][i] = base
        pos = lt["position_range"][i, :3].astype(np.float64)
        rng = float(lt["position_range"][i, 3])
        typ = int(lt["light_type"][i])
        d = lt["direction_outer"][i, :3].astype(np.float64)
        if typ == L.LIGHT_POINT:
            proj = perspective_rh_dx(math.radians(90.0), 1.0, 0.05, max(rng, 0.1))
            for f, ax in enumerate(SHADOW_CUBE_AXES):
                mats[base + f] = _cols(proj @ _look(pos, ax))
        elif typ == L.LIGHT_SPOT:
            half = math.acos(min(max(float(lt["direction_outer"][i, 3]), -1.0), 1.0))
            fov = min(max(2.0 * half, math.radians(2.0)), math.radians(170.0))
            mats[base] = _cols(perspective_rh_dx(fov, 1.0, 0.05, max(rng, 0.1)) @ _look(pos, d))
        else:  # directional: cascades around the camera
            dn = d / np.linalg.norm(d)
            for c, split in enumerate(L.CSM_SPLITS):
                view = _look(cam.eye - dn * 500.0, dn)
                mats[base + c] = _cols(orthographic_rh_dx(split, split, 0.1, 1000.0) @ view)
                kinds[base + c] = "ortho"
    return ShadowScene(lt, mats, L.shadow_config(quality), kinds, max_lights)


def shadow_atlases(kinds, size: int, seed: int, xp=np, device=None):
    """Dynamic and static Depth32Float atlases (layers, size, size): smooth depth fields
    per layer (sums of sinusoids with layer-dependent phases), in [0.99, 1] for
    perspective layers and [0.2, 1] for orthographic cascades, so that part of every
    layer's receivers is occluded; the static atlas is empty (1.0) outside blobs.
    ``xp`` is numpy or torch (with ``device``) for large atlases."""
    n = len(kinds)
    ph = uniform(seed, 300, 6 * n, 0.0, 2 * math.pi).reshape(n, 6)
    lo = np.array([0.99 if k == "persp" else 0.2 for k in kinds])
    if xp is np:
        t = np.arange(size, dtype=np.float64) / size
        Y, X = np.meshgrid(t, t, indexing="ij")
        dyn = np.empty((n, size, size), np.float32)
        sta = np.empty((n, size, size), np.float32)
        for i in range(n):
            a = 0.5 + 0.25 * np.sin(2 * math.pi * (3 * X + ph[i, 0])) + 0.25 * np.sin(2 * math.pi * (5 * Y + ph[i, 1]))
            b = np.sin(2 * math.pi * (2 * X + ph[i, 2])) * np.sin(2 * math.pi * (3 * Y + ph[i, 3]))
            dyn[i] = lo[i] + (1 - lo[i]) * np.clip(a, 0, 1)
            sta[i] = np.where(b > 0.5, lo[i] + (1 - lo[i]) * (1.5 - b), 1.0)
        return dyn, sta
    torch = xp
    t = torch.arange(size, dtype=torch.float32, device=device) / size
    Y, X = torch.meshgrid(t, t, indexing="ij")
    dyn = torch.empty((n, size, size), dtype=torch.float32, device=device)
    sta = torch.empty((n, size, size), dtype=torch.float32, device=device)
    for i in range(n):
        p = [float(v) for v in ph[i]]
        a = 0.5 + 0.25 * torch.sin(2 * math.pi * (3 * X + p[0])) + 0.25 * torch.sin(2 * math.pi * (5 * Y + p[1]))
        b = torch.sin(2 * math.pi * (2 * X + p[2])) * torch.sin(2 * math.pi * (3 * Y + p[3]))
        dyn[i] = float(lo[i]) + (1 - float(lo[i])) * a.clamp(0, 1)
        sta[i] = torch.where(b > 0.5, float(lo[i]) + (1 - float(lo[i])) * (1.5 - b), torch.ones_like(b))
    return dyn, sta


# ----------------------------------------------------------------------------------
# Radiance-cascade probes
# ----------------------------------------------------------------------------------


def rc_probes(seed: int, scale: float = 0.5) -> np.ndarray:
    """A synthetic rc_cascade0 texture, (1024, 64, 4) float16: every probe (x, y, z) of the
    16^3 grid and direction (dx, dy) holds a smooth irradiance in [0, scale) per channel,
    so the RC weight clamp(4 |irradiance|, 0, 1) takes partial and full values."""
    P, D = L.RC_PROBE_DIM, L.RC_DIR_DIM
    x = np.arange(P * D)[None, :] / (P * D)
    y = np.arange(P * P * D)[:, None] / (P * P * D)
    ph = uniform(seed, 400, 6, 0.0, 2 * math.pi)
    out = np.empty((P * P * D, P * D, 4), np.float16)
    for ch in range(3):
        v = 0.5 + 0.25 * np.sin(2 * math.pi * (3 * x + ph[ch])) + 0.25 * np.sin(2 * math.pi * (7 * y + ph[ch + 3]))
        out[..., ch] = (scale * v).astype(np.float16)
    out[..., 3] = np.float16(1.0)
    return out


def rc_globals(globals_rec: np.ndarray, world_min, world_max) -> np.ndarray:
    """A copy of a DeferredGlobals with radiance-cascade GI on over the given volume."""
    g = globals_rec.copy()
    g["has_rc_gi"] = 1
    g["rc_world_min"] = (*world_min, 0.0)
    g["rc_world_max"] = (*world_max, 0.0)
    return g


def reflection_images(width: int, height: int, seed: int):
    """Synthetic inputs of the reflection draw: (ssr, planar, lightmap_uv) as float16
    arrays (H, W, 4), (H, W, 4), (H, W, 2). SSR hits carry colour in [0, 4) and a
    confidence that is 0 on about a third of the pixels, partial elsewhere and 1 on a
    tenth; planar hits cover a horizontal band (confidence 0 outside it); lightmap UVs
    mix the no-lightmap sentinel (-1, -1), the virtual-geometry sentinel (-2, -2) and
    atlas UVs in [0, 1)."""
    rng = np.random.default_rng(seed)
    H, W = height, width
    ssr = np.empty((H, W, 4), np.float32)
    ssr[..., :3] = rng.uniform(0.0, 4.0, (H, W, 3))
    a = rng.uniform(0.0, 1.0, (H, W))
    a[rng.uniform(size=(H, W)) < 0.33] = 0.0
    a[rng.uniform(size=(H, W)) < 0.1] = 1.0
    ssr[..., 3] = a
    planar = np.zeros((H, W, 4), np.float32)
    band = slice(H // 2, H // 2 + max(1, H // 4))
    planar[band, :, :3] = rng.uniform(0.0, 2.0, (planar[band].shape[0], W, 3))
    planar[band, :, 3] = rng.uniform(0.2, 1.0, (planar[band].shape[0], W))
    lm = rng.uniform(0.0, 1.0, (H, W, 2)).astype(np.float32)
    k = rng.integers(0, 3, (H, W))
    lm[k == 0] = -1.0
    lm[k == 1] = -2.0
    return ssr.astype(np.float16), planar.astype(np.float16), lm.astype(np.float16)


def reflection_env(seed: int, face_size: int = 16, mip_levels: int = 5, layers: int = 5, n_captures: int = 6):
    """Reflection captures and their cube-map array for the reflection draw's
    environment term: a dict with ``captures`` (REFLECTION_CAPTURE records: spheres and
    oriented boxes of radius / half-extent 10-35 placed in front of the default camera,
    cubemap layers 1.., one capture without a cubemap), ``texels`` (float16 RGBA cube
    array, layer-major, 6 faces, each face's mip chain; radiance in [0, 3), alpha 1),
    ``face_size``, ``mip_levels`` and ``layers`` (layer 0 is the skylight)."""
    rng = np.random.default_rng(seed)
    chain = sum(max(1, face_size >> m) ** 2 for m in range(mip_levels))
    texels = np.ones((layers * 6 * chain, 4), np.float32)
    texels[:, :3] = rng.uniform(0.0, 3.0, (layers * 6 * chain, 3))
    caps = np.zeros(n_captures, L.REFLECTION_CAPTURE)
    for i in range(n_captures):
        centre = np.array([rng.uniform(-25, 25), rng.uniform(-12, 12), rng.uniform(-90, -10)])
        box = i % 2 == 1
        caps[i]["position_radius"] = (*centre, rng.uniform(10.0, 35.0))
        caps[i]["cubemap_index"] = 1 + i % (layers - 1) if i != n_captures - 1 else -1
        caps[i]["shape"] = L.CAPTURE_BOX if box else L.CAPTURE_SPHERE
        caps[i]["brightness"] = rng.uniform(0.5, 2.0)
        m = np.eye(4)
        if box:
            a = rng.uniform(0.0, 2.0 * math.pi)
            rot = np.array([[math.cos(a), 0.0, math.sin(a)], [0.0, 1.0, 0.0], [-math.sin(a), 0.0, math.cos(a)]])
            m[:3, :3] = rot.T
            m[:3, 3] = -rot.T @ centre
            caps[i]["extents_transition"] = (*rng.uniform(8.0, 30.0, 3), rng.uniform(0.5, 4.0))
        caps[i]["world_to_local"] = m.T.reshape(16).astype(np.float32)  # column major
    return dict(captures=caps, texels=texels.astype(np.float16), face_size=face_size, mip_levels=mip_levels,
                layers=layers)
