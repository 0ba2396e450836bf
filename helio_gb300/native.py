"""ctypes binding of the C ABI (include/helio_gb300.h).

The library ``helio_gb300/_lib/libhelio_gb300.so`` is built by
``helio_gb300.build``. There is no fallback: if the library is missing or no CUDA
device is usable, every call raises. Device memory is passed as raw pointers; the
helpers accept torch CUDA tensors for convenience (``tensor.data_ptr()``).
"""
from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from . import build as _build

HL_OK = 0
HL_ERR_INVALID_ARGUMENT = -1
HL_ERR_LAYOUT = -2
HL_ERR_SIZE = -3
HL_ERR_CUDA = -4
HL_ERR_TIMEOUT = -5
HL_ERR_CAPACITY = -6
HL_ERR_DEVICE_BOUNDS = -7
HL_ERR_NOT_SUPPORTED = -8

GBUF_REFERENCE, GBUF_F32, GBUF_F16 = 0, 1, 2
GRID_TILES, GRID_FROXELS = 0, 1
TARGET_RGBA32F, TARGET_RGBA16F = 0, 1
MAX_PLANES = 6


class HelioError(RuntimeError):
    """A non-OK status returned by the C ABI."""

    def __init__(self, status: int, message: str):
        super().__init__(f"[{status}] {message}")
        self.status = status


class FroxelParams(C.Structure):
    _fields_ = [
        ("grid_x", C.c_uint32), ("grid_y", C.c_uint32), ("grid_z", C.c_uint32),
        ("width", C.c_uint32), ("height", C.c_uint32),
        ("slice_near", C.c_float), ("slice_far", C.c_float), ("reserved", C.c_uint32),
    ]


class FroxelLists(C.Structure):
    _fields_ = [("offsets", C.c_void_p), ("indices", C.c_void_p), ("capacity", C.c_uint32), ("reserved", C.c_uint32)]


class GBuffer(C.Structure):
    _fields_ = [
        ("layout", C.c_uint32), ("width", C.c_uint32), ("height", C.c_uint32), ("reserved", C.c_uint32),
        ("planes", C.c_void_p * MAX_PLANES), ("pitch", C.c_uint64 * MAX_PLANES),
    ]


class LightGrid(C.Structure):
    _fields_ = [
        ("kind", C.c_uint32), ("lists_capacity", C.c_uint32),
        ("lists", C.c_void_p), ("counts", C.c_void_p), ("froxel", FroxelParams),
    ]


class Target(C.Structure):
    _fields_ = [("data", C.c_void_p), ("pitch", C.c_uint64), ("format", C.c_uint32), ("reserved", C.c_uint32)]


class View(C.Structure):
    _fields_ = [("camera", C.c_void_p), ("gbuffer", GBuffer), ("radiance", Target)]


class BatchConfig(C.Structure):
    _fields_ = [
        ("autotune", C.c_uint32), ("grid_x", C.c_uint32), ("grid_y", C.c_uint32), ("grid_z", C.c_uint32),
        ("cache_path", C.c_char_p),
    ]


class FragmentParams(C.Structure):
    _fields_ = [("mode", C.c_uint32), ("num_tiles_x", C.c_uint32), ("ambient_intensity", C.c_float),
                ("ambient_color", C.c_float * 3)]


FRAGMENTS_FORWARD, FRAGMENTS_TRANSPARENT = 0, 1

GBUFFER_TARGETS = 8
MAX_MATERIAL_TEXTURES = 256


class Texture(C.Structure):
    """hl_texture: a texture's level 0 (device texels) and its sampler."""
    _fields_ = [("texels", C.c_void_p), ("pitch", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32),
                ("format", C.c_uint32), ("address_u", C.c_uint32), ("address_v", C.c_uint32),
                ("filter", C.c_uint32)]


class ShadowMaps(C.Structure):
    """hl_shadow_maps: two Depth32Float atlases, the light matrices and ShadowConfig."""
    _fields_ = [("dynamic_atlas", C.c_void_p), ("static_atlas", C.c_void_p), ("matrices", C.c_void_p),
                ("config", C.c_void_p), ("size", C.c_uint32), ("layers", C.c_uint32),
                ("max_shadow_lights", C.c_uint32), ("reserved", C.c_uint32)]


class RcCascade(C.Structure):
    """hl_rc_cascade: the radiance-cascade probe texture (RGBA16F)."""
    _fields_ = [("texels", C.c_void_p), ("pitch", C.c_uint64), ("width", C.c_uint32), ("height", C.c_uint32)]


class ShadeBindings(C.Structure):
    """hl_shade_bindings: optional shadow maps and radiance-cascade probes."""
    _fields_ = [("shadows", C.POINTER(ShadowMaps)), ("rc", C.POINTER(RcCascade))]


class ReflectionEnv(C.Structure):
    """hl_reflection_env: reflection captures and their pre-filtered cube-map array."""
    _fields_ = [("captures", C.c_void_p), ("count", C.c_uint32), ("face_size", C.c_uint32),
                ("mip_levels", C.c_uint32), ("layers", C.c_uint32), ("texels", C.c_void_p)]


class ReflectionInputs(C.Structure):
    """hl_reflection_inputs: SSR and planar hit images (RGBA16F), lightmap UVs (RG16F),
    radiance-cascade probes and the capture environment, each optional (NULL)."""
    _fields_ = [("ssr", C.c_void_p), ("ssr_pitch", C.c_uint64), ("planar", C.c_void_p),
                ("planar_pitch", C.c_uint64), ("lightmap_uv", C.c_void_p), ("lightmap_uv_pitch", C.c_uint64),
                ("rc", C.POINTER(RcCascade)), ("env", C.POINTER(ReflectionEnv))]


class GBufferTargets(C.Structure):
    """hl_gbuffer_targets: albedo, normal, orm, emissive (required), lightmap_uv, sss,
    extra, velocity (optional)."""
    _fields_ = [("width", C.c_uint32), ("height", C.c_uint32), ("reserved", C.c_uint32 * 2),
                ("planes", C.c_void_p * GBUFFER_TARGETS), ("pitch", C.c_uint64 * GBUFFER_TARGETS)]


EXPORTS = [
    "hl_abi_version", "hl_status_string", "hl_create", "hl_destroy", "hl_last_error_message", "hl_sync_status",
    "hl_tile_count", "hl_bin_tiles_ref", "hl_froxel_slice_table", "hl_bin_froxels", "hl_shade", "hl_shade_stats",
    "hl_shade_adjoint", "hl_batch_plan_create", "hl_batch_execute", "hl_batch_plan_view_grid",
    "hl_batch_plan_destroy", "hl_probe_fp32_peak", "hl_bin_froxels_noalloc", "hl_shade_fragments",
    "hl_write_gbuffer", "hl_shade_shadowed", "hl_shade_ex", "hl_shade_reflections", "hl_set_pair_log",
    "hl_inject_binning_stall",
]

_lock = threading.Lock()
_lib = None


def lib_path() -> Path:
    return _build.lib_path()


def load(path: Path | None = None):
    """Load (once) and bind the shared library. Raises if it has not been built."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else lib_path()
        if not p.exists():
            raise RuntimeError(f"helio_gb300 CUDA library not built: {p} missing (run helio_gb300.build.build())")
        l = C.CDLL(str(p))
        _bind(l)
        if path is None:
            _lib = l
        return l


def _bind(l):
    vp, u32, i32 = C.c_void_p, C.c_uint32, C.c_int32
    P = C.POINTER
    l.hl_abi_version.restype = u32
    l.hl_status_string.restype = C.c_char_p
    l.hl_status_string.argtypes = [i32]
    l.hl_create.argtypes = [P(vp), C.c_int]
    l.hl_create.restype = i32
    l.hl_destroy.argtypes = [vp]
    l.hl_destroy.restype = i32
    l.hl_last_error_message.argtypes = [vp]
    l.hl_last_error_message.restype = C.c_char_p
    l.hl_sync_status.argtypes = [vp, vp]
    l.hl_sync_status.restype = i32
    l.hl_tile_count.argtypes = [u32, u32]
    l.hl_tile_count.restype = u32
    l.hl_bin_tiles_ref.argtypes = [vp, vp, vp, u32, u32, u32, vp, vp, vp]
    l.hl_bin_tiles_ref.restype = i32
    l.hl_froxel_slice_table.argtypes = [P(FroxelParams), P(C.c_float)]
    l.hl_froxel_slice_table.restype = i32
    l.hl_bin_froxels.argtypes = [vp, vp, vp, u32, P(FroxelParams), P(FroxelLists), vp]
    l.hl_bin_froxels.restype = i32
    l.hl_shade.argtypes = [vp, vp, vp, P(GBuffer), vp, u32, P(LightGrid), P(Target), vp]
    l.hl_shade.restype = i32
    l.hl_shade_stats.argtypes = [vp, vp, vp, P(GBuffer), vp, u32, P(LightGrid), vp, vp]
    l.hl_shade_stats.restype = i32
    l.hl_inject_binning_stall.argtypes = [vp, u32, u32]
    l.hl_inject_binning_stall.restype = i32
    l.hl_set_pair_log.argtypes = [vp, vp, u32, vp]
    l.hl_set_pair_log.restype = i32
    l.hl_shade_adjoint.argtypes = [vp, vp, vp, P(GBuffer), vp, u32, P(LightGrid), vp, C.c_uint64, vp, vp, vp]
    l.hl_shade_adjoint.restype = i32
    l.hl_batch_plan_create.argtypes = [vp, P(View), u32, vp, u32, vp, P(BatchConfig), P(vp), vp]
    l.hl_batch_plan_create.restype = i32
    l.hl_batch_execute.argtypes = [vp, vp, vp]
    l.hl_batch_execute.restype = i32
    l.hl_batch_plan_view_grid.argtypes = [vp, u32, P(u32)]
    l.hl_batch_plan_view_grid.restype = i32
    l.hl_batch_plan_destroy.argtypes = [vp]
    l.hl_batch_plan_destroy.restype = i32
    l.hl_probe_fp32_peak.argtypes = [vp, P(C.c_double)]
    l.hl_probe_fp32_peak.restype = i32
    l.hl_bin_froxels_noalloc.argtypes = [vp, vp, u32, P(FroxelParams), P(FroxelLists), vp]
    l.hl_bin_froxels_noalloc.restype = i32
    l.hl_shade_fragments.argtypes = [vp, vp, P(FragmentParams), vp, u32, vp, u32, vp, vp, u32, P(LightGrid), vp, vp]
    l.hl_shade_fragments.restype = i32
    l.hl_write_gbuffer.argtypes = [vp, vp, vp, C.c_uint64, vp, vp, u32, P(Texture), u32, P(GBufferTargets), vp]
    l.hl_write_gbuffer.restype = i32
    l.hl_shade_shadowed.argtypes = [vp, vp, vp, P(GBuffer), vp, u32, P(LightGrid), P(ShadowMaps), P(Target), vp]
    l.hl_shade_shadowed.restype = i32
    l.hl_shade_ex.argtypes = [vp, vp, vp, P(GBuffer), vp, u32, P(LightGrid), P(ShadeBindings), P(Target), vp]
    l.hl_shade_ex.restype = i32
    l.hl_shade_reflections.argtypes = [vp, vp, vp, P(GBuffer), P(ReflectionInputs), P(Target), vp]
    l.hl_shade_reflections.restype = i32


def status_string(status: int) -> str:
    return load().hl_status_string(status).decode()


def froxel_params(grid_x, grid_y, grid_z, width, height, slice_far, slice_near=0.5) -> FroxelParams:
    return FroxelParams(grid_x, grid_y, grid_z, width, height, slice_near, slice_far, 0)


def froxel_params_from_numpy(p) -> FroxelParams:
    r = p[0] if getattr(p, "shape", ()) else p
    return FroxelParams(int(r["grid_x"]), int(r["grid_y"]), int(r["grid_z"]), int(r["width"]), int(r["height"]),
                        float(r["slice_near"]), float(r["slice_far"]), 0)


def slice_table(params: FroxelParams):
    out = (C.c_float * (params.grid_z + 1))()
    st = load().hl_froxel_slice_table(C.byref(params), out)
    if st != HL_OK:
        raise HelioError(st, status_string(st))
    return list(out)


def _ptr(x) -> int:
    if x is None:
        return 0
    if isinstance(x, int):
        return x
    return int(x.data_ptr())


def _stream(stream) -> int:
    if stream is None:
        return 0
    if isinstance(stream, int):
        return stream
    return int(stream.cuda_stream)


def gbuffer_struct(layout: int, width: int, height: int, planes, pitches=None) -> GBuffer:
    """``planes``: device tensors (or pointers) in the layout's plane order;
    ``pitches`` default to the tensors' row strides in bytes."""
    g = GBuffer()
    g.layout, g.width, g.height, g.reserved = layout, width, height, 0
    for i, pl in enumerate(planes):
        g.planes[i] = _ptr(pl)
        if pitches is not None:
            g.pitch[i] = int(pitches[i])
        else:
            g.pitch[i] = int(pl.stride(0) * pl.element_size())
    return g


class Context:
    """Owns an ``hl_ctx``. Methods mirror the C ABI and raise ``HelioError``."""

    def __init__(self, device: int = 0):
        self._l = load()
        h = C.c_void_p()
        st = self._l.hl_create(C.byref(h), device)
        if st != HL_OK:
            raise HelioError(st, f"hl_create(device={device}) failed: {status_string(st)}")
        self._h = h
        self.device = device

    @property
    def handle(self):
        return self._h

    def close(self):
        if getattr(self, "_h", None):
            self._l.hl_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, st: int, what: str):
        if st != HL_OK:
            msg = self._l.hl_last_error_message(self._h).decode()
            raise HelioError(st, f"{what}: {status_string(st)}: {msg}")

    def probe_fp32_peak(self) -> float:
        """Measured FP32 FMA throughput in TFLOP/s."""
        v = C.c_double()
        self._check(self._l.hl_probe_fp32_peak(self._h, C.byref(v)), "hl_probe_fp32_peak")
        return float(v.value)

    def sync_status(self, stream=None):
        self._check(self._l.hl_sync_status(self._h, _stream(stream)), "hl_sync_status")

    def bin_tiles_ref(self, camera, lights, n_lights, width, height, tile_lists, tile_counts, stream=None):
        self._check(self._l.hl_bin_tiles_ref(self._h, _ptr(camera), _ptr(lights), n_lights, width, height,
                                             _ptr(tile_lists), _ptr(tile_counts), _stream(stream)), "hl_bin_tiles_ref")

    def bin_froxels(self, camera, lights, n_lights, params: FroxelParams, offsets, indices, capacity, stream=None):
        out = FroxelLists(_ptr(offsets), _ptr(indices), capacity, 0)
        self._check(self._l.hl_bin_froxels(self._h, _ptr(camera), _ptr(lights), n_lights, C.byref(params),
                                           C.byref(out), _stream(stream)), "hl_bin_froxels")

    def shade(self, camera, globals_, gbuffer: GBuffer, lights, n_lights, grid: LightGrid, target: Target, stream=None):
        self._check(self._l.hl_shade(self._h, _ptr(camera), _ptr(globals_), C.byref(gbuffer), _ptr(lights), n_lights,
                                     C.byref(grid), C.byref(target), _stream(stream)), "hl_shade")

    def shade_shadowed(self, camera, globals_, gbuffer: GBuffer, lights, n_lights, grid: LightGrid,
                       shadows: "ShadowMaps", target: Target, stream=None):
        """hl_shade with the shadow term (shadows=None: plain hl_shade)."""
        self._check(self._l.hl_shade_shadowed(self._h, _ptr(camera), _ptr(globals_), C.byref(gbuffer), _ptr(lights),
                                              n_lights, C.byref(grid), C.byref(shadows) if shadows else None,
                                              C.byref(target), _stream(stream)), "hl_shade_shadowed")

    def shade_ex(self, camera, globals_, gbuffer: GBuffer, lights, n_lights, grid: LightGrid, target: Target,
                 shadows: "ShadowMaps" = None, rc: "RcCascade" = None, stream=None):
        """hl_shade with the optional bindings (shadow maps, radiance-cascade probes)."""
        b = ShadeBindings()
        b.shadows = C.pointer(shadows) if shadows is not None else None
        b.rc = C.pointer(rc) if rc is not None else None
        self._check(self._l.hl_shade_ex(self._h, _ptr(camera), _ptr(globals_), C.byref(gbuffer), _ptr(lights),
                                        n_lights, C.byref(grid), C.byref(b), C.byref(target), _stream(stream)),
                    "hl_shade_ex")

    def shade_reflections(self, camera, globals_, gbuffer: GBuffer, target: Target, ssr=None, planar=None,
                          lightmap_uv=None, rc: "RcCascade" = None, env: "ReflectionEnv" = None, stream=None):
        """The reflection draw (fs_reflection) added over ``target``; ``ssr`` / ``planar``:
        device float16 tensors (H, W, 4), ``lightmap_uv``: (H, W, 2), ``env``: captures
        and cube array (reflection_env_struct), each optional."""
        inp = ReflectionInputs()
        for name, t in (("ssr", ssr), ("planar", planar), ("lightmap_uv", lightmap_uv)):
            if t is not None:
                setattr(inp, name, _ptr(t))
                setattr(inp, name + "_pitch", int(t.stride(0) * t.element_size()))
        inp.rc = C.pointer(rc) if rc is not None else None
        inp.env = C.pointer(env) if env is not None else None
        self._check(self._l.hl_shade_reflections(self._h, _ptr(camera), _ptr(globals_), C.byref(gbuffer),
                                                 C.byref(inp), C.byref(target), _stream(stream)),
                    "hl_shade_reflections")

    def shade_stats(self, camera, globals_, gbuffer: GBuffer, lights, n_lights, grid: LightGrid, counts, stream=None):
        self._check(self._l.hl_shade_stats(self._h, _ptr(camera), _ptr(globals_), C.byref(gbuffer), _ptr(lights),
                                           n_lights, C.byref(grid), _ptr(counts), _stream(stream)), "hl_shade_stats")

    def inject_binning_stall(self, item: int, spins: int):
        """The next bin_froxels on this context runs with work item ``item`` withholding
        its running total; the others give up after ``spins`` polls (HL_ERR_TIMEOUT)."""
        self._check(self._l.hl_inject_binning_stall(self._h, item, spins), "hl_inject_binning_stall")

    def set_pair_log(self, pairs=None, count=None):
        """Record the (pixel, light) pairs later shading launches light into ``pairs``
        (int32 device tensor (capacity, 2)) and ``count`` (int32 device tensor, zeroed by
        the caller); ``pairs=None`` stops recording."""
        if pairs is None:
            self._check(self._l.hl_set_pair_log(self._h, None, 0, None), "hl_set_pair_log")
        else:
            self._check(self._l.hl_set_pair_log(self._h, _ptr(pairs), int(pairs.shape[0]), _ptr(count)),
                        "hl_set_pair_log")

    def shade_adjoint(self, camera, globals_, gbuffer: GBuffer, lights, n_lights, grid: LightGrid, d_radiance,
                      d_radiance_pitch, d_lights, d_pixels, stream=None):
        self._check(self._l.hl_shade_adjoint(self._h, _ptr(camera), _ptr(globals_), C.byref(gbuffer), _ptr(lights),
                                             n_lights, C.byref(grid), _ptr(d_radiance), int(d_radiance_pitch),
                                             _ptr(d_lights), _ptr(d_pixels), _stream(stream)), "hl_shade_adjoint")

    def shade_fragments(self, camera, params: FragmentParams, fragments, n_fragments, lights, n_lights,
                        grid: LightGrid, out_rgba, entity_indices=None, transforms=None, n_transforms=0, stream=None):
        """Forward+ / transparent light loops over hl_fragment records (80 B each)."""
        self._check(self._l.hl_shade_fragments(self._h, _ptr(camera), C.byref(params), _ptr(fragments), n_fragments,
                                               _ptr(lights), n_lights, _ptr(entity_indices), _ptr(transforms),
                                               n_transforms, C.byref(grid), _ptr(out_rgba), _stream(stream)),
                    "hl_shade_fragments")

    def write_gbuffer(self, globals_, surfaces, surfaces_pitch, materials, material_textures, n_materials,
                      textures, targets: "GBufferTargets", stream=None):
        """G-buffer pass fragment stage; ``textures`` is a list of ``Texture``."""
        arr = (Texture * max(1, len(textures)))(*textures)
        self._check(self._l.hl_write_gbuffer(self._h, _ptr(globals_), _ptr(surfaces), int(surfaces_pitch),
                                             _ptr(materials), _ptr(material_textures), n_materials, arr,
                                             len(textures), C.byref(targets), _stream(stream)), "hl_write_gbuffer")

    def batch_plan(self, views, lights, n_lights, globals_, grid=None, autotune=False, cache_path=None,
                   stream=None) -> "BatchPlan":
        """Plan lighting every view of ``views`` (a list of ``View``) with one light buffer:
        ``grid`` = (gx, gy, gz) for every view, or ``autotune`` to time candidate grids per
        view size (results kept in ``cache_path`` if given)."""
        arr = (View * len(views))(*views)
        cfg = BatchConfig()
        cfg.autotune = 1 if autotune else 0
        cfg.grid_x, cfg.grid_y, cfg.grid_z = grid if grid is not None else (0, 0, 0)
        cfg.cache_path = cache_path.encode() if cache_path else None
        h = C.c_void_p()
        self._check(self._l.hl_batch_plan_create(self._h, arr, len(views), _ptr(lights), n_lights, _ptr(globals_),
                                                 C.byref(cfg), C.byref(h), _stream(stream)), "hl_batch_plan_create")
        return BatchPlan(self, h, len(views))


class BatchPlan:
    """A plan of hl_batch_plan_create; ``execute`` replays its CUDA graph."""

    def __init__(self, ctx: Context, handle, n_views: int):
        self._ctx, self._h, self.n_views = ctx, handle, n_views

    def execute(self, stream=None):
        self._ctx._check(self._ctx._l.hl_batch_execute(self._ctx.handle, self._h, _stream(stream)), "hl_batch_execute")

    def view_grid(self, view: int):
        g = (C.c_uint32 * 3)()
        st = self._ctx._l.hl_batch_plan_view_grid(self._h, view, g)
        if st != HL_OK:
            raise HelioError(st, f"hl_batch_plan_view_grid: {status_string(st)}")
        return tuple(int(v) for v in g)

    def close(self):
        if getattr(self, "_h", None):
            self._ctx._l.hl_batch_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def view_struct(camera, gbuffer: GBuffer, target: Target) -> View:
    v = View()
    v.camera = _ptr(camera)
    v.gbuffer = gbuffer
    v.radiance = target
    return v


def tile_grid_struct(lists, counts) -> LightGrid:
    g = LightGrid()
    g.kind, g.lists_capacity, g.lists, g.counts = GRID_TILES, 0, _ptr(lists), _ptr(counts)
    return g


def froxel_grid_struct(indices, offsets, params: FroxelParams, capacity: int = 0) -> LightGrid:
    g = LightGrid()
    g.kind, g.lists_capacity, g.lists, g.counts = GRID_FROXELS, capacity, _ptr(indices), _ptr(offsets)
    g.froxel = params
    return g


def target_struct(data, fmt: int = TARGET_RGBA32F, pitch: int | None = None) -> Target:
    t = Target()
    t.data = _ptr(data)
    t.pitch = int(pitch if pitch is not None else data.stride(0) * data.element_size())
    t.format = fmt
    return t


def texture_struct(texels, fmt: int, address_u: int = 0, address_v: int = 0, filt: int = 1) -> Texture:
    """``texels``: a device tensor of shape (h, w, 4) (uint8, float16 or float32)."""
    t = Texture()
    t.texels = _ptr(texels)
    t.pitch = int(texels.stride(0) * texels.element_size())
    t.height, t.width = int(texels.shape[0]), int(texels.shape[1])
    t.format, t.address_u, t.address_v, t.filter = fmt, address_u, address_v, filt
    return t


def shadow_maps_struct(dynamic, static, matrices, config, max_shadow_lights: int = 42) -> ShadowMaps:
    """``dynamic``/``static``: device tensors (layers, size, size) float32; ``matrices``:
    device tensor of GpuShadowMatrix records; ``config``: device ShadowConfig bytes."""
    m = ShadowMaps()
    m.dynamic_atlas, m.static_atlas = _ptr(dynamic), _ptr(static)
    m.matrices, m.config = _ptr(matrices), _ptr(config)
    m.layers, m.size = int(dynamic.shape[0]), int(dynamic.shape[1])
    m.max_shadow_lights = max_shadow_lights
    return m


def reflection_env_struct(captures, n_captures: int, texels, face_size: int, mip_levels: int,
                          layers: int) -> ReflectionEnv:
    """hl_reflection_env over device tensors: ``captures`` (n x 112 bytes), ``texels``
    (RGBA16F cube array, layer-major, 6 faces, each face's mip chain)."""
    return ReflectionEnv(_ptr(captures), n_captures, face_size, mip_levels, layers, _ptr(texels))


def rc_cascade_struct(texels) -> RcCascade:
    """``texels``: a device float16 tensor (height, width, 4)."""
    r = RcCascade()
    r.texels = _ptr(texels)
    r.pitch = int(texels.stride(0) * texels.element_size())
    r.height, r.width = int(texels.shape[0]), int(texels.shape[1])
    return r


def gbuffer_targets_struct(width: int, height: int, planes) -> GBufferTargets:
    """``planes``: 8 device tensors or None (albedo, normal, orm, emissive, lightmap_uv,
    sss, extra, velocity); pitches are the tensors' row strides in bytes."""
    t = GBufferTargets()
    t.width, t.height = width, height
    for i, pl in enumerate(planes):
        if pl is None:
            continue
        t.planes[i] = _ptr(pl)
        t.pitch[i] = int(pl.stride(0) * pl.element_size())
    return t


NOALLOC_MAX_LIGHTS = 4096
NOALLOC_MAX_FROXELS = 32768


def bin_froxels_noalloc(camera, lights, n_lights, params: FroxelParams, offsets, indices, capacity, stream=None):
    """Froxel clustering without a context and without device allocation, for callers
    that cannot allocate (their frame runs inside a stream capture, or a pool owns all
    device memory). Scratch lives in one static device array of the library, so calls
    that overlap on the GPU race; make the first call on a device before any capture.
    Raises HelioError (HL_ERR_SIZE beyond NOALLOC_MAX_LIGHTS / NOALLOC_MAX_FROXELS)."""
    out = FroxelLists(_ptr(offsets), _ptr(indices), capacity, 0)
    st = load().hl_bin_froxels_noalloc(_ptr(camera), _ptr(lights), n_lights, C.byref(params), C.byref(out),
                                       _stream(stream))
    if st != HL_OK:
        raise HelioError(st, f"hl_bin_froxels_noalloc: {status_string(st)}")
