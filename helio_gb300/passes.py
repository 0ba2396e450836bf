"""Host-side mirror of the reference's pass interface for the deferred-lighting path.

The reference drives this path through ``helio_core::RenderPass``
(helio-core/src/traits.rs:315-530): ``name``, ``reads``/``writes``,
``prepare``, ``execute``, ``publish`` and ``on_resize``. The classes here keep the
same names, resource names, caching and error behaviour, and run the CUDA library
through the C ABI instead of wgpu:

- ``LightCullPass``     helio-pass-light-cull/src/lib.rs:41-362 — tile lists, the
                        (camera_gen, lights_gen, light_count) cull cache, clearing on
                        zero lights, "tile grid overflow" on oversize viewports.
- ``FroxelCullPass``    same interface, froxel lists (no reference counterpart).
- ``DeferredLightPass`` helio-pass-deferred-light/src/lib.rs:110-1199 — reads the
                        G-buffer and the published light grid, writes ``pre_aa``;
                        a missing G-buffer is ``InvalidPassConfig``
                        (deferred-light/src/lib.rs:914-919).

Device buffers are torch CUDA tensors (PyTorch is the allocator here, not the
compute path).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import layouts as L
from . import native as N


class InvalidPassConfig(RuntimeError):
    """helio_core::Error::InvalidPassConfig (helio-core/src/error.rs:63-92)."""


@dataclass
class SceneResources:
    """What passes read from the scene (helio-core/src/scene/resources.rs:129-255):
    the camera and light buffers with their generation counters."""

    camera: object  # device tensor, GpuCameraUniforms bytes
    lights: object  # device tensor, GpuLight[n] bytes
    movable_light_count: int
    camera_generation: int = 0
    movable_lights_generation: int = 0


@dataclass
class FrameResources:
    """Per-frame resource table (libhelio/src/frame.rs:229-234,486-491): passes
    publish buffers here for later passes to read."""

    entries: dict = field(default_factory=dict)

    def write(self, name, value, writer):
        self.entries[name] = (value, writer)

    def get(self, name):
        v = self.entries.get(name)
        return None if v is None else v[0]


@dataclass
class PassContext:
    ctx: N.Context
    scene: SceneResources
    frame: FrameResources
    width: int
    height: int
    stream: object = None


def _torch():
    import torch

    return torch


class LightCullPass:
    """Tile light culling (helio-pass-light-cull)."""

    TILE_SIZE = L.TILE_SIZE
    MAX_LIGHTS_PER_TILE = L.MAX_LIGHTS_PER_TILE

    def __init__(self, width: int, height: int, device="cuda"):
        self.device = device
        self.cull_cache_key = None
        self.on_resize(width, height)

    def name(self):
        return "LightCull"

    def reads(self):
        return ()

    def writes(self):
        return ("tile_light_lists", "tile_light_counts")

    def on_resize(self, width: int, height: int):
        tx, ty = L.tile_grid(width, height)
        tiles = tx * ty
        if tiles * self.MAX_LIGHTS_PER_TILE * 4 >= 1 << 32:
            raise OverflowError("tile grid overflow: viewport dimensions too large")
        torch = _torch()
        self.tile_light_lists = torch.zeros(max(tiles * self.MAX_LIGHTS_PER_TILE, 1), dtype=torch.int32, device=self.device)
        self.tile_light_counts = torch.zeros(max(tiles, 1), dtype=torch.int32, device=self.device)
        self.num_tiles_x, self.num_tiles_y = tx, ty
        self.width, self.height = width, height
        self.cull_cache_key = None

    def prepare(self, pc: PassContext):
        self.num_tiles_x, self.num_tiles_y = L.tile_grid(pc.width, pc.height)

    def execute(self, pc: PassContext):
        key = (pc.scene.camera_generation, pc.scene.movable_lights_generation, pc.scene.movable_light_count)
        if pc.scene.movable_light_count == 0:
            self.cull_cache_key = None  # the library clears both buffers
        elif self.cull_cache_key == key:
            return  # camera, lights and count unchanged: reuse last frame's lists
        else:
            self.cull_cache_key = key
        pc.ctx.bin_tiles_ref(pc.scene.camera, pc.scene.lights, pc.scene.movable_light_count, self.width, self.height,
                             self.tile_light_lists, self.tile_light_counts, pc.stream)

    def publish(self, frame: FrameResources):
        frame.write("tile_light_lists", self.tile_light_lists, "LightCull")
        frame.write("tile_light_counts", self.tile_light_counts, "LightCull")
        frame.write("light_grid", N.tile_grid_struct(self.tile_light_lists, self.tile_light_counts), "LightCull")


class FroxelCullPass:
    """Froxel light clustering with the same pass interface."""

    def __init__(self, width: int, height: int, grid=(16, 9, 24), far: float = 100.0, capacity: int | None = None,
                 device="cuda"):
        self.grid = tuple(grid)
        self.far = far
        self.device = device
        self.capacity = capacity
        self.cull_cache_key = None
        self.on_resize(width, height)

    def name(self):
        return "FroxelCull"

    def reads(self):
        return ()

    def writes(self):
        return ("froxel_offsets", "froxel_indices")

    def on_resize(self, width: int, height: int):
        torch = _torch()
        gx, gy, gz = self.grid
        self.params = N.froxel_params(gx, gy, gz, width, height, self.far)
        F = gx * gy * gz
        self.offsets = torch.zeros(F + 1, dtype=torch.int32, device=self.device)
        cap = self.capacity if self.capacity is not None else max(1024, F * 64)
        self.indices = torch.zeros(cap, dtype=torch.int32, device=self.device)
        self.width, self.height = width, height
        self.cull_cache_key = None

    def prepare(self, pc: PassContext):
        pass

    def execute(self, pc: PassContext):
        key = (pc.scene.camera_generation, pc.scene.movable_lights_generation, pc.scene.movable_light_count)
        if self.cull_cache_key == key:
            return
        self.cull_cache_key = key
        pc.ctx.bin_froxels(pc.scene.camera, pc.scene.lights, pc.scene.movable_light_count, self.params, self.offsets,
                           self.indices, self.indices.numel(), pc.stream)

    def publish(self, frame: FrameResources):
        frame.write("froxel_offsets", self.offsets, "FroxelCull")
        frame.write("froxel_indices", self.indices, "FroxelCull")
        frame.write("light_grid", N.froxel_grid_struct(self.indices, self.offsets, self.params,
                                                       self.indices.numel()), "FroxelCull")


class DeferredLightPass:
    """Deferred lighting into ``pre_aa`` (helio-pass-deferred-light)."""

    def __init__(self, target_format: int = N.TARGET_RGBA32F, ambient_color=(0.5, 0.5, 0.6), ambient_intensity=1.0,
                 debug_mode: int = 0, device="cuda"):
        self.target_format = target_format
        self.ambient_color = ambient_color
        self.ambient_intensity = ambient_intensity
        self.debug_mode = debug_mode
        self.device = device
        self.globals_buf = None
        self.pre_aa = None

    def name(self):
        return "DeferredLight"

    def reads(self):
        return ("gbuffer", "depth", "tile_light_lists", "tile_light_counts", "pre_aa")

    def writes(self):
        return ("pre_aa",)

    def on_resize(self, width: int, height: int):
        self.pre_aa = None

    def prepare(self, pc: PassContext):
        torch = _torch()
        tx, _ = L.tile_grid(pc.width, pc.height)
        g = L.make_globals(tx, pc.scene.movable_light_count, self.ambient_color, self.ambient_intensity,
                           self.debug_mode)
        host = torch.from_numpy(np.frombuffer(g.tobytes(), np.uint8).copy())
        if self.globals_buf is None:
            self.globals_buf = torch.empty(L.DEFERRED_GLOBALS.itemsize, dtype=torch.uint8, device=self.device)
        self.globals_buf.copy_(host, non_blocking=False)
        if self.pre_aa is None or self.pre_aa.shape[:2] != (pc.height, pc.width):
            dt = torch.float32 if self.target_format == N.TARGET_RGBA32F else torch.float16
            self.pre_aa = torch.zeros((pc.height, pc.width, 4), dtype=dt, device=self.device)

    def execute(self, pc: PassContext):
        gb = pc.frame.get("gbuffer")
        if gb is None:
            raise InvalidPassConfig("DeferredLightPass: G-buffer not published")
        grid = pc.frame.get("light_grid")
        if grid is None:
            raise InvalidPassConfig("DeferredLightPass: no light grid published")
        pc.ctx.shade(pc.scene.camera, self.globals_buf, gb, pc.scene.lights, pc.scene.movable_light_count, grid,
                     N.target_struct(self.pre_aa, self.target_format), pc.stream)

    def publish(self, frame: FrameResources):
        frame.write("pre_aa", self.pre_aa, "DeferredLight")
