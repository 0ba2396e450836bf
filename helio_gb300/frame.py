"""Device residency of one frame's inputs: camera, globals, lights and G-buffer planes
as torch CUDA tensors, plus the C-ABI structs that point at them."""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import layouts as L
from . import native as N


def _torch():
    import torch

    return torch


def bytes_tensor(arr: np.ndarray, device="cuda", pinned=False):
    """A uint8 tensor holding ``arr``'s bytes (on ``device``, or pinned host)."""
    torch = _torch()
    host = torch.from_numpy(np.frombuffer(np.ascontiguousarray(arr).tobytes(), np.uint8).copy())
    if device == "cpu":
        return host.pin_memory() if pinned else host
    return host.to(device)


def plane_tensor(arr: np.ndarray, device="cuda", pinned=False):
    torch = _torch()
    t = torch.from_numpy(np.ascontiguousarray(arr))
    if device == "cpu":
        return t.pin_memory() if pinned else t
    return t.to(device)


@dataclass
class DeviceFrame:
    width: int
    height: int
    layout: int
    camera: object
    globals_: object
    lights: object
    n_lights: int
    planes: list

    @property
    def gbuffer(self) -> N.GBuffer:
        return N.gbuffer_struct(self.layout, self.width, self.height, self.planes)

    @property
    def gbuffer_bytes(self) -> int:
        return sum(int(p.numel() * p.element_size()) for p in self.planes)


def upload(camera_rec, globals_rec, lights, gbuffer, device="cuda") -> DeviceFrame:
    """Copies one frame's inputs (numpy / synthetic.GBuffer) to the device."""
    return DeviceFrame(
        width=gbuffer.width,
        height=gbuffer.height,
        layout=gbuffer.layout,
        camera=bytes_tensor(camera_rec, device),
        globals_=bytes_tensor(globals_rec, device),
        lights=bytes_tensor(lights, device) if len(lights) else bytes_tensor(np.zeros(1, L.GPU_LIGHT), device),
        n_lights=len(lights),
        planes=[plane_tensor(p, device) for p in gbuffer.planes],
    )


def upload_workload(w, device="cuda") -> DeviceFrame:
    return upload(w.camera.record, w.globals_, w.lights, w.gbuffer, device)


# ----------------------------------------------------------------------------------
# The G-buffer pass's inputs and targets
# ----------------------------------------------------------------------------------


@dataclass
class DeviceMaterialScene:
    """A synthetic.MaterialScene on the device, with the C-ABI texture table."""
    width: int
    height: int
    globals_: object
    surfaces: object
    materials: object
    material_textures: object
    n_materials: int
    textures: list
    texture_table: list
    depth: object

    @property
    def surfaces_pitch(self) -> int:
        return int(self.surfaces.stride(0) * self.surfaces.element_size())

    def write(self, ctx: N.Context, targets: N.GBufferTargets, stream=None):
        """hl_write_gbuffer of this scene into ``targets``."""
        ctx.write_gbuffer(self.globals_, self.surfaces, self.surfaces_pitch, self.materials,
                          self.material_textures, self.n_materials, self.texture_table, targets, stream)


def upload_material_scene(scene, device="cuda") -> DeviceMaterialScene:
    H, W = scene.surfaces.shape
    srf = bytes_tensor(scene.surfaces, device).view(H, W * L.SURFACE.itemsize)
    texs = [plane_tensor(t[0], device) for t in scene.textures]
    table = [N.texture_struct(d, fmt, au, av, flt) for d, (_, fmt, au, av, flt) in zip(texs, scene.textures)]
    return DeviceMaterialScene(W, H, bytes_tensor(scene.globals_, device), srf, bytes_tensor(scene.materials, device),
                               bytes_tensor(scene.material_textures, device), len(scene.materials), texs, table,
                               plane_tensor(scene.depth, device))


GBUFFER_TARGET_SHAPES = (("albedo", 4, "u8"), ("normal", 4, "f16"), ("orm", 4, "u8"), ("emissive", 4, "f16"),
                         ("lightmap_uv", 2, "f16"), ("sss", 4, "f16"), ("extra", 4, "f16"), ("velocity", 2, "f16"))


def gbuffer_targets(width: int, height: int, optional: bool = True, fill: int = 0xAB, device="cuda"):
    """The eight G-buffer targets as device tensors (the optional four None unless
    ``optional``), every byte set to ``fill``; and the hl_gbuffer_targets struct."""
    torch = _torch()
    planes = []
    for i, (_, ch, kind) in enumerate(GBUFFER_TARGET_SHAPES):
        if i >= 4 and not optional:
            planes.append(None)
            continue
        nbytes = ch * (1 if kind == "u8" else 2)
        raw = torch.full((height, width * nbytes), fill, dtype=torch.uint8, device=device)
        planes.append(raw.view(torch.uint8 if kind == "u8" else torch.float16).view(height, width, ch))
    return planes, N.gbuffer_targets_struct(width, height, planes)


def reference_gbuffer(planes, depth) -> N.GBuffer:
    """The HL_GBUF_REFERENCE G-buffer formed by the written albedo, normal, orm and
    emissive targets and the rasteriser's depth."""
    H, W = int(depth.shape[0]), int(depth.shape[1])
    return N.gbuffer_struct(N.GBUF_REFERENCE, W, H, [planes[0], planes[1], planes[2], planes[3], depth])


# ----------------------------------------------------------------------------------
# Frames from host memory, pipelined
# ----------------------------------------------------------------------------------


def _align(n: int, a: int = 256) -> int:
    return (n + a - 1) // a * a


class PackedFrame:
    """One frame's inputs packed in one pinned host buffer (camera, globals, lights,
    then each G-buffer plane at 256-byte offsets), so that its upload is one copy."""

    def __init__(self, camera_rec, globals_rec, lights, gbuffer):
        torch = _torch()
        parts = [np.ascontiguousarray(camera_rec), np.ascontiguousarray(globals_rec),
                 np.ascontiguousarray(lights) if len(lights) else np.zeros(1, L.GPU_LIGHT)]
        parts += [np.ascontiguousarray(p) for p in gbuffer.planes]
        self.offsets, off = [], 0
        for a in parts:
            self.offsets.append(off)
            off = _align(off + a.nbytes)
        self.nbytes = off
        self.host = torch.empty(off, dtype=torch.uint8).pin_memory()
        h = self.host.numpy()
        for a, o in zip(parts, self.offsets):
            h[o:o + a.nbytes] = np.frombuffer(a.tobytes(), np.uint8)
        self.plane_specs = [(p.dtype, p.shape) for p in gbuffer.planes]
        self.width, self.height, self.layout = gbuffer.width, gbuffer.height, gbuffer.layout
        self.n_lights = len(lights)


class HostFramePipeline:
    """Lights frames that live in pinned host memory and returns their radiance to
    pinned host memory: the upload of frame k+1, the binning and shading of frame k and
    the download of frame k-1 run on three CUDA streams with two device buffer sets, so
    copies overlap the kernels. Every frame still makes its own host->device copy of
    all its inputs and its own device->host copy of its radiance (RGBA32F, or RGBA16F
    like the reference's pre_aa target with ``target_format=N.TARGET_RGBA16F``). Sky
    pixels (depth 1) come back as zeros: the device targets are cleared once and shading
    never writes them."""

    def __init__(self, ctx: N.Context, like: PackedFrame, froxel_grid, slice_far, capacity=None, device="cuda",
                 target_format=N.TARGET_RGBA32F):
        torch = _torch()
        self.ctx = ctx
        self.like = like
        self.target_format = target_format
        self.target_dtype = torch.float32 if target_format == N.TARGET_RGBA32F else torch.float16
        W, H = like.width, like.height
        self.fp = N.froxel_params(*froxel_grid, W, H, slice_far)
        F = froxel_grid[0] * froxel_grid[1] * froxel_grid[2]
        self.capacity = capacity if capacity is not None else F * max(1, min(like.n_lights, 256))
        self.slots = []
        for _ in range(2):
            buf = torch.empty(like.nbytes, dtype=torch.uint8, device=device)
            planes = []
            for (dt, shape), o in zip(like.plane_specs, like.offsets[3:]):
                n = int(np.prod(shape)) * np.dtype(dt).itemsize
                t = buf[o:o + n].view(getattr(torch, np.dtype(dt).name)).view(*shape)
                planes.append(t)
            slot = {
                "buf": buf,
                "camera": buf[like.offsets[0]:],
                "globals": buf[like.offsets[1]:],
                "lights": buf[like.offsets[2]:],
                "gbuffer": N.gbuffer_struct(like.layout, W, H, planes),
                "planes": planes,
                "offsets": torch.empty(F + 1, dtype=torch.int32, device=device),
                "indices": torch.empty(self.capacity, dtype=torch.int32, device=device),
                # cleared once: sky pixels (depth 1) are never written, as in the reference
                "target": torch.zeros((H, W, 4), dtype=self.target_dtype, device=device),
                "up": torch.cuda.Event(), "done": torch.cuda.Event(), "down": torch.cuda.Event(),
            }
            slot["grid"] = N.froxel_grid_struct(slot["indices"], slot["offsets"], self.fp, self.capacity)
            slot["tgt"] = N.target_struct(slot["target"], target_format)
            self.slots.append(slot)
        self.s_up, self.s_comp, self.s_down = torch.cuda.Stream(), torch.cuda.Stream(), torch.cuda.Stream()
        self.k = 0

    @property
    def streams(self):
        return self.s_up, self.s_comp, self.s_down

    def submit(self, frame: PackedFrame, host_out):
        """Enqueues one frame; ``host_out`` (pinned, H x W x 4, float32 or float16 as the
        target format) receives its radiance once the download stream has passed this
        frame."""
        torch = _torch()
        s = self.slots[self.k % 2]
        first = self.k < 2
        with torch.cuda.stream(self.s_up):
            if not first:
                self.s_up.wait_event(s["done"])  # kernels of frame k-2 are done with the inputs
            s["buf"].copy_(frame.host, non_blocking=True)
            s["up"].record(self.s_up)
        self.s_comp.wait_event(s["up"])
        if not first:
            self.s_comp.wait_event(s["down"])  # frame k-2's radiance has been read
        sh = self.s_comp.cuda_stream
        n = frame.n_lights
        self.ctx.bin_froxels(s["camera"], s["lights"], n, self.fp, s["offsets"], s["indices"], self.capacity, sh)
        self.ctx.shade(s["camera"], s["globals"], s["gbuffer"], s["lights"], n, s["grid"], s["tgt"], sh)
        s["done"].record(self.s_comp)
        with torch.cuda.stream(self.s_down):
            self.s_down.wait_event(s["done"])
            host_out.copy_(s["target"], non_blocking=True)
            s["down"].record(self.s_down)
        self.k += 1

    def synchronize(self):
        for st in self.streams:
            st.synchronize()
