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
