"""torch.autograd bridge over the C ABI: the direct-lighting radiance as a
differentiable function of the lights and of the per-pixel material.

Forward = hl_bin_froxels + hl_shade on an HL_GBUF_F32 G-buffer; backward =
hl_shade_adjoint (hand-written adjoint kernel, f64 cross-block light reduction). The
froxel lists are rebuilt from the light positions on every forward; the backward holds
them, and every branch of pbr_direct_light (deferred_lighting.wgsl:699-820), fixed.

Parameters:
  light_params [n, 7] float32: position xyz, intensity, colour rgb (the GpuLight fields
      position_range.xyz, color_intensity.w, color_intensity.rgb);
  pixel_params [H, W, 5] float32: albedo rgb, roughness, metallic (the F32 G-buffer's
      plane 0 rgb/a and plane 1 w).
Everything else (camera, globals, normals, depth, the other light fields) is fixed
scene data held by ShadeScene.
"""
from __future__ import annotations

import torch

from . import layouts as L
from . import native as N

# float32 column of each light parameter inside the 128-byte GpuLight record
LIGHT_PARAM_COLUMNS = (0, 1, 2, 11, 8, 9, 10)


class ShadeScene:
    """Fixed inputs of a differentiable shading call, all on one CUDA device.

    camera, globals_: uint8 tensors holding GpuCameraUniforms / DeferredGlobals;
    lights: uint8 tensor of n GpuLight records (the template the parameters are
    written into); normal [H, W, 3] and depth [H, W] float32; froxel: FroxelParams."""

    def __init__(self, ctx: N.Context, camera, globals_, lights, normal, depth, froxel: N.FroxelParams,
                 capacity: int | None = None):
        self.ctx = ctx
        self.camera = camera
        self.globals_ = globals_
        self.n_lights = lights.numel() // L.GPU_LIGHT.itemsize
        self.lights = lights.view(torch.float32).reshape(self.n_lights, L.GPU_LIGHT.itemsize // 4)
        self.normal = normal
        self.depth = depth
        self.froxel = froxel
        self.height, self.width = depth.shape
        n_froxels = froxel.grid_x * froxel.grid_y * froxel.grid_z
        self.capacity = capacity if capacity is not None else max(1, n_froxels * max(self.n_lights, 1))
        if froxel.width != self.width or froxel.height != self.height:
            raise ValueError("froxel grid and G-buffer sizes differ")

    def light_records(self, light_params: torch.Tensor) -> torch.Tensor:
        rec = self.lights.clone()
        rec[:, list(LIGHT_PARAM_COLUMNS)] = light_params.to(torch.float32)
        return rec

    def planes(self, pixel_params: torch.Tensor):
        p = pixel_params.to(torch.float32)
        plane0 = torch.cat([p[..., 0:3], p[..., 3:4]], -1).contiguous()
        plane1 = torch.cat([self.normal, p[..., 4:5]], -1).contiguous()
        return plane0, plane1, self.depth.contiguous()

    def bin(self, rec: torch.Tensor):
        dev = rec.device
        n_froxels = self.froxel.grid_x * self.froxel.grid_y * self.froxel.grid_z
        offsets = torch.empty(n_froxels + 1, dtype=torch.int32, device=dev)
        indices = torch.empty(self.capacity, dtype=torch.int32, device=dev)
        self.ctx.bin_froxels(self.camera, rec, self.n_lights, self.froxel, offsets, indices, self.capacity)
        return offsets, indices


class DeferredShade(torch.autograd.Function):
    """radiance [H, W, 4] = shade(light_params, pixel_params; scene)."""

    @staticmethod
    def forward(fctx, light_params, pixel_params, scene: ShadeScene):
        rec = scene.light_records(light_params)
        planes = scene.planes(pixel_params)
        offsets, indices = scene.bin(rec)
        gb = N.gbuffer_struct(N.GBUF_F32, scene.width, scene.height, planes)
        grid = N.froxel_grid_struct(indices, offsets, scene.froxel, scene.capacity)
        rad = torch.zeros(scene.height, scene.width, 4, dtype=torch.float32, device=rec.device)
        scene.ctx.shade(scene.camera, scene.globals_, gb, rec, scene.n_lights, grid, N.target_struct(rad))
        fctx.scene = scene
        fctx.save_for_backward(rec, *planes, offsets, indices)
        fctx.param_dtypes = (light_params.dtype, pixel_params.dtype)
        return rad

    @staticmethod
    def backward(fctx, grad_radiance):
        scene: ShadeScene = fctx.scene
        rec, p0, p1, p2, offsets, indices = fctx.saved_tensors
        g = grad_radiance.to(torch.float32).contiguous()
        gb = N.gbuffer_struct(N.GBUF_F32, scene.width, scene.height, (p0, p1, p2))
        grid = N.froxel_grid_struct(indices, offsets, scene.froxel, scene.capacity)
        d_lights = torch.empty(max(scene.n_lights, 1), 7, dtype=torch.float64, device=rec.device)
        d_pixels = torch.empty(scene.height, scene.width, 5, dtype=torch.float32, device=rec.device)
        scene.ctx.shade_adjoint(scene.camera, scene.globals_, gb, rec, scene.n_lights, grid, g,
                                g.stride(0) * g.element_size(), d_lights, d_pixels)
        ldt, pdt = fctx.param_dtypes
        return d_lights[: scene.n_lights].to(ldt), d_pixels.to(pdt), None


def shade(light_params: torch.Tensor, pixel_params: torch.Tensor, scene: ShadeScene) -> torch.Tensor:
    return DeferredShade.apply(light_params, pixel_params, scene)


def light_params_of(lights_np) -> torch.Tensor:
    """[n, 7] float32 parameters of a numpy GPU_LIGHT array (CPU tensor)."""
    f = lights_np.view(L.GPU_LIGHT).view("<f4").reshape(len(lights_np), -1)
    return torch.from_numpy(f[:, list(LIGHT_PARAM_COLUMNS)].copy())
