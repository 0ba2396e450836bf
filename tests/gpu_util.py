"""Helpers of the GPU parity tests: run the library through the C ABI on torch
device buffers and bring results back as numpy arrays."""
from __future__ import annotations

import numpy as np

from helio_gb300 import frame as FR
from helio_gb300 import layouts as L
from helio_gb300 import native as N


def torch():
    import torch as t

    return t


def gpu_bin_tiles(ctx, camera_rec, lights, width, height):
    T = torch()
    tx, ty = L.tile_grid(width, height)
    tiles = tx * ty
    cam = FR.bytes_tensor(camera_rec)
    lt = FR.bytes_tensor(lights) if len(lights) else FR.bytes_tensor(np.zeros(1, L.GPU_LIGHT))
    lists = T.full((tiles * 64,), -1, dtype=T.int32, device="cuda")
    counts = T.full((tiles,), -1, dtype=T.int32, device="cuda")
    ctx.bin_tiles_ref(cam, lt, len(lights), width, height, lists, counts)
    ctx.sync_status()
    return (lists.cpu().numpy().view(np.uint32).reshape(tiles, 64), counts.cpu().numpy().view(np.uint32))


def assert_tile_lists_equal(got, want):
    gl, gc = got
    wl, wc = want
    np.testing.assert_array_equal(gc, wc)
    for t in np.nonzero(wc)[0]:
        c = int(wc[t])
        if not np.array_equal(gl[t, :c], wl[t, :c]):
            raise AssertionError(f"tile {t}: got {gl[t, :c].tolist()} want {wl[t, :c].tolist()}")


def gpu_bin_froxels(ctx, camera_rec, lights, params_np, capacity=None, expect_status=N.HL_OK):
    T = torch()
    p = N.froxel_params_from_numpy(params_np)
    F = p.grid_x * p.grid_y * p.grid_z
    cap = capacity if capacity is not None else max(64, F * max(1, min(len(lights), 256)))
    cam = FR.bytes_tensor(camera_rec)
    lt = FR.bytes_tensor(lights) if len(lights) else FR.bytes_tensor(np.zeros(1, L.GPU_LIGHT))
    offsets = T.full((F + 1,), -1, dtype=T.int32, device="cuda")
    indices = T.full((max(cap, 1),), -1, dtype=T.int32, device="cuda")
    ctx.bin_froxels(cam, lt, len(lights), p, offsets, indices, cap)
    status = N.HL_OK
    try:
        ctx.sync_status()
    except N.HelioError as e:
        status = e.status
    assert status == expect_status, f"status {status}, expected {expect_status}"
    off = offsets.cpu().numpy().view(np.uint32)
    total = int(off[-1])
    idx = indices.cpu().numpy().view(np.uint32)[: min(total, cap)]
    return off, idx, (cam, lt, offsets, indices, p, cap)


def gpu_shade(ctx, df: FR.DeviceFrame, grid: N.LightGrid, target_format=N.TARGET_RGBA32F, fill=7.0, stats=False):
    """Runs hl_shade (or hl_shade_stats) and returns the (H, W, 4) image as float64
    (or (H, W, 3) uint32 counts)."""
    T = torch()
    if stats:
        counts = T.full((df.height, df.width, 3), -1, dtype=T.int32, device="cuda")
        ctx.shade_stats(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, counts)
        ctx.sync_status()
        return counts.cpu().numpy().view(np.uint32)
    dt = T.float32 if target_format == N.TARGET_RGBA32F else T.float16
    out = T.full((df.height, df.width, 4), fill, dtype=dt, device="cuda")
    ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, N.target_struct(out, target_format))
    ctx.sync_status()
    return out.float().cpu().numpy().astype(np.float64)


def gpu_shade_logged(ctx, df: FR.DeviceFrame, grid: N.LightGrid, target_format=N.TARGET_RGBA32F, fill=7.0,
                     capacity=None):
    """hl_shade with the lit-pair record on (hl_set_pair_log): returns the image as
    gpu_shade does and the (K, 2) uint32 (y * W + x, light) pairs the kernel lit."""
    T = torch()
    cap = capacity if capacity is not None else max(1 << 16, df.width * df.height * 4)
    while True:
        pairs = T.zeros((cap, 2), dtype=T.int32, device="cuda")
        count = T.zeros((1,), dtype=T.int32, device="cuda")
        ctx.set_pair_log(pairs, count)
        try:
            img = gpu_shade(ctx, df, grid, target_format=target_format, fill=fill)
        finally:
            ctx.set_pair_log(None)
        n = int(count.item())
        if n <= cap:
            return img, pairs[:n].cpu().numpy().view(np.uint32)
        cap = n  # the count covers every lit pair: one more launch records them all
        del pairs
