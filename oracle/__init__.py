"""ctypes wrapper of the CPU oracle (oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA library. Only tests/,
__graft_entry__.smoke() and bench.py's cpu_baseline / reference legs import this
package. Parity against the reference's own execution is UNPINNED (see the header of
oracle.cpp); the restatement is pinned by layout constants, known-answer cases and the
golden vectors under tests/golden/.

Build recipe: ``python -m oracle.build`` or ``oracle.build()``; compiles oracle.cpp with
g++ (-O3 -ffp-contract=off -fopenmp) into oracle/_build/liboracle.so.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD_DIR = HERE / "_build"
LIB_PATH = BUILD_DIR / "liboracle.so"
SOURCES = [HERE / "oracle.cpp", HERE / "gbuffer_write.cpp", HERE / "shadow_factor.h", HERE / "rc_gi.h"]

_lock = threading.Lock()
_lib = None


def build(force: bool = False) -> Path:
    """Compile the oracle if it is missing or older than its source."""
    BUILD_DIR.mkdir(exist_ok=True)
    newest = max(p.stat().st_mtime for p in SOURCES)
    if not force and LIB_PATH.exists() and LIB_PATH.stat().st_mtime >= newest:
        return LIB_PATH
    tmp = LIB_PATH.with_suffix(f".{os.getpid()}.tmp")
    cmd = [
        "g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
        "-ffp-contract=off", "-fno-fast-math", "-fno-strict-aliasing",
        *[str(p) for p in SOURCES if p.suffix == ".cpp"], "-o", str(tmp),
    ]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def lib():
    global _lib
    with _lock:
        if _lib is None:
            build()
            _lib = _bind(C.CDLL(str(LIB_PATH)))
    return _lib


def _bind(l):
    vp, u32, u64p, u32p, f32p, f64p = C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p
    l.oracle_bin_tiles_ref_f32.argtypes = [vp, vp, u32, u32, u32, u32p, u32p]
    l.oracle_bin_tiles_ref_f64.argtypes = [vp, vp, u32, u32, u32, u32p, u32p]
    l.oracle_froxel_slice_table.argtypes = [vp, f32p]
    l.oracle_bin_froxels_f32.argtypes = [vp, vp, u32, vp, u32p, u32p, u32]
    shade_args = [vp, vp, u32, u32, u32, vp, u64p, vp, u32, u32, u32p, u32p, vp, f64p, u32p, u32, u32]
    l.oracle_shade_f64.argtypes = shade_args
    l.oracle_shade_f32.argtypes = shade_args
    l.oracle_shade_ex_f64.argtypes = [vp, vp, u32, u32, u32, vp, u64p, vp, u32, u32, u32p, u32p, vp, vp, vp, f64p,
                                      u32p, u32, u32, vp]
    l.oracle_shade_forced_f64.argtypes = [vp, vp, u32, u32, u32, vp, u64p, vp, u32, u32, u32p, u32p, vp, vp, u32p,
                                          u32p, f64p, u32p, u32, u32, vp]
    l.oracle_reflections_f64.argtypes = [vp, vp, u32, u32, u32, vp, u64p, vp, C.c_uint64, vp, C.c_uint64, vp,
                                         C.c_uint64, vp, vp, f64p, vp]
    l.oracle_shade_adjoint_f64.argtypes = [vp, vp, u32, u32, u32, vp, u64p, vp, u32, u32, u32p, u32p, vp, f64p, f64p, f64p]
    frag_args = [vp, vp, vp, u32, vp, u32, u32p, vp, u32, u32, u32p, u32p, vp, f64p]
    l.oracle_shade_fragments_f64.argtypes = frag_args
    l.oracle_shade_fragments_f32.argtypes = frag_args
    l.oracle_light_dir_from_rotation.argtypes = [f32p, f64p]
    l.oracle_write_gbuffer.argtypes = [vp, vp, C.c_uint64, vp, vp, u32, vp, u32, u32, u32, f64p, vp, vp]
    l.oracle_set_threads.argtypes = [C.c_int]
    l.oracle_num_threads.restype = C.c_int
    return l


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def set_threads(n: int) -> None:
    lib().oracle_set_threads(int(n))


def num_threads() -> int:
    return int(lib().oracle_num_threads())


# ----------------------------------------------------------------------------------
# Binning
# ----------------------------------------------------------------------------------


def bin_tiles_ref(camera_rec, lights, width, height, precision="f32"):
    """Reference tile lists (light_cull.wgsl:123-180): (lists[tiles,64], counts[tiles])."""
    tx, ty = (width + 15) // 16, (height + 15) // 16
    lists = np.zeros((tx * ty, 64), np.uint32)
    counts = np.zeros(tx * ty, np.uint32)
    cam = np.ascontiguousarray(camera_rec)
    lts = np.ascontiguousarray(lights)
    fn = lib().oracle_bin_tiles_ref_f32 if precision == "f32" else lib().oracle_bin_tiles_ref_f64
    fn(_ptr(cam), _ptr(lts) if len(lts) else None, len(lts), width, height, _ptr(lists), _ptr(counts))
    return lists, counts


def froxel_slice_table(params) -> np.ndarray:
    p = np.ascontiguousarray(params)
    out = np.zeros(int(p["grid_z"][0]) + 1, np.float32)
    lib().oracle_froxel_slice_table(_ptr(p), _ptr(out))
    return out


def bin_froxels(camera_rec, lights, params, capacity=None):
    """Froxel lists in the documented f32 order: (offsets[F+1], indices[total])."""
    p = np.ascontiguousarray(params)
    F = int(p["grid_x"][0] * p["grid_y"][0] * p["grid_z"][0])
    n = len(lights)
    cap = capacity if capacity is not None else max(1, F * max(n, 1))
    cap = min(cap, 1 << 28)
    offsets = np.zeros(F + 1, np.uint32)
    indices = np.zeros(cap, np.uint32)
    lts = np.ascontiguousarray(lights)
    lib().oracle_bin_froxels_f32(_ptr(np.ascontiguousarray(camera_rec)), _ptr(lts) if n else None, n, _ptr(p),
                                 _ptr(offsets), _ptr(indices), cap)
    total = int(offsets[F])
    return offsets, indices[: min(total, cap)].copy()


# ----------------------------------------------------------------------------------
# Shading
# ----------------------------------------------------------------------------------


def _planes(gb):
    arrs = [np.ascontiguousarray(p) for p in gb.planes]
    ptrs = (C.c_void_p * 6)(*([a.ctypes.data for a in arrs] + [None] * (6 - len(arrs))))
    pitch = (C.c_uint64 * 6)(*([a.strides[0] for a in arrs] + [0] * (6 - len(arrs))))
    return arrs, ptrs, pitch


def _grid_args(grid):
    """grid: ('tiles', lists, counts) or ('froxels', indices, offsets, params)."""
    kind = grid[0]
    if kind == "tiles":
        lists = np.ascontiguousarray(grid[1], np.uint32)
        counts = np.ascontiguousarray(grid[2], np.uint32)
        return 0, lists, counts, None
    lists = np.ascontiguousarray(grid[1], np.uint32)
    if lists.size == 0:
        lists = np.zeros(1, np.uint32)
    offsets = np.ascontiguousarray(grid[2], np.uint32)
    params = np.ascontiguousarray(grid[3])
    return 1, lists, offsets, params


def shade(camera_rec, globals_rec, gb, lights, grid, precision="f64", rows=None, pair_counts=False):
    """Radiance (H, W, 4) float64 of fs_main's direct + ambient + emissive terms.
    Sky pixels (depth >= 1) are NaN. Optionally per-pixel (listed, in_range, full)."""
    W, H = gb.width, gb.height
    r0, r1 = (0, H) if rows is None else rows
    out = np.full((H, W, 4), np.nan, np.float64)
    pc = np.zeros((H, W, 3), np.uint32) if pair_counts else None
    arrs, ptrs, pitch = _planes(gb)
    kind, lists, counts, params = _grid_args(grid)
    lts = np.ascontiguousarray(lights)
    fn = lib().oracle_shade_f64 if precision == "f64" else lib().oracle_shade_f32
    fn(_ptr(np.ascontiguousarray(camera_rec)), _ptr(np.ascontiguousarray(globals_rec)), gb.layout, W, H, ptrs, pitch,
       _ptr(lts) if len(lts) else None, len(lts), kind, _ptr(lists), _ptr(counts),
       _ptr(params) if params is not None else None, _ptr(out), _ptr(pc) if pc is not None else None, r0, r1)
    return (out, pc) if pair_counts else out


def shade_shadowed(camera_rec, globals_rec, gb, lights, grid, shadows, rows=None, pair_counts=False):
    """``shade`` (f64) with the shadow term. ``shadows``: dict with numpy arrays
    ``dynamic`` and ``static`` (layers, size, size) float32, ``matrices`` (layers, 16)
    float32 column-major, ``config`` (a SHADOW_CONFIG record) and ``max_lights``.
    Returns (radiance, pair_counts or None, bounds_flag)."""
    return shade_ex(camera_rec, globals_rec, gb, lights, grid, shadows=shadows, rows=rows, pair_counts=pair_counts)


def shade_ex(camera_rec, globals_rec, gb, lights, grid, shadows=None, rc=None, rows=None, pair_counts=False):
    """``shade`` (f64) with the pass's optional bindings: ``shadows`` as for
    ``shade_shadowed`` (or None) and ``rc``, the radiance-cascade probe texture as a
    (height, width, 4) float16 array (or None). Returns (radiance, pair_counts or None,
    bounds_flag)."""
    from helio_gb300 import layouts as L

    W, H = gb.width, gb.height
    r0, r1 = (0, H) if rows is None else rows
    out = np.full((H, W, 4), np.nan, np.float64)
    pc = np.zeros((H, W, 3), np.uint32) if pair_counts else None
    arrs, ptrs, pitch = _planes(gb)
    kind, lists, counts, params = _grid_args(grid)
    lts = np.ascontiguousarray(lights)
    desc = None
    if shadows is not None:
        dyn = np.ascontiguousarray(shadows["dynamic"], np.float32)
        sta = np.ascontiguousarray(shadows["static"], np.float32)
        mats = np.ascontiguousarray(shadows["matrices"], np.float32)
        cfg = np.ascontiguousarray(shadows["config"])
        desc = np.zeros(1, L.SHADOW_MAPS)
        desc["dynamic_atlas"], desc["static_atlas"] = dyn.ctypes.data, sta.ctypes.data
        desc["matrices"], desc["config"] = mats.ctypes.data, cfg.ctypes.data
        desc["size"], desc["layers"] = dyn.shape[1], dyn.shape[0]
        desc["max_shadow_lights"] = shadows["max_lights"]
    rcd = None
    if rc is not None:
        rct = np.ascontiguousarray(rc, np.float16)
        rcd = np.zeros(1, L.RC_CASCADE)
        rcd["texels"], rcd["pitch"] = rct.ctypes.data, rct.strides[0]
        rcd["height"], rcd["width"] = rct.shape[0], rct.shape[1]
    bounds = np.zeros(1, np.int32)
    lib().oracle_shade_ex_f64(_ptr(np.ascontiguousarray(camera_rec)), _ptr(np.ascontiguousarray(globals_rec)),
                              gb.layout, W, H, ptrs, pitch, _ptr(lts) if len(lts) else None, len(lts), kind,
                              _ptr(lists), _ptr(counts), _ptr(params) if params is not None else None,
                              _ptr(desc) if desc is not None else None, _ptr(rcd) if rcd is not None else None,
                              _ptr(out), _ptr(pc) if pc is not None else None, r0, r1, _ptr(bounds))
    return out, pc, bool(bounds[0])


def forced_csr(pairs, n_pixels):
    """(offsets[n_pixels+1], lights) of (pixel, light) pairs, each pixel's lights
    ascending and without duplicates."""
    pr = np.asarray(pairs, np.uint64).reshape(-1, 2)
    key = np.unique((pr[:, 0] << np.uint64(32)) | pr[:, 1])
    pix = (key >> np.uint64(32)).astype(np.int64)
    if pix.size and pix.max() >= n_pixels:
        raise ValueError("pair pixel index beyond the image")
    offsets = np.zeros(n_pixels + 1, np.uint32)
    np.cumsum(np.bincount(pix, minlength=n_pixels), out=offsets[1:])
    return offsets, (key & np.uint64(0xFFFFFFFF)).astype(np.uint32)


def _shadow_desc(shadows):
    from helio_gb300 import layouts as L

    dyn = np.ascontiguousarray(shadows["dynamic"], np.float32)
    sta = np.ascontiguousarray(shadows["static"], np.float32)
    mats = np.ascontiguousarray(shadows["matrices"], np.float32)
    cfg = np.ascontiguousarray(shadows["config"])
    desc = np.zeros(1, L.SHADOW_MAPS)
    desc["dynamic_atlas"], desc["static_atlas"] = dyn.ctypes.data, sta.ctypes.data
    desc["matrices"], desc["config"] = mats.ctypes.data, cfg.ctypes.data
    desc["size"], desc["layers"] = dyn.shape[1], dyn.shape[0]
    desc["max_shadow_lights"] = shadows["max_lights"]
    return desc, (dyn, sta, mats, cfg)


def shade_forced(camera_rec, globals_rec, gb, lights, grid, lit_pairs, shadows=None, rows=None):
    """``shade`` (f64) with another evaluation's branch decisions: ``lit_pairs`` (K, 2)
    are the (y * W + x, light) pairs that evaluation lit (as hl_set_pair_log records
    them), or their forced_csr. Those pairs are evaluated as lit whatever the f64 cuts decide, every other
    listed pair contributes nothing, so the radiance is comparable at every pixel,
    including those where f32 and f64 fall on different sides of a cut. Returns
    (radiance, flips, unlisted): per pixel the number of listed pairs whose f64 decision
    differs, and of lit pairs whose light is not in the pixel's list (must be 0)."""
    W, H = gb.width, gb.height
    r0, r1 = (0, H) if rows is None else rows
    out = np.full((H, W, 4), np.nan, np.float64)
    fl = np.zeros((H, W), np.uint32)
    arrs, ptrs, pitch = _planes(gb)
    kind, lists, counts, params = _grid_args(grid)
    lts = np.ascontiguousarray(lights)
    off, fls = lit_pairs if isinstance(lit_pairs, tuple) else forced_csr(lit_pairs, W * H)
    if fls.size == 0:
        fls = np.zeros(1, np.uint32)
    desc, keep = _shadow_desc(shadows) if shadows is not None else (None, None)
    bounds = np.zeros(1, np.int32)
    lib().oracle_shade_forced_f64(_ptr(np.ascontiguousarray(camera_rec)), _ptr(np.ascontiguousarray(globals_rec)),
                                  gb.layout, W, H, ptrs, pitch, _ptr(lts) if len(lts) else None, len(lts), kind,
                                  _ptr(lists), _ptr(counts), _ptr(params) if params is not None else None,
                                  _ptr(desc) if desc is not None else None, _ptr(off), _ptr(fls), _ptr(out), _ptr(fl),
                                  r0, r1, _ptr(bounds))
    return out, (fl & 0xFFFF).astype(np.uint32), (fl >> 16).astype(np.uint32)


def _rc_desc(rc):
    """(descriptor record, texel array) of an RC probe texture, or (None, None)."""
    from helio_gb300 import layouts as L

    if rc is None:
        return None, None
    rct = np.ascontiguousarray(rc, np.float16)
    rcd = np.zeros(1, L.RC_CASCADE)
    rcd["texels"], rcd["pitch"] = rct.ctypes.data, rct.strides[0]
    rcd["height"], rcd["width"] = rct.shape[0], rct.shape[1]
    return rcd, rct


def reflections(camera_rec, globals_rec, gb, base, ssr=None, planar=None, lightmap_uv=None, rc=None, env=None):
    """fs_reflection (f64) blended over ``base`` (H, W, 4), the lit target: returns
    (result (H, W, 4) float64, unsupported flag). ``ssr`` / ``planar``: (H, W, 4) float16
    hit images, ``lightmap_uv``: (H, W, 2) float16, ``rc``: the probe texture, ``env``:
    dict(captures=REFLECTION_CAPTURE array, texels=float16 cube array, face_size,
    mip_levels, layers); each None for the pass's fallback."""
    W, H = gb.width, gb.height
    out = np.array(base, np.float64, copy=True, order="C")
    assert out.shape == (H, W, 4)
    arrs, ptrs, pitch = _planes(gb)
    imgs = []
    for a, ch in ((ssr, 4), (planar, 4), (lightmap_uv, 2)):
        if a is None:
            imgs += [None, 0]
            continue
        a = np.ascontiguousarray(a, np.float16)
        assert a.shape == (H, W, ch)
        arrs.append(a)
        imgs += [_ptr(a), a.strides[0]]
    rcd, rct = _rc_desc(rc)
    envd = None
    if env is not None:
        from helio_gb300 import layouts as L

        caps = np.ascontiguousarray(env["captures"])
        tex = np.ascontiguousarray(env["texels"], np.float16)
        envd = np.zeros(1, L.REFLECTION_ENV)
        envd["captures"], envd["count"], envd["texels"] = caps.ctypes.data, len(caps), tex.ctypes.data
        envd["face_size"], envd["mip_levels"], envd["layers"] = env["face_size"], env["mip_levels"], env["layers"]
        arrs += [caps, tex]
    flag = np.zeros(1, np.int32)
    lib().oracle_reflections_f64(_ptr(np.ascontiguousarray(camera_rec)), _ptr(np.ascontiguousarray(globals_rec)),
                                 gb.layout, W, H, ptrs, pitch, *imgs, _ptr(rcd) if rcd is not None else None,
                                 _ptr(envd) if envd is not None else None, _ptr(out), _ptr(flag))
    return out, bool(flag[0])


def shade_fragments(camera_rec, params, fragments, lights, grid, entity_indices=None, transforms=None,
                    precision="f64"):
    """Lit fragments (n, 4) float64 of the Forward+ (params mode 0) or transparent (mode 1)
    light loop; discarded fragments (forward, alpha <= 0.001) are NaN. ``params``: one
    FRAGMENT_PARAMS record; ``transforms``: TRANSFORM records indexed by
    ``entity_indices`` (forward mode)."""
    fr = np.ascontiguousarray(fragments)
    out = np.full((len(fr), 4), np.nan, np.float64)
    kind, lists, counts, fparams = _grid_args(grid)
    lts = np.ascontiguousarray(lights)
    ent = np.ascontiguousarray(entity_indices, np.uint32) if entity_indices is not None else None
    xf = np.ascontiguousarray(transforms) if transforms is not None else None
    fn = lib().oracle_shade_fragments_f64 if precision == "f64" else lib().oracle_shade_fragments_f32
    fn(_ptr(np.ascontiguousarray(camera_rec)), _ptr(np.ascontiguousarray(params)), _ptr(fr) if len(fr) else None,
       len(fr), _ptr(lts) if len(lts) else None, len(lts), _ptr(ent) if ent is not None else None,
       _ptr(xf) if xf is not None and len(xf) else None, len(xf) if xf is not None else 0, kind, _ptr(lists),
       _ptr(counts), _ptr(fparams) if fparams is not None else None, _ptr(out))
    return out


def light_dir_from_rotation(rotation_deg):
    """Unit direction of a Transform rotation (degrees: pitch x, yaw y, roll z)."""
    r = np.ascontiguousarray(rotation_deg, np.float32)
    out = np.zeros(3, np.float64)
    lib().oracle_light_dir_from_rotation(_ptr(r), _ptr(out))
    return out


def shade_adjoint(camera_rec, globals_rec, gb, lights, grid, weights):
    """FP64 gradient of sum(weights * radiance) (branch decisions fixed):
    (d_lights[n,7], d_pixels[H,W,5])."""
    W, H = gb.width, gb.height
    arrs, ptrs, pitch = _planes(gb)
    kind, lists, counts, params = _grid_args(grid)
    lts = np.ascontiguousarray(lights)
    w = np.ascontiguousarray(weights, np.float64).reshape(H, W, 4)
    dl = np.zeros((len(lts), 7), np.float64)
    dp = np.zeros((H, W, 5), np.float64)
    lib().oracle_shade_adjoint_f64(_ptr(np.ascontiguousarray(camera_rec)), _ptr(np.ascontiguousarray(globals_rec)),
                                   gb.layout, W, H, ptrs, pitch, _ptr(lts) if len(lts) else None, len(lts), kind,
                                   _ptr(lists), _ptr(counts), _ptr(params) if params is not None else None, _ptr(w),
                                   _ptr(dl), _ptr(dp))
    return dl, dp


# ----------------------------------------------------------------------------------
# G-buffer write (gbuffer.wgsl fs_main, default PBR template)
# ----------------------------------------------------------------------------------


def write_gbuffer(globals_rec, surfaces, materials, material_textures, textures):
    """f64 G-buffer values before quantisation, per pixel: (values[H,W,20], written[H,W],
    bounds). values: albedo 0-3, normal 4-7, orm 8-11, emissive 12-15, lightmap_uv
    16-17, velocity 18-19. ``surfaces``: (H, W) array of SURFACE records;
    ``textures``: list of (texels ndarray [h, w, 4], format, address_u, address_v,
    filter)."""
    from helio_gb300 import layouts as L

    srf = np.ascontiguousarray(surfaces)
    H, W = srf.shape
    keep = [np.ascontiguousarray(t[0]) for t in textures]
    desc = np.zeros(max(1, len(textures)), L.TEXTURE)
    for i, (t, (_, fmt, au, av, flt)) in enumerate(zip(keep, textures)):
        desc[i] = (t.ctypes.data, t.strides[0], t.shape[1], t.shape[0], fmt, au, av, flt)
    mats = np.ascontiguousarray(materials)
    mtex = np.ascontiguousarray(material_textures)
    out = np.zeros((H, W, 20), np.float64)
    written = np.zeros((H, W), np.uint8)
    bounds = np.zeros(1, np.int32)
    lib().oracle_write_gbuffer(_ptr(np.ascontiguousarray(globals_rec)), _ptr(srf), srf.strides[0],
                               _ptr(mats) if len(mats) else None, _ptr(mtex) if len(mtex) else None, len(mats),
                               _ptr(desc), len(textures), W, H, _ptr(out), _ptr(written), _ptr(bounds))
    return out, written.astype(bool), bool(bounds[0])
