"""A few frames of one workload through the C ABI, for profiler captures.

    python profile_run.py --workload 1 --frames 3            # bin + shade
    python profile_run.py --workload 4 --frames 3 --adjoint  # + adjoint
    python profile_run.py --batched --frames 3              # 98-view plan
    python profile_run.py --workload 1 --frames 3 --fragments  # + fragment loop
    python profile_run.py --gbuffer-write --frames 3        # G-buffer pass only
    python profile_run.py --workload 1 --shadows --atlas 256 --frames 3  # + shadow term
    python profile_run.py --workload 1 --rc --frames 3      # + radiance-cascade GI

Every frame launches the same kernels as one bench step (froxel binning: 1 launch,
candidate light table: 1, shading: 1, adjoint: 2), so ``ncu -k <kernel> -s <n> -c 1``
can pick one warm launch.
Prints one line with the device time of the last frame.
"""
from __future__ import annotations

import argparse


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", type=int, default=1, choices=[0, 1, 2, 4])
    ap.add_argument("--frames", type=int, default=3)
    ap.add_argument("--adjoint", action="store_true")
    ap.add_argument("--batched", action="store_true")
    ap.add_argument("--fragments", action="store_true",
                    help="also light one raster-ordered fragment per pixel (transparent mode)")
    ap.add_argument("--gbuffer-write", action="store_true",
                    help="only the G-buffer pass: hl_write_gbuffer over the bench's 1080p material scene")
    ap.add_argument("--shadows", action="store_true",
                    help="shade with the shadow term: lights 0-41 cast shadows (hl_shade_ex)")
    ap.add_argument("--atlas", type=int, default=1024, help="shadow atlas size in texels")
    ap.add_argument("--rc", action="store_true", help="shade with radiance-cascade GI (hl_shade_ex)")
    ap.add_argument("--reflections", action="store_true",
                    help="the reflection draw (hl_shade_reflections) over a reference-layout G-buffer")
    ap.add_argument("--scale", type=float, default=1.0)
    args = ap.parse_args(argv)

    import torch

    from helio_gb300 import frame as FR
    from helio_gb300 import layouts as L
    from helio_gb300 import native as N
    from helio_gb300 import synthetic as S

    ctx = N.Context(0)
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if args.gbuffer_write:
        cam = S.default_camera(max(16, int(1920 * args.scale)), max(16, int(1080 * args.scale)))
        ds = FR.upload_material_scene(S.material_scene(cam, 1001))
        _, tg = FR.gbuffer_targets(cam.width, cam.height, optional=True, fill=0)
        for _ in range(args.frames):
            ev0.record()
            ds.write(ctx, tg)
            ev1.record()
        ctx.sync_status()
        print(f"G-buffer write {cam.width}x{cam.height}: {ev0.elapsed_time(ev1) * 1e3:.1f} us per frame", flush=True)
        return
    if args.reflections:
        cam = S.default_camera(max(16, int(1920 * args.scale)), max(16, int(1080 * args.scale)))
        gb = S.make_gbuffer(cam, S.LAYOUT_REFERENCE, seed=23)
        glb = L.make_globals(L.tile_grid(cam.width, cam.height)[0], 0)
        df = FR.upload(cam.record, glb, [], gb)
        imgs = [torch.from_numpy(a).cuda() for a in S.reflection_images(cam.width, cam.height, 77)]
        out = torch.ones((cam.height, cam.width, 4), dtype=torch.float32, device="cuda")
        for _ in range(args.frames):
            ev0.record()
            ctx.shade_reflections(df.camera, df.globals_, df.gbuffer, N.target_struct(out), ssr=imgs[0],
                                  planar=imgs[1], lightmap_uv=imgs[2])
            ev1.record()
        ctx.sync_status()
        print(f"reflections {cam.width}x{cam.height}: {ev0.elapsed_time(ev1) * 1e3:.1f} us per frame", flush=True)
        return
    if args.batched:
        views, lights = S.batched_views(args.scale)
        glb = L.make_globals(1, len(lights), ambient_color=(0.4, 0.45, 0.5), ambient_intensity=0.3)
        d_l, d_g = FR.bytes_tensor(lights), FR.bytes_tensor(glb)
        frames = [FR.upload(v.camera.record, glb, lights, v.gbuffer) for v in views]
        outs = [torch.zeros((f.height, f.width, 4), dtype=torch.float32, device="cuda") for f in frames]
        vs = [N.view_struct(f.camera, f.gbuffer, N.target_struct(o)) for f, o in zip(frames, outs)]
        plan = ctx.batch_plan(vs, d_l, len(lights), d_g, grid=(8, 8, 24))
        for _ in range(args.frames):
            ev0.record()
            plan.execute()
            ev1.record()
        ctx.sync_status()
        plan.close()
        print(f"batched: {len(views)} views, {ev0.elapsed_time(ev1) * 1e3:.1f} us per frame", flush=True)
        return
    w = S.workload(args.workload, args.scale)
    W, H = w.gbuffer.width, w.gbuffer.height
    fp = N.froxel_params_from_numpy(L.froxel_params(*w.froxel_grid, W, H, w.camera.far))
    F = fp.grid_x * fp.grid_y * fp.grid_z
    df = FR.upload_workload(w)
    cap = F * max(1, min(df.n_lights, 256))
    off = torch.zeros(F + 1, dtype=torch.int32, device="cuda")
    idx = torch.zeros(cap, dtype=torch.int32, device="cuda")
    out = torch.zeros((H, W, 4), dtype=torch.float32, device="cuda")
    grid = N.froxel_grid_struct(idx, off, fp, cap)
    if args.adjoint:
        g = torch.Generator(device="cuda")
        g.manual_seed(args.workload)
        d_rad = torch.randn((H, W, 4), dtype=torch.float32, device="cuda", generator=g)
        d_l = torch.zeros((max(df.n_lights, 1), 7), dtype=torch.float64, device="cuda")
        d_p = torch.zeros((H, W, 5), dtype=torch.float32, device="cuda")
    if args.fragments:
        fr = S.make_fragments(w.camera, 11, W * H, raster_order=True)
        d_fr = FR.bytes_tensor(fr)
        f_out = torch.zeros((len(fr), 4), dtype=torch.float32, device="cuda")
        prm = S.fragment_params(L.FRAGMENTS_TRANSPARENT, L.tile_grid(W, H)[0])
        fpar = N.FragmentParams(int(prm["mode"][0]), int(prm["num_tiles_x"][0]), float(prm["ambient_intensity"][0]),
                                (N.C.c_float * 3)(*[float(v) for v in prm["ambient_color"][0]]))
    maps = rcs = None
    glb = df.globals_
    if args.shadows:
        sc = S.shadow_scene(w.camera, w.lights, L.MAX_SHADOW_LIGHTS)
        dyn, sta = S.shadow_atlases(sc.kinds, args.atlas, seed=1, xp=torch, device="cuda")
        mats = torch.from_numpy(sc.matrices).cuda()
        cfg = FR.bytes_tensor(sc.config)
        maps = N.shadow_maps_struct(dyn, sta, mats, cfg, sc.max_lights)
        df = FR.upload(w.camera.record, w.globals_, sc.lights, w.gbuffer)
        glb = df.globals_
    if args.rc:
        d_rc = torch.from_numpy(S.rc_probes(7)).cuda()
        rcs = N.rc_cascade_struct(d_rc)
        glb = FR.bytes_tensor(S.rc_globals(w.globals_, (-60.0, -40.0, -110.0), (60.0, 40.0, 0.0)))
    for _ in range(args.frames):
        ev0.record()
        ctx.bin_froxels(df.camera, df.lights, df.n_lights, fp, off, idx, cap)
        if args.shadows or args.rc:
            ctx.shade_ex(df.camera, glb, df.gbuffer, df.lights, df.n_lights, grid, N.target_struct(out),
                         shadows=maps, rc=rcs)
        else:
            ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, N.target_struct(out))
        if args.adjoint:
            ctx.shade_adjoint(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, d_rad, W * 16, d_l,
                              d_p)
        if args.fragments:
            ctx.shade_fragments(df.camera, fpar, d_fr, len(fr), df.lights, df.n_lights, grid, f_out)
        ev1.record()
    ctx.sync_status()
    print(f"w{args.workload}: {ev0.elapsed_time(ev1) * 1e3:.1f} us per frame", flush=True)


if __name__ == "__main__":
    main()
