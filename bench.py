"""Benchmark of the deferred-lighting path on GB300.

Workload (the configuration the headline metric is quoted on): one 1920x1080 frame,
FP16 G-buffer (18 B/px: RGBA16F albedo+roughness, RG16F octahedral normal, R16F
metallic, R32F depth), 1024 GpuLights (768 point, 256 spot), froxel grid 16x9x24.
A step is one frame: froxel binning (hl_bin_froxels) + shading (hl_shade) into an
RGBA32F radiance target. Inputs are seeded synthetic data (helio_gb300.synthetic).

  value   Mpix/s with inputs resident in HBM, L2 flushed (256 MiB write) before every
          step; each step timed with CUDA events on the launching stream, its two calls
          issued back to back (the shading launches start while the binning runs).
  e2e     the same metric through the C ABI with pinned host buffers: every step
          copies the G-buffer, lights, camera and globals host->device (one packed
          copy) and the radiance device->host inside the timed region; the copies of
          neighbouring steps overlap the kernels on separate streams
          (helio_gb300.frame.HostFramePipeline).
  roofline  the shading kernel (the dominant kernel) against the measured HBM copy
          bandwidth (MEASURED_PEAKS.json) and the measured FP32 FMA rate
          (hl_probe_fp32_peak), with algorithmic bytes and FLOPs (include/hl_flops.h);
          its duration from the same steps run again with an event between the calls.
  cpu_baseline  the f32 CPU restatement of the same path (OpenMP over rows), full
          frames on the host's cores.

``--impl reference`` times the CPU restatement of the reference algorithm alone (the
reference itself is WGSL run by wgpu on a graphics driver, which this machine lacks).
Multi-GPU: the path does not exchange data between views, so N ranks run N
independent replicas ("replicas only"); value = pixels of all ranks / max rank time.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "Mpix/s lit, 1080p×1024 lights: plain fwd vs batched fwd+adjoint; % roofline"
WORKLOAD = "w1: 1920x1080 FP16 G-buffer (18 B/px), 1024 GpuLights (768 point + 256 spot), froxels 16x9x24"
L2_FLUSH_BYTES = 256 << 20


def flops_constants():
    text = (ROOT / "include" / "hl_flops.h").read_text()
    get = lambda k: int(re.search(rf"#define {k} (\d+)", text).group(1))
    return get("HL_FLOPS_CULL"), get("HL_FLOPS_FULL"), get("HL_FLOPS_PIXEL")


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "MEASURED_PEAKS.json hbm_gbs (copy bandwidth, measured)"
    return 6800.0, "fallback 6.8 TB/s"


def profile_traffic():
    """DRAM bytes per shading launch from the committed ncu summary, if present."""
    p = ROOT / "profiles" / "shade_w1_ncu.md"
    if not p.exists():
        return None
    m = re.search(r"dram_bytes_per_launch:\s*([0-9.eE+]+)", p.read_text())
    return float(m.group(1)) if m else None


class ClockSampler:
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [s.strip() for s in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if os.environ.get("HL_BENCH_BACKEND", "nccl") == "nccl" else "gloo")
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(world, v: float) -> float:
    if world == 1:
        return v
    import torch
    import torch.distributed as dist

    t = torch.tensor([v], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, pixels_per_step: int, steps: int, seconds: float):
    """Whole-job Mpix/s of ``world`` independent replicas, each lighting ``steps`` frames
    of ``pixels_per_step`` pixels: all ranks' pixels over the slowest rank's time.
    Returns (Mpix/s, slowest rank's seconds)."""
    t = max_over_ranks(world, seconds)
    return pixels_per_step * steps * world / t / 1e6, t


# ----------------------------------------------------------------------------------
# CPU arm (the f32 restatement of the reference algorithm)
# ----------------------------------------------------------------------------------


def cpu_frame_time(w, p, reps):
    import oracle

    times = []
    for _ in range(reps):
        t0 = time.perf_counter()
        off, idx = oracle.bin_froxels(w.camera.record, w.lights, p, capacity=1 << 22)
        oracle.shade(w.camera.record, w.globals_, w.gbuffer, w.lights, ("froxels", idx, off, p), precision="f32")
        times.append(time.perf_counter() - t0)
    return times


def run_reference(args, world, rank):
    if rank != 0:
        return
    import oracle
    from helio_gb300 import layouts as L
    from helio_gb300 import synthetic as S

    w = S.workload(1)
    W, H = w.gbuffer.width, w.gbuffer.height
    p = L.froxel_params(*w.froxel_grid, W, H, w.camera.far)
    cores = os.cpu_count() or 1
    oracle.set_threads(cores)
    cpu_frame_time(w, p, max(1, min(args.warmup, 3)))
    times = cpu_frame_time(w, p, args.steps)
    t = sum(times) / len(times)
    v = W * H / t / 1e6
    line = {
        "metric": METRIC, "value": round(v, 3), "unit": "Mpix/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(t * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
        "config": {"workload": WORKLOAD},
        "cpu_baseline": {"value": round(v, 3), "unit": "Mpix/s", "cores": cores, "kind": "port",
                         "sample": "full 1920x1080 frames: froxel binning + f32 shading (CPU restatement of "
                                   "light_cull/deferred_lighting WGSL; the reference's own WGSL needs a graphics "
                                   "stack, unavailable on this box)"},
        "e2e": {"value": round(v, 3), "unit": "Mpix/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------------
# GPU arm
# ----------------------------------------------------------------------------------


def run_ours(args, world, rank, local):
    import torch

    from helio_gb300 import frame as FR
    from helio_gb300 import layouts as L
    from helio_gb300 import native as N
    from helio_gb300 import synthetic as S

    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    w = S.workload(1)
    W, H = w.gbuffer.width, w.gbuffer.height
    p_np = L.froxel_params(*w.froxel_grid, W, H, w.camera.far)
    fp = N.froxel_params_from_numpy(p_np)
    F = fp.grid_x * fp.grid_y * fp.grid_z
    ctx = N.Context(local)
    df = FR.upload_workload(w, dev)
    stream = torch.cuda.current_stream()
    sh = stream.cuda_stream

    offsets = torch.zeros(F + 1, dtype=torch.int32, device=dev)
    cap = F * 64
    indices = torch.zeros(cap, dtype=torch.int32, device=dev)
    target = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
    grid = N.froxel_grid_struct(indices, offsets, fp, cap)
    tgt = N.target_struct(target)
    gbs = df.gbuffer
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)

    def frame():
        ctx.bin_froxels(df.camera, df.lights, df.n_lights, fp, offsets, indices, cap, sh)
        ctx.shade(df.camera, df.globals_, gbs, df.lights, df.n_lights, grid, tgt, sh)

    for _ in range(max(3, args.warmup)):
        frame()
    ctx.sync_status(sh)
    total_listed = int(offsets[-1].item())

    # ---------------- device-resident timed loop ----------------
    # The two calls are recorded back to back, as a renderer issues them: the shading's
    # launches start while the binning runs (programmatic dependent launches) and set
    # their pixels up before they wait for the lists. An event between the two calls
    # would end that overlap, so the kernels' own durations come from a second pass.
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for k in range(args.steps):
            flush.fill_(float(k))
            ev[k][0].record(stream)
            ctx.bin_froxels(df.camera, df.lights, df.n_lights, fp, offsets, indices, cap, sh)
            ctx.shade(df.camera, df.globals_, gbs, df.lights, df.n_lights, grid, tgt, sh)
            ev[k][1].record(stream)
        torch.cuda.synchronize()
    barrier(world)
    ctx.sync_status(sh)
    step_ms = [ev[k][0].elapsed_time(ev[k][1]) for k in range(args.steps)]

    # ---------------- kernel durations: the same steps with an event between the calls ----
    evk = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    torch.cuda.synchronize()
    for k in range(args.steps):
        flush.fill_(float(k))
        evk[k][0].record(stream)
        ctx.bin_froxels(df.camera, df.lights, df.n_lights, fp, offsets, indices, cap, sh)
        evk[k][1].record(stream)
        ctx.shade(df.camera, df.globals_, gbs, df.lights, df.n_lights, grid, tgt, sh)
        evk[k][2].record(stream)
    torch.cuda.synchronize()
    ctx.sync_status(sh)
    bin_ms = [evk[k][0].elapsed_time(evk[k][1]) for k in range(args.steps)]
    shade_ms = [evk[k][1].elapsed_time(evk[k][2]) for k in range(args.steps)]
    value, t_total = replica_throughput(world, W * H, args.steps, sum(step_ms) / 1e3)
    ms_per_step = t_total * 1e3 / args.steps
    clk = clocks.summary()

    # ---------------- end-to-end through the C ABI with host buffers ----------------
    # Every step uploads all of its inputs from pinned host memory (one packed copy) and
    # downloads its radiance; HostFramePipeline overlaps step k's kernels with the copies
    # of steps k+1 and k-1 on separate streams, as a renderer streaming frames would.
    pf = FR.PackedFrame(w.camera.record, w.globals_, w.lights, w.gbuffer)
    pipe = FR.HostFramePipeline(ctx, pf, w.froxel_grid, w.camera.far, capacity=cap, device=dev)
    host_outs = [torch.empty((H, W, 4), dtype=torch.float32).pin_memory() for _ in range(2)]
    h2d = pf.nbytes
    d2h = host_outs[0].numel() * host_outs[0].element_size()
    for k in range(max(3, args.warmup)):
        pipe.submit(pf, host_outs[k % 2])
    pipe.synchronize()
    s_up, s_comp, s_down = pipe.streams
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier(world)
    torch.cuda.synchronize()
    e0.record(s_up)
    for k in range(args.steps):
        pipe.submit(pf, host_outs[k % 2])
    e1.record(s_down)
    pipe.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    e2e_value, e2e_t = replica_throughput(world, W * H, args.steps, e0.elapsed_time(e1) / 1e3)
    ctx.sync_status(sh)
    e2e_check = bool(np.array_equal(host_outs[(args.steps - 1) % 2].numpy(), target.cpu().numpy()))

    # ---------------- roofline of the shading kernel ----------------
    counts = torch.zeros((H, W, 3), dtype=torch.int32, device=dev)
    ctx.shade_stats(df.camera, df.globals_, gbs, df.lights, df.n_lights, grid, counts, sh)
    ctx.sync_status(sh)
    c = counts.view(-1, 3).to(torch.int64).sum(0).tolist()
    depth = df.planes[-1]
    lit = int((depth < 1.0).sum().item())
    c_cull, c_full, c_px = flops_constants()
    flops = c[0] * c_cull + c[2] * c_full + lit * c_px
    bytes_alg = w.gbuffer.bytes_per_pixel * W * H + 16 * lit
    t_shade = statistics.median(shade_ms) / 1e3
    hbm_peak, hbm_src = measured_peaks()
    fp32_peak = ctx.probe_fp32_peak()
    gbs_ach = bytes_alg / t_shade / 1e9
    tf_ach = flops / t_shade / 1e12
    frac_hbm = gbs_ach / hbm_peak
    frac_fp32 = tf_ach / fp32_peak
    traffic = profile_traffic()
    if frac_hbm >= frac_fp32:
        roof = {"bound": "hbm", "achieved": round(gbs_ach, 1), "peak": hbm_peak, "unit": "GB/s",
                "frac": round(frac_hbm, 4), "traffic": traffic, "peak_source": hbm_src + ", of measured"}
    else:
        roof = {"bound": "fp32", "achieved": round(tf_ach, 3), "peak": round(fp32_peak, 2), "unit": "TFLOP/s",
                "frac": round(frac_fp32, 4), "traffic": traffic,
                "peak_source": "hl_probe_fp32_peak FFMA loop, of measured"}
    roof.update({
        "kernel": "shade_f16_kernel<RGBA32F> (FP16 G-buffer, froxel grid, 32x16 tile)",
        "kernel_ms": round(t_shade * 1e3, 4),
        "algorithmic_bytes": int(bytes_alg),
        "algorithmic_flops": int(flops),
        "hbm_frac": round(frac_hbm, 4),
        "fp32_frac": round(frac_fp32, 4),
        "fp32_peak_tflops": round(fp32_peak, 2),
        "pairs": {"listed": int(c[0]), "in_range": int(c[1]), "full": int(c[2]), "lit_pixels": lit},
    })

    # ---------------- the reference's 16x16 tile culling and tile-list frames ----------------
    ref_tiles = ref_tiles_form(ctx, dev, stream, flush, w, df, target)

    line = {
        "metric": METRIC, "value": round(value, 1), "unit": "Mpix/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 4), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP16 G-buffer)", "data": "synthetic",
        "config": {"workload": WORKLOAD, "l2": "flushed before every step (256 MiB write)",
                   "parallelism": f"replicas x{world}", "froxel_listed": total_listed},
        "breakdown_ms": {"bin_froxels": round(statistics.median(bin_ms), 4),
                         "shade": round(statistics.median(shade_ms), 4),
                         "note": "each kernel alone (an event between the calls); in the timed steps the "
                                 "shading launches start while the binning runs"},
        "e2e": {"value": round(e2e_value, 1), "unit": "Mpix/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(e2e_t * 1e3 / args.steps, 4),
                "pipelining": "3 streams x 2 buffer sets: upload k+1 / kernels k / download k-1",
                "result_matches_device_run": e2e_check},
        "gpu_launches": 3 * args.steps,  # timed steps: froxel binning, candidate light table, shading
        "ref_tiles": ref_tiles,
        "roofline": roof,
        "clocks": clk,
    }

    if rank == 0 and not args.no_cpu:
        import oracle
        from helio_gb300 import metrics

        cores = os.cpu_count() or 1
        oracle.set_threads(cores)
        cpu_frame_time(w, p_np, 1)
        times = cpu_frame_time(w, p_np, 5)
        t_cpu = statistics.median(times)
        line["cpu_baseline"] = {"value": round(W * H / t_cpu / 1e6, 3), "unit": "Mpix/s", "cores": cores,
                                "kind": "port",
                                "sample": "5 full 1920x1080 frames, froxel binning + f32 shading, OpenMP over rows"}
        off_o, idx_o = oracle.bin_froxels(w.camera.record, w.lights, p_np, capacity=1 << 22)
        # the FP64 oracle with the timed kernel's branch decisions at the cuts of
        # pbr_direct_light, recorded by one more launch of the same kernel
        img, pairs = logged_shade(ctx, dev, sh, df, grid, tgt, target, W * H * 4)
        ref, flips, unlisted = oracle.shade_forced(w.camera.record, w.globals_, w.gbuffer, w.lights,
                                                   ("froxels", idx_o, off_o, p_np), pairs)
        e = metrics.radiance_error(img, ref, flip_pixels=flips)
        e["unlisted_lit_pairs"] = int(unlisted.sum())
        e["lit_pairs"] = int(len(pairs))
        off_g = offsets.cpu().numpy().view(np.uint32)
        line["error_vs_fp64_oracle"] = {k: (round(v, 9) if isinstance(v, float) else v) for k, v in e.items()}
        line["error_vs_fp64_oracle"]["lists_bit_exact"] = bool(np.array_equal(off_g, off_o))
    if rank == 0 and not args.no_forms:
        line["forms"] = run_forms(ctx, dev, stream, flush, with_oracle=not args.no_cpu)
    if rank == 0:
        print(json.dumps(line), flush=True)
    ctx.close()


def logged_shade(ctx, dev, sh, df, grid, tgt, target, capacity):
    """One hl_shade launch with the lit-pair record on: (image as float64, (K, 2) uint32
    (y * W + x, light) pairs the kernel lit)."""
    import torch

    while True:
        pairs = torch.zeros((capacity, 2), dtype=torch.int32, device=dev)
        count = torch.zeros(1, dtype=torch.int32, device=dev)
        ctx.set_pair_log(pairs, count)
        ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, tgt, sh)
        ctx.set_pair_log(None)
        ctx.sync_status(sh)
        n = int(count.item())
        if n <= capacity:
            return target.double().cpu().numpy(), pairs[:n].cpu().numpy().view(np.uint32)
        capacity = n


def ref_tiles_form(ctx, dev, stream, flush, w1, df1, target1):
    """The reference's observable frame: its 16x16 tile culling (at most 64 lights per
    tile, light_cull.wgsl:123-180) and the shading over those tile lists, on w1 and on
    w2 (3840x2160, 4096 clumped lights), beside the froxel path ("exact": every light in
    range). Reports the tiles at the 64-light cap, the tile culling and tile-frame times,
    the froxel binning time, and how far the tile frame's radiance is from the exact one."""
    import torch

    from helio_gb300 import frame as FR
    from helio_gb300 import layouts as L
    from helio_gb300 import metrics
    from helio_gb300 import native as N
    from helio_gb300 import synthetic as S

    sh = stream.cuda_stream
    out = {}
    for name, wi in (("w1", 1), ("w2", 2)):
        w = w1 if wi == 1 else S.workload(2)
        df = df1 if wi == 1 else FR.upload_workload(w, dev)
        W, H = w.gbuffer.width, w.gbuffer.height
        tiles = N.load().hl_tile_count(W, H)
        t_lists = torch.zeros(tiles * 64, dtype=torch.int32, device=dev)
        t_counts = torch.zeros(tiles, dtype=torch.int32, device=dev)
        t_bin = _median_ms(lambda: ctx.bin_tiles_ref(df.camera, df.lights, df.n_lights, W, H, t_lists, t_counts, sh),
                           stream, flush, 30)
        tg = N.tile_grid_struct(t_lists, t_counts)
        rad_t = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
        tt = N.target_struct(rad_t)

        def tile_frame():
            ctx.bin_tiles_ref(df.camera, df.lights, df.n_lights, W, H, t_lists, t_counts, sh)
            ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, tg, tt, sh)

        t_frame = _median_ms(tile_frame, stream, flush, 30)
        fp = N.froxel_params_from_numpy(L.froxel_params(*w.froxel_grid, W, H, w.camera.far))
        F = fp.grid_x * fp.grid_y * fp.grid_z
        cap = F * 256
        off = torch.zeros(F + 1, dtype=torch.int32, device=dev)
        idx = torch.zeros(cap, dtype=torch.int32, device=dev)
        t_fbin = _median_ms(lambda: ctx.bin_froxels(df.camera, df.lights, df.n_lights, fp, off, idx, cap, sh),
                            stream, flush, 30)
        rad_x = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
        ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, N.froxel_grid_struct(idx, off, fp, cap),
                  N.target_struct(rad_x), sh)
        ctx.sync_status(sh)
        d = metrics.radiance_error(rad_t.cpu().numpy(), rad_x.cpu().numpy())
        out[name] = {
            "tiles": int(tiles), "at_cap_64": int((t_counts == 64).sum().item()),
            "max_tile_count": int(t_counts.max().item()),
            "bin_tiles_ref_ms": round(t_bin, 4), "tile_frame_ms": round(t_frame, 4),
            "bin_froxels_ms": round(t_fbin, 4), "froxel_grid": list(w.froxel_grid),
            "tile_vs_exact": {"max_rel": float(f"{d['max']:.3e}"), "p9999": float(f"{d['p9999']:.3e}"),
                              "mean_rel": float(f"{d['mean']:.3e}"), "pixels_over_2e-3": d["n_over_2e3"]},
        }
        del t_lists, rad_t, rad_x, off, idx
    return out


def _median_ms(fn, stream, flush, reps, warm=3):
    import torch

    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    ts = []
    for k in range(reps):
        flush.fill_(float(k))
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        ts.append(a.elapsed_time(b))
    return statistics.median(ts)


def run_forms(ctx, dev, stream, flush, with_oracle=True):
    """The other forms of the path, each timed with CUDA events (L2 flushed): adjoint
    (w4), batched views (w3), and the fragment light loops (Forward+ and transparent)
    over w1's lists."""
    import torch

    from helio_gb300 import frame as FR
    from helio_gb300 import layouts as L
    from helio_gb300 import native as N
    from helio_gb300 import synthetic as S

    sh = stream.cuda_stream
    forms = {}

    # ---- adjoint: w4, 1920x1080 FP32 G-buffer, 256 point lights ----
    w = S.workload(4)
    W, H = w.gbuffer.width, w.gbuffer.height
    fp = N.froxel_params_from_numpy(L.froxel_params(*w.froxel_grid, W, H, w.camera.far))
    F = fp.grid_x * fp.grid_y * fp.grid_z
    df = FR.upload_workload(w, dev)
    cap = F * max(df.n_lights, 1)
    off = torch.zeros(F + 1, dtype=torch.int32, device=dev)
    idx = torch.zeros(cap, dtype=torch.int32, device=dev)
    rad = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
    grid = N.froxel_grid_struct(idx, off, fp, cap)
    gen = torch.Generator(device=dev)
    gen.manual_seed(4)
    d_rad = torch.randn((H, W, 4), dtype=torch.float32, device=dev, generator=gen)
    d_l = torch.zeros((df.n_lights, 7), dtype=torch.float64, device=dev)
    d_p = torch.zeros((H, W, 5), dtype=torch.float32, device=dev)

    def fwd():
        ctx.bin_froxels(df.camera, df.lights, df.n_lights, fp, off, idx, cap, sh)
        ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, N.target_struct(rad), sh)

    def adj():
        ctx.shade_adjoint(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, d_rad, W * 16, d_l, d_p,
                          sh)

    t_f = _median_ms(fwd, stream, flush, 50)
    t_a = _median_ms(adj, stream, flush, 50)
    ctx.sync_status(sh)
    first = d_l.clone()
    adj()
    torch.cuda.synchronize()
    hbm_peak, _ = measured_peaks()
    # algorithmic bytes of the adjoint: FP32 G-buffer read, dL/dradiance read, pixel gradients written
    adj_bytes = W * H * (w.gbuffer.bytes_per_pixel + 16 + 20)
    forms["adjoint"] = {
        "workload": "w4: 1920x1080 FP32 G-buffer, 256 point lights, froxels 16x9x24",
        "fwd_ms": round(t_f, 4), "adjoint_ms": round(t_a, 4),
        "fwd_plus_adjoint_over_fwd": round((t_f + t_a) / t_f, 3),
        "fwd_plus_adjoint_mpix_s": round(W * H / ((t_f + t_a) / 1e3) / 1e6, 1),
        "deterministic": bool(torch.equal(first, d_l)),
        "adjoint_hbm_frac": round(adj_bytes / (t_a / 1e3) / 1e9 / hbm_peak, 4),
    }
    if with_oracle:
        import oracle

        p_np = L.froxel_params(*w.froxel_grid, W, H, w.camera.far)
        off_h = off.cpu().numpy().view(np.uint32)
        idx_h = idx.cpu().numpy().view(np.uint32)[: int(off_h[-1])]
        o_l, o_p = oracle.shade_adjoint(w.camera.record, w.globals_, w.gbuffer, w.lights, ("froxels", idx_h, off_h, p_np),
                                        d_rad.double().cpu().numpy())
        g_l, g_p = d_l.cpu().numpy(), d_p.double().cpu().numpy()
        sky = ~(w.gbuffer.planes[-1] < 1.0)
        rel_l = (np.abs(g_l - o_l).max(0) / np.maximum(np.abs(o_l).max(0), 1e-30)).max()
        ps = np.abs(o_p[~sky]).max(0)
        rel_p = (np.abs(g_p[~sky] - o_p[~sky]) / (np.abs(o_p[~sky]) + 1e-3 * ps)).max(1)
        forms["adjoint"]["error_vs_fp64_oracle"] = {
            "light_grad_max_over_scale": float(f"{rel_l:.3e}"),
            "pixel_grad_p9999": float(f"{np.quantile(rel_p, 0.9999):.3e}"),
            "pixel_grad_max": float(f"{rel_p.max():.3e}"),
        }
        # the forward radiance of this FP32 G-buffer against the FP64 oracle
        from helio_gb300 import metrics

        fwd()
        img, pairs = logged_shade(ctx, dev, sh, df, grid, N.target_struct(rad), rad, W * H * 4)
        ref, flips, _ = oracle.shade_forced(w.camera.record, w.globals_, w.gbuffer, w.lights,
                                            ("froxels", idx_h, off_h, p_np), pairs)
        e = metrics.radiance_error(img, ref, flip_pixels=flips)
        forms["adjoint"]["forward_error_vs_fp64_oracle"] = {
            "max": float(f"{e['max']:.3e}"), "p9999": float(f"{e['p9999']:.3e}"), "n": e["n"], "flips": e["flips"],
            "n_over_1e5": e["n_over_1e5"]}
    del df, off, idx, rad, d_rad, d_l, d_p

    # ---- batched: w3, 96 cube faces + 1080p + 720p, 2048 lights ----
    views, lights = S.batched_views()
    glb = L.make_globals(1, len(lights), ambient_color=(0.4, 0.45, 0.5), ambient_intensity=0.3)
    d_lights, d_glb = FR.bytes_tensor(lights, dev), FR.bytes_tensor(glb, dev)
    frames = [FR.upload(v.camera.record, glb, lights, v.gbuffer, dev) for v in views]
    outs = [torch.zeros((f.height, f.width, 4), dtype=torch.float32, device=dev) for f in frames]
    vs = [N.view_struct(f.camera, f.gbuffer, N.target_struct(o)) for f, o in zip(frames, outs)]
    t0 = time.time()
    cache = Path(tempfile.gettempdir()) / "helio_gb300_batch_tune.txt"
    plan = ctx.batch_plan(vs, d_lights, len(lights), d_glb, autotune=True, cache_path=str(cache), stream=sh)
    tune_s = time.time() - t0
    t_b = _median_ms(lambda: plan.execute(sh), stream, flush, 20)
    ctx.sync_status(sh)
    per = []
    big = max(plan.view_grid(i)[0] * plan.view_grid(i)[1] * plan.view_grid(i)[2] for i in range(len(frames)))
    sizing = torch.zeros(big * len(lights), dtype=torch.int32, device=dev)
    for i, f in enumerate(frames):
        g = plan.view_grid(i)
        p = N.froxel_params(*g, f.width, f.height, views[i].camera.far)
        Fv = g[0] * g[1] * g[2]
        o = torch.zeros(Fv + 1, dtype=torch.int32, device=dev)
        ctx.bin_froxels(f.camera, d_lights, len(lights), p, o, sizing, sizing.numel(), sh)
        c = max(1024, 2 * int(o[-1].item()))
        ix = torch.zeros(c, dtype=torch.int32, device=dev)
        per.append((f, p, o, ix, c, N.target_struct(outs[i])))
    del sizing

    def per_view():
        for f, p, o, ix, c, t in per:
            ctx.bin_froxels(f.camera, d_lights, len(lights), p, o, ix, c, sh)
            ctx.shade(f.camera, d_glb, f.gbuffer, d_lights, len(lights), N.froxel_grid_struct(ix, o, p, c), t, sh)

    t_v = _median_ms(per_view, stream, flush, 10)
    ctx.sync_status(sh)
    px = sum(f.width * f.height for f in frames)
    plan.execute(sh)  # the plan's own radiance for the error check
    torch.cuda.synchronize()
    ctx.sync_status(sh)
    batch_err = None
    if with_oracle:
        import oracle
        from helio_gb300 import metrics

        batch_err = {}
        for vi in (0, 40, 97):  # a 128^2 face, a 512^2 face, the 1280x720 viewport
            f, p, o, ix, c, _ = per[vi]
            plan_img = outs[vi].cpu().numpy().astype(np.float64)
            # the single-view path gives the plan's image bit for bit; its lit pairs are the plan's
            one = torch.zeros_like(outs[vi])
            img1, pairs = logged_shade(ctx, dev, sh, f, N.froxel_grid_struct(ix, o, p, c), N.target_struct(one), one,
                                       f.width * f.height * 4)
            off_h = o.cpu().numpy().view(np.uint32)
            idx_h = ix.cpu().numpy().view(np.uint32)[: int(off_h[-1])]
            pn = L.froxel_params(p.grid_x, p.grid_y, p.grid_z, p.width, p.height, p.slice_far, p.slice_near)
            ref, flips, _ = oracle.shade_forced(views[vi].camera.record, glb, views[vi].gbuffer, lights,
                                                ("froxels", idx_h, off_h, pn), pairs)
            e = metrics.radiance_error(plan_img, ref, flip_pixels=flips)
            batch_err[f"view{vi}_{f.width}x{f.height}"] = {"max": float(f"{e['max']:.3e}"),
                                                          "p9999": float(f"{e['p9999']:.3e}"), "flips": e["flips"],
                                                          "plan_equals_single_view": bool(np.array_equal(plan_img,
                                                                                                         img1))}
    forms["batched"] = {
        "workload": "w3: 16 probes x 6 cube faces (128^2/256^2/512^2) + 1920x1080 + 1280x720, FP16 G-buffers, "
                    "2048 lights",
        "views": len(frames), "pixels": px, "batched_ms": round(t_b, 4), "per_view_launches_ms": round(t_v, 4),
        "speedup": round(t_v / t_b, 2), "batched_mpix_s": round(px / (t_b / 1e3) / 1e6, 1),
        "launches": {"batched": 2, "per_view": 3 * len(frames)}, "autotune_s": round(tune_s, 2),
        "batched_form": "one persistent launch: froxel binning items of every view, then (view, tile) shading "
                        "items by device ticket (after one launch writing the views' candidate light tables)",
        "grids": sorted({(f.width, f.height) + plan.view_grid(i) for i, f in enumerate(frames)}),
        "hbm_frac": round(px * (18 + 16) / (t_b / 1e3) / 1e9 / measured_peaks()[0], 4),
        "error_vs_fp64_oracle": batch_err,
    }
    plan.close()

    # ---- fragments: Forward+ and transparent light loops over w1's froxel lists ----
    w = S.workload(1)
    W, H = w.gbuffer.width, w.gbuffer.height
    p_np = L.froxel_params(*w.froxel_grid, W, H, w.camera.far)
    fp = N.froxel_params_from_numpy(p_np)
    F = fp.grid_x * fp.grid_y * fp.grid_z
    df = FR.upload_workload(w, dev)
    cap = F * 64
    off = torch.zeros(F + 1, dtype=torch.int32, device=dev)
    idx = torch.zeros(cap, dtype=torch.int32, device=dev)
    ctx.bin_froxels(df.camera, df.lights, df.n_lights, fp, off, idx, cap, sh)
    ctx.sync_status(sh)
    grid = N.froxel_grid_struct(idx, off, fp, cap)
    n_frag = W * H
    fr = S.make_fragments(w.camera, 11, n_frag, raster_order=True)
    d_fr = FR.bytes_tensor(fr, dev)
    out = torch.zeros((n_frag, 4), dtype=torch.float32, device=dev)
    hbm_peak, _ = measured_peaks()
    frag = {"workload": "w1 camera, lights and froxel lists; one fragment per pixel (view depth U[2, 14], "
                        "raster order), 80 B hl_fragment records, RGBA32F out", "fragments": n_frag}
    sel = np.random.default_rng(12).choice(n_frag, 65536, replace=False)
    off_h = off.cpu().numpy().view(np.uint32)
    idx_h = idx.cpu().numpy().view(np.uint32)[: int(off_h[-1])]
    for mode, name in ((L.FRAGMENTS_FORWARD, "forward"), (L.FRAGMENTS_TRANSPARENT, "transparent")):
        prm = S.fragment_params(mode, L.tile_grid(W, H)[0])
        fpar = N.FragmentParams(int(prm["mode"][0]), int(prm["num_tiles_x"][0]), float(prm["ambient_intensity"][0]),
                                (N.C.c_float * 3)(*[float(v) for v in prm["ambient_color"][0]]))
        t_f = _median_ms(lambda: ctx.shade_fragments(df.camera, fpar, d_fr, n_frag, df.lights, df.n_lights, grid, out,
                                                     stream=sh), stream, flush, 20)
        ctx.sync_status(sh)
        entry = {"ms": round(t_f, 4), "mfrag_s": round(n_frag / t_f / 1e3, 1),
                 "hbm_frac": round(n_frag * (80 + 16) / (t_f / 1e3) / 1e9 / hbm_peak, 4)}
        if with_oracle:
            import oracle

            want = oracle.shade_fragments(w.camera.record, prm, fr[sel], w.lights, ("froxels", idx_h, off_h, p_np))
            got = out.cpu().numpy().astype(np.float64)[sel]
            keep = ~np.isnan(want[:, 0])
            g, o = got[keep][:, :3], want[keep][:, :3]
            rel = (np.abs(g - o) / np.maximum(np.abs(o), 1e-6 * np.abs(o).max())).max(1)
            entry["error_vs_fp64_oracle"] = {"sample": int(keep.sum()), "max": float(f"{rel.max():.3e}"),
                                             "p9999": float(f"{np.quantile(rel, 0.9999):.3e}"),
                                             "over_1e-3": int((rel > 1e-3).sum())}
        frag[name] = entry
    forms["fragments"] = frag

    # ---- the same w1 frame into an RGBA16F target (the reference's pre_aa format) ----
    out32 = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
    out16 = torch.zeros((H, W, 4), dtype=torch.float16, device=dev)
    t16 = N.target_struct(out16, N.TARGET_RGBA16F)

    def frame16():
        ctx.bin_froxels(df.camera, df.lights, df.n_lights, fp, off, idx, cap, sh)
        ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, t16, sh)

    t_16 = _median_ms(frame16, stream, flush, 50)
    ctx.shade(df.camera, df.globals_, df.gbuffer, df.lights, df.n_lights, grid, N.target_struct(out32), sh)
    ctx.sync_status(sh)
    a32, a16 = out32[..., :3].double(), out16[..., :3].double()
    floor = 1e-6 * float(a32.abs().max())  # the error metric's floor of 1e-6 x the image maximum
    rel16 = ((a16 - a32).abs().amax(-1) / a32.abs().amax(-1).clamp_min(floor)).flatten()
    pf = FR.PackedFrame(w.camera.record, w.globals_, w.lights, w.gbuffer)
    pipe = FR.HostFramePipeline(ctx, pf, w.froxel_grid, w.camera.far, capacity=cap, device=dev,
                                target_format=N.TARGET_RGBA16F)
    host16 = [torch.empty((H, W, 4), dtype=torch.float16).pin_memory() for _ in range(2)]
    for k in range(3):
        pipe.submit(pf, host16[k % 2])
    pipe.synchronize()
    s_up, s_comp, s_down = pipe.streams
    steps16 = 200
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(s_up)
    for k in range(steps16):
        pipe.submit(pf, host16[k % 2])
    e1.record(s_down)
    pipe.synchronize()
    torch.cuda.synchronize()
    t_e2e16 = e0.elapsed_time(e1) / steps16
    forms["pre_aa_rgba16f"] = {
        "workload": WORKLOAD + ", radiance into an RGBA16F target (the reference's pre_aa format)",
        "frame_ms": round(t_16, 4), "mpix_s": round(W * H / t_16 / 1e3, 1),
        "e2e": {"mpix_s": round(W * H / t_e2e16 / 1e3, 1), "steps": steps16, "h2d_bytes_per_step": int(pf.nbytes),
                "d2h_bytes_per_step": int(host16[0].numel() * host16[0].element_size())},
        "rel_vs_rgba32f": {"max": float(f"{float(rel16.max()):.3e}"),
                           "p9999": float(f"{float(torch.quantile(rel16[::16].float(), 0.9999)):.3e}")},
        "result_matches_device_run": bool(torch.equal(host16[(steps16 - 1) % 2], out16.cpu())),
    }

    # ---- the G-buffer pass's fragment stage, and a reference-layout frame it feeds ----
    forms["gbuffer_write"] = gbuffer_write_form(ctx, dev, stream, flush, w, df, fp, off, idx, cap, grid, with_oracle)
    # ---- the w1 frame with the shadow term of the light loop ----
    forms["shadows"] = shadows_form(ctx, dev, stream, flush, w, fp, off, idx, cap, grid, with_oracle)
    return forms


def shadows_form(ctx, dev, stream, flush, w, fp, off, idx, cap, grid, with_oracle=True):
    """The w1 frame (froxel binning + shading into RGBA32F) with shadow_factor: the first
    42 lights (the shader's MAX_SHADOW_LIGHTS; all point lights in w1) cast shadows from
    six 1024^2 cube faces each, dynamic and static Depth32Float atlases of 252 layers
    (2.1 GB), the default (Medium) ShadowConfig: 12-tap Vogel PCF over both atlases."""
    import torch

    from helio_gb300 import frame as FR
    from helio_gb300 import layouts as L
    from helio_gb300 import metrics
    from helio_gb300 import native as N
    from helio_gb300 import synthetic as S

    sh = stream.cuda_stream
    W, H = w.gbuffer.width, w.gbuffer.height
    sc = S.shadow_scene(w.camera, w.lights, L.MAX_SHADOW_LIGHTS, quality="medium")
    dyn, sta = S.shadow_atlases(sc.kinds, L.SHADOW_ATLAS_SIZE, seed=1, xp=torch, device=dev)
    mats = torch.from_numpy(sc.matrices).to(dev)
    cfg = FR.bytes_tensor(sc.config, dev)
    maps = N.shadow_maps_struct(dyn, sta, mats, cfg, sc.max_lights)
    d_lights = FR.bytes_tensor(sc.lights, dev)
    dfs = FR.upload(w.camera.record, w.globals_, sc.lights, w.gbuffer, dev)
    rad = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
    tgt = N.target_struct(rad)

    def frame():
        ctx.bin_froxels(dfs.camera, d_lights, dfs.n_lights, fp, off, idx, cap, sh)
        ctx.shade_shadowed(dfs.camera, dfs.globals_, dfs.gbuffer, d_lights, dfs.n_lights, grid, maps, tgt, sh)

    t_s = _median_ms(frame, stream, flush, 50)
    ctx.sync_status(sh)
    casters = [int(v) for v in np.bincount(sc.lights["light_type"][: L.MAX_SHADOW_LIGHTS], minlength=3)]
    entry = {"workload": WORKLOAD + ", lights 0-41 cast shadows (1024^2 cube faces, dynamic + static atlases of "
                                    "252 layers), Medium ShadowConfig (12-tap PCF)",
             "casters_by_type": {"directional": casters[0], "point": casters[1], "spot": casters[2]},
             "frame_ms": round(t_s, 4), "mpix_s": round(W * H / t_s / 1e3, 1),
             "atlas_bytes": int(2 * dyn.numel() * 4)}
    if with_oracle:
        import oracle

        off_h = off.cpu().numpy().view(np.uint32)
        idx_h = idx.cpu().numpy().view(np.uint32)[: int(off_h[-1])]
        p_np = L.froxel_params(*w.froxel_grid, W, H, w.camera.far)
        shadows = dict(dynamic=dyn.cpu().numpy(), static=sta.cpu().numpy(), matrices=sc.matrices, config=sc.config,
                       max_lights=sc.max_lights)
        ref, pc, _ = oracle.shade_shadowed(w.camera.record, w.globals_, w.gbuffer, sc.lights,
                                           ("froxels", idx_h, off_h, p_np), shadows, pair_counts=True)
        st = torch.zeros((H, W, 3), dtype=torch.int32, device=dev)
        ctx.shade_stats(dfs.camera, dfs.globals_, dfs.gbuffer, d_lights, dfs.n_lights, grid, st, sh)
        ctx.sync_status(sh)
        e = metrics.radiance_error(rad.double().cpu().numpy(), ref, st.cpu().numpy().view(np.uint32)[..., 2],
                                   pc[..., 2])
        plain = oracle.shade(w.camera.record, w.globals_, w.gbuffer, sc.lights, ("froxels", idx_h, off_h, p_np))
        sky = np.isnan(ref[..., 0])
        darker = float((ref[~sky][:, :3] < plain[~sky][:, :3] * (1 - 1e-6)).any(-1).mean())
        entry["pixels_darkened_by_shadows"] = round(darker, 4)
        entry["error_vs_fp64_oracle"] = {"max": float(f"{e['max']:.3e}"), "p9999": float(f"{e['p9999']:.3e}"),
                                         "n_over_2e3": e["n_over_2e3"], "flips": e["flips"], "n": e["n"]}

    # the same frame with radiance-cascade GI as well (hl_shade_ex: shadows + RC probes)
    probes = S.rc_probes(7)
    d_rc = torch.from_numpy(probes).to(dev)
    rcs = N.rc_cascade_struct(d_rc)
    glb_rc = S.rc_globals(w.globals_, (-60.0, -40.0, -110.0), (60.0, 40.0, 0.0))
    d_glb_rc = FR.bytes_tensor(glb_rc, dev)

    def frame_rc():
        ctx.bin_froxels(dfs.camera, d_lights, dfs.n_lights, fp, off, idx, cap, sh)
        ctx.shade_ex(dfs.camera, d_glb_rc, dfs.gbuffer, d_lights, dfs.n_lights, grid, tgt, shadows=maps, rc=rcs,
                     stream=sh)

    t_rc = _median_ms(frame_rc, stream, flush, 50)
    ctx.sync_status(sh)
    rc_entry = {"frame_ms": round(t_rc, 4), "mpix_s": round(W * H / t_rc / 1e3, 1),
                "volume": "rc_world [-60,-40,-110]..[60,40,0], synthetic 64x1024 RGBA16F probes"}
    if with_oracle:
        ref, pc, _ = oracle.shade_ex(w.camera.record, glb_rc, w.gbuffer, sc.lights, ("froxels", idx_h, off_h, p_np),
                                     shadows=shadows, rc=probes, pair_counts=True)
        e = metrics.radiance_error(rad.double().cpu().numpy(), ref, st.cpu().numpy().view(np.uint32)[..., 2],
                                   pc[..., 2])
        rc_entry["error_vs_fp64_oracle"] = {"max": float(f"{e['max']:.3e}"), "p9999": float(f"{e['p9999']:.3e}"),
                                            "n_over_2e3": e["n_over_2e3"], "n": e["n"]}
    entry["with_rc_gi"] = rc_entry
    del dyn, sta
    torch.cuda.empty_cache()
    return entry


def gbuffer_write_form(ctx, dev, stream, flush, w, df, fp, off, idx, cap, grid, with_oracle=True):
    """hl_write_gbuffer over a 1920x1080 material scene (64 materials, 24 textures, all
    eight targets), and the frame write -> froxel binning -> shading of the written
    HL_GBUF_REFERENCE G-buffer (28 B/px) with w1's camera and lights. Algorithmic bytes
    of the write: the 64-byte surface record of every pixel read, 48 bytes of targets
    per written pixel; material and texture reads (L2-resident tables) not counted."""
    import torch

    from helio_gb300 import frame as FR
    from helio_gb300 import native as N
    from helio_gb300 import synthetic as S

    sh = stream.cuda_stream
    W, H = w.gbuffer.width, w.gbuffer.height
    scene = S.material_scene(w.camera, 1001)
    ds = FR.upload_material_scene(scene, dev)
    planes, tg = FR.gbuffer_targets(W, H, optional=True, fill=0, device=dev)
    t_w = _median_ms(lambda: ds.write(ctx, tg, sh), stream, flush, 50)
    ctx.sync_status(sh)
    written = (planes[1].view(torch.int16) != 0).any(-1)  # a written normal is a unit vector
    n_written = int(written.sum())
    alg = W * H * 64 + n_written * 48
    hbm_peak, _ = measured_peaks()
    entry = {"workload": "1920x1080 material scene (64 materials, 24 textures RGBA8 sRGB/unorm, RGBA16F, "
                         "RGBA32F, 128-512 texels, repeat/clamp/mirror, linear/nearest), 64 B surface records, "
                         "all eight targets", "pixels": W * H, "written": n_written,
             "ms": round(t_w, 4), "mpix_s": round(W * H / t_w / 1e3, 1), "algorithmic_bytes": alg,
             "hbm_frac": round(alg / (t_w / 1e3) / 1e9 / hbm_peak, 4)}
    if with_oracle:
        import oracle

        want, wr, _ = oracle.write_gbuffer(scene.globals_, scene.surfaces, scene.materials, scene.material_textures,
                                           scene.textures)
        wt = want[wr]
        host = [p.cpu().numpy() for p in planes]
        u8_err = max(float(np.abs(host[i][wr].astype(np.float64) - np.clip(wt[:, s], 0, 1) * 255.0).max())
                     for i, s in ((0, slice(0, 4)), (2, slice(8, 12))))
        off16 = 0
        unit = np.array([2e-6, 2e-6, 2e-6, 0.0])  # absolute f32 error of unit-normal components
        for i, s, fl in ((1, slice(4, 8), unit), (3, slice(12, 16), 0.0), (4, slice(16, 18), 0.0),
                         (7, slice(18, 20), 0.0)):
            g, o = host[i][wr].astype(np.float64), wt[:, s]
            off16 += int((np.abs(g - o) > 2.0 ** -11 * np.maximum(np.abs(o), 2.0 ** -14) + 1e-5 * np.abs(o)
                          + fl).sum())
        entry["error_vs_fp64_oracle"] = {"written_mask_equal": bool(np.array_equal(wr, written.cpu().numpy())),
                                         "unorm8_max_abs_byte_error": round(u8_err, 4),
                                         "f16_values_beyond_half_ulp": off16}
    depth = torch.where(written, ds.depth, torch.ones_like(ds.depth))  # discarded fragments write no depth
    gbs = FR.reference_gbuffer(planes, depth)
    rad = torch.zeros((H, W, 4), dtype=torch.float32, device=dev)
    tgt = N.target_struct(rad)

    def frame():
        ds.write(ctx, tg, sh)
        ctx.bin_froxels(df.camera, df.lights, df.n_lights, fp, off, idx, cap, sh)
        ctx.shade(df.camera, df.globals_, gbs, df.lights, df.n_lights, grid, tgt, sh)

    t_f = _median_ms(frame, stream, flush, 50)
    ctx.sync_status(sh)
    entry["reference_layout_frame"] = {
        "steps": "hl_write_gbuffer + hl_bin_froxels + hl_shade (HL_GBUF_REFERENCE, 28 B/px), w1 lights",
        "ms": round(t_f, 4), "mpix_s": round(W * H / t_f / 1e3, 1)}
    # The reflection draw over the lit frame: SSR and planar hits and lightmap UVs
    # (synthetic, 1920x1080). Algorithmic bytes per pixel: the G-buffer planes the draw
    # reads (normal 8, orm 4, emissive 8, depth 4), the three images (8 + 8 + 4) and the
    # RGBA32F target's read-modify-write (16 + 16).
    ssr, planar, lm = (torch.from_numpy(a).to(dev) for a in S.reflection_images(W, H, 77))
    t_r = _median_ms(lambda: ctx.shade_reflections(df.camera, df.globals_, gbs, tgt, ssr=ssr, planar=planar,
                                                   lightmap_uv=lm, stream=sh), stream, flush, 50)
    ctx.sync_status(sh)
    alg_r = W * H * 76
    entry["reflections"] = {
        "steps": "hl_shade_reflections (fs_reflection: SSR + planar, lightmap UVs, no RC) over the written "
                 "HL_GBUF_REFERENCE G-buffer, RGBA32F target", "ms": round(t_r, 4),
        "mpix_s": round(W * H / t_r / 1e3, 1), "algorithmic_bytes": alg_r,
        "hbm_frac": round(alg_r / (t_r / 1e3) / 1e9 / hbm_peak, 4)}
    return entry


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-forms", action="store_true", help="skip the adjoint / batched-views forms")
    args = ap.parse_args()
    if args.impl == "reference":
        # CPU arm: rank 0 alone runs; other ranks exit without work.
        run_reference(args, int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")))
        return
    world, rank, local = dist_setup(args.gpus)
    run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
