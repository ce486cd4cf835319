"""Benchmark of the rebin path: views/s at 3M Gaussians, SH degree 3, 1080p.

Workload (the headline configuration): a 3,000,000-splat scene of 64
isotropic clusters with SH degree 3 colour, rendered at 1920x1080 with 16x16
tiles from a 64-pose orbit (radius 12, +-20 degree elevation jitter).  One
step = one pass of the rebin path over every view of the orbit.  The scene is
uploaded once (as SceneSyncer does); inputs (732 MB of splat data) are larger
than the 129 MB L2, so no L2 flush is interposed.

Arms:
  default             the library through its C ABI, CUDA events on the stream
                      the library enqueues on; `e2e` re-times the same views
                      through the public C entry point with host camera
                      structs in and a device->pinned-host image copy out.
  --impl reference    the reference path's CPU restatement (the oracle, all
                      host threads) on a bounded sample: one view per step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "webgpu-3dgs_gb300"))

METRIC = "views/s at 3M Gaussians 1080p, learned+batched vs plain, same image"
WORKLOAD = ("3M Gaussians fp32 SH3 (64 clusters, seed 0), 1920x1080, 64-pose orbit "
            "r=12 +-20deg; plain path at the reference's 16x16 tiles, batched path at the "
            "autotuned tile size / digit width / raster batch (same image)")
N_SPLATS, WIDTH, HEIGHT, TILE = 3_000_000, 1920, 1080, 16
STAGES = ["preprocess-splats", "prefix-scan", "emit-tile-refs", "radix-sort",
          "identify-tile-ranges", "rasterize-tiles"]


def peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for name, val in zip(names, parts[4:8]):
                if val.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(n_views: int, rank: int = 0):
    """The 3M-splat scene and `n_views` orbit cameras.  Every rank renders the
    same scene from its own poses (elevation jitter seeded by the rank), so
    ranks hold disjoint views and rank 0's are the single-GPU workload."""
    from gs3d import scenes
    data = scenes.scene_clusters(N_SPLATS, seed=0, sh_degree=3)
    return data, workload_cameras(n_views, rank)


def workload_cameras(n_views: int, rank: int = 0):
    """Camera uniforms of `rank`'s views: the 64-pose orbit (radius 12,
    +-20 deg elevation jitter seeded by the rank), repeated to `n_views`."""
    from gs3d import scenes
    eyes = scenes.orbit_eyes(64, radius=12.0, jitter_deg=20.0, seed=rank)
    return [scenes.camera_at(eyes[i % 64], WIDTH, HEIGHT).getUniformData(WIDTH, HEIGHT)
            for i in range(n_views)]


def max_over_ranks(value: float, world: int, device: str = "cuda") -> float:
    """The largest of every rank's `value` (the slowest rank's time), on all
    ranks; the identity for a single process."""
    if world <= 1:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def c0_workload():
    """The small benchmark scene: 100k splats (seed 0), SH 0, one camera at
    distance 6, 1280x720 (rendered at 16x16 tiles)."""
    from gs3d import scenes
    w, h = 1280, 720
    return scenes.scene_small(100_000, seed=0), \
        scenes.small_camera(w, h).getUniformData(w, h), (w, h)


def cpu_c0_stages(threads):
    """The oracle's six stages on the small benchmark scene, each timed, at
    `threads` threads (the scan, emit and identify restatements are serial)."""
    from oracle import Oracle
    o = Oracle()
    data, u, (w, h) = c0_workload()
    tx, ty = -(-w // TILE), -(-h // TILE)
    t = {}
    t0 = time.perf_counter()
    proj, counts = o.preprocess(u, (tx, ty), (np.float32(1.0 / TILE), np.float32(1.0 / TILE)),
                                data.positions, data.scales, data.rotations, data.colors,
                                threads=threads)
    t1 = time.perf_counter()
    off, total = o.prefix_scan(counts)
    t2 = time.perf_counter()
    keys, vals = o.emit(tx, proj, off, total)
    t3 = time.perf_counter()
    keys, vals = o.radix_sort(keys, vals, threads)
    t4 = time.perf_counter()
    toff = o.identify(keys, tx * ty)
    t5 = time.perf_counter()
    o.rasterize(w, h, TILE, TILE, proj, toff, vals, threads)
    t6 = time.perf_counter()
    t = {"preprocess-splats": t1 - t0, "prefix-scan": t2 - t1, "emit-tile-refs": t3 - t2,
         "radix-sort": t4 - t3, "identify-tile-ranges": t5 - t4, "rasterize-tiles": t6 - t5}
    total_s = t6 - t0
    return {"views_per_s": round(1.0 / total_s, 2), "threads": threads,
            "stage_ms": {k: round(v * 1e3, 2) for k, v in t.items()}}


def algorithmic_bytes(n, R, tiles, tile_passes, sh_floats, fused, views_per_scene=1):
    """Minimum bytes each stage must move for one view (inputs read once,
    outputs written once), the numerator of the per-stage roofline.  The
    batched preprocess reads a scene's splats once per launch for all
    `views_per_scene` views of it, so a view is charged that share of the read."""
    full_passes = 4 + tile_passes
    return {
        # splat SoA (64 B) + SH rest read once per scene and launch; per
        # splat-view the record and count, fused: + depth key, depth id and
        # the one-word tile rectangle
        "preprocess-splats": n * (64 + 4 * sh_floats) / views_per_scene
                             + n * (64 + 4 + (12 if fused else 0)),
        "depth-sort": 4 * n + 4 * 16 * n,
        "prefix-scan": 12 * n if fused else 8 * n,
        # fused: depth id, depth key, offset and one-word rectangle per splat-view
        "emit-tile-refs": n * (4 + 4 + 4 + 4) + 12 * R if fused else n * (24 + 4) + 12 * R,
        "radix-sort": tile_passes * 24 * R if fused else 8 * R + full_passes * 24 * R,
        "identify-tile-ranges": 4 * R + 4 * (tiles + 1),
        "rasterize-tiles": 44 * R + 8 * WIDTH * HEIGHT,
    }


# DRAM bytes per unit of the HBM-bound kernels, from ncu captures of a
# 2-view batch of the same workload (profiles/), scaled to a launch by the
# units it processes: tile-digit pass per ref (by tile size); preprocess per
# scene splat read + per splat-view written; emit per (splat-view, ref) with
# one-word rectangles.
DRAM_PER_REF_PASS = {(32, 32): 22.4, (16, 16): 25.1, (64, 32): 21.2}
DRAM_PREPROCESS = (732.1e6 / 3e6, 434.7e6 / 6e6)
DRAM_EMIT = {(32, 32): (365.2e6, 6e6, 23.7e6), (64, 32): (273.4e6, 6e6, 16.99e6)}


def dominant_traffic(stage, tile, refs_per_launch, splats_per_launch, scene_splats):
    """Measured DRAM bytes of one launch of the dominant HBM-bound kernel, or
    None where no capture covers it."""
    if stage == "radix-sort" and tile in DRAM_PER_REF_PASS:
        return int(DRAM_PER_REF_PASS[tile] * refs_per_launch)
    if stage == "preprocess-splats":
        return int(DRAM_PREPROCESS[0] * scene_splats + DRAM_PREPROCESS[1] * splats_per_launch)
    if stage == "emit-tile-refs" and tile in DRAM_EMIT:
        b, n, r = DRAM_EMIT[tile]
        return int(b * (0.5 * splats_per_launch / n + 0.5 * refs_per_launch / r))
    return None


# Pipe use of the raster kernel (ncu --set full, one launch of the headline
# path's raster at 32x32 tiles, 2-view batch;
# profiles/raster_culled2_t32_2views_3M_sh3_1080p.md).
RASTER_NCU = {"kernel": "raster_kernel_culled2", "issue_active": 0.732, "pipe_fma": 0.442,
              "pipe_alu": 0.589, "pipe_xu": 0.173, "warps_active": 0.497,
              "source": "profiles/raster_culled2_t32_2views_3M_sh3_1080p.md (raster_t32c)"}


def raster_work(view=0, tile=TILE):
    """(pixel, splat) pairs of the reference raster loop on one full-size view,
    counted by the oracle: iterated (tile lists walked up to each pixel's
    termination), exp evaluated, blended."""
    from oracle import Oracle
    o = Oracle()
    data, cams = make_workload(view + 1)
    r = o.rebin(cams[view], WIDTH, HEIGHT, tile, tile, data.positions, data.scales,
                data.rotations, data.colors, data.sphericalHarmonics, 3,
                key_capacity=N_SPLATS * 16)
    return o.raster_pairs(WIDTH, HEIGHT, tile, tile, r["projected_splats"], r["tile_offsets"],
                          r["sort_values_a"])


def install_cost_model(lib, ctx, tile_w, tile_h=None):
    """Cost model trained for this tile size, behind its gate; returns the
    schedule to use and the model's held-out metrics (None when no model
    exists for the tile size: key counts)."""
    from gs3d import _lib, learned
    path = learned.checkpoint_for(tile_w, tile_w if tile_h is None else tile_h)
    if path is None:
        return _lib.SCHEDULE_KEY_COUNT, None
    mp, mmean, mstd, mmetrics, mbound = learned.load(path)
    if not learned.gate(mmetrics, mbound):
        return _lib.SCHEDULE_KEY_COUNT, mmetrics
    f32 = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
    mp, mmean, mstd = f32(mp), f32(mmean), f32(mstd)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    if lib.gs3d_set_cost_model(ctx, ptr(mp), ptr(mmean), ptr(mstd)) != 0:
        raise RuntimeError(lib.gs3d_last_error(ctx).decode())
    return _lib.SCHEDULE_LEARNED, mmetrics


def run_ours(args, rank, world):
    import torch

    from gs3d import _lib
    from gs3d.camera import camera_struct

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream()
    lib = _lib.load()
    ctx = C.c_void_p()
    cfg = _lib.Config_t(dev, TILE, TILE, 16, C.c_void_p(stream.cuda_stream), 0)
    rc = lib.gs3d_create(C.byref(ctx), C.byref(cfg))
    if rc != 0:
        raise RuntimeError(f"gs3d_create failed: {rc}")

    def check(rc):
        if rc != 0:
            raise RuntimeError(lib.gs3d_last_error(ctx).decode())

    data, cams = make_workload(args.views, rank)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    check(lib.gs3d_set_splats(ctx, data.splatCount, ptr(data.positions), ptr(data.scales),
                              ptr(data.rotations), ptr(data.colors),
                              ptr(data.sphericalHarmonics), 3, 0))
    cam_structs = [camera_struct(u) for u in cams]

    def set_tuning(tile, digit_bits, raster_batch):
        check(lib.gs3d_set_tuning(ctx, C.byref(_lib.Tuning_t(tile, tile, digit_bits,
                                                              raster_batch))))

    # first pass at the reference's 16x16 tiles: size the key buffers and
    # record the per-view ref counts
    refs = []
    for cs in cam_structs:
        for _ in range(3):
            check(lib.gs3d_rebin(ctx, C.byref(cs), WIDTH, HEIGHT))
            rc = lib.gs3d_synchronize(ctx)
            if rc != _lib.ERR_CAPACITY:
                check(rc)
                break
        r = C.c_uint32()
        check(lib.gs3d_ref_count(ctx, C.byref(r)))
        refs.append(r.value)

    B = args.batch
    batches = []
    for b0 in range(0, len(cams), B):
        arr = (_lib.View_t * min(B, len(cams) - b0))()
        for i in range(len(arr)):
            arr[i].camera = cam_structs[b0 + i]
            arr[i].scene = 0
            arr[i].width, arr[i].height = WIDTH, HEIGHT
        batches.append(arr)

    # autotuner over the first batch (tile size, digit width, raster batch);
    # every candidate renders the same image
    tune_out = (_lib.TuneResult_t * 64)()
    n_tuned = C.c_uint32()
    check(lib.gs3d_set_flags(ctx, _lib.FLAG_CUDA_GRAPH))
    check(lib.gs3d_autotune(ctx, C.cast(batches[0], C.c_void_p), len(batches[0]), 2, tune_out,
                            64, C.byref(n_tuned)))
    check(lib.gs3d_set_flags(ctx, 0))
    tuned = _lib.Tuning_t()
    check(lib.gs3d_get_tuning(ctx, C.byref(tuned)))
    tune_table = sorted(({"tile": [r.tuning.tile_w, r.tuning.tile_h],
                          "digit_bits": r.tuning.digit_bits,
                          "raster_batch": r.tuning.raster_batch,
                          "ms_per_view": round(float(r.ms_per_view), 4),
                          "tile_passes": int(r.tile_passes)}
                         for r in tune_out[:n_tuned.value]), key=lambda r: r["ms_per_view"])
    best = next(r for r in tune_out[:n_tuned.value]
                if (r.tuning.tile_w, r.tuning.tile_h, r.tuning.digit_bits,
                    r.tuning.raster_batch) ==
                (tuned.tile_w, tuned.tile_h, tuned.digit_bits, tuned.raster_batch))
    tuned_R = best.refs / len(batches[0])
    tuned_passes = int(best.tile_passes)
    batched_schedule, tuned_model = install_cost_model(lib, ctx, tuned.tile_w, tuned.tile_h)

    def run_step(path):
        if path == "batched":
            for arr in batches:
                check(lib.gs3d_rebin_batch(ctx, C.cast(arr, C.c_void_p), len(arr)))
        else:
            for cs in cam_structs:
                check(lib.gs3d_rebin(ctx, C.byref(cs), WIDTH, HEIGHT))

    def timed(path: str, schedule, graph=False):
        flags = (_lib.FLAG_CUDA_GRAPH if graph else _lib.FLAG_STAGE_TIMING) | \
            (_lib.FLAG_STAGEWISE_REBIN if path == "stagewise" else 0)
        check(lib.gs3d_set_flags(ctx, flags))
        check(lib.gs3d_set_schedule(ctx, schedule))
        for _ in range(3):  # size the key buffers for this path's batch
            run_step(path)
            rc = lib.gs3d_synchronize(ctx)
            if rc != _lib.ERR_CAPACITY:
                check(rc)
                break
        for _ in range(args.warmup):
            run_step(path)
        check(lib.gs3d_synchronize(ctx))
        check(lib.gs3d_read_stage_times(ctx, None, None))  # reset
        start, stop = (torch.cuda.Event(enable_timing=True) for _ in range(2))
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        with ClockSampler(dev) as clocks:
            start.record(stream)
            for _ in range(args.steps):
                run_step(path)
            stop.record(stream)
            torch.cuda.synchronize()
        check(lib.gs3d_synchronize(ctx))
        ms = (C.c_double * 7)()
        cnt = (C.c_uint32 * 7)()
        check(lib.gs3d_read_stage_times(ctx, ms, cnt))
        check(lib.gs3d_set_flags(ctx, 0))
        check(lib.gs3d_set_schedule(ctx, _lib.SCHEDULE_ROW_MAJOR))
        total = max_over_ranks(start.elapsed_time(stop), world)
        views = args.steps * len(cam_structs)
        per_stage = {name: (ms[i] / views, cnt[i] / views) for i, name in
                     enumerate(_lib.STAGE_NAMES) if cnt[i]}  # per view
        return total, per_stage, clocks.summary()

    views = args.steps * len(cam_structs)
    # headline: batched, autotuned, CUDA graph replays, under each raster
    # order (the same image); the headline value is the fastest order's
    orders = [("row_major", _lib.SCHEDULE_ROW_MAJOR), ("key_count", _lib.SCHEDULE_KEY_COUNT)]
    if batched_schedule == _lib.SCHEDULE_LEARNED:
        orders.append(("learned", _lib.SCHEDULE_LEARNED))
    graph_runs = {}
    for name, sc in orders:
        ms_, _, clk = timed("batched", sc, graph=True)
        graph_runs[name] = (ms_, clk, sc)
    best_order = min(graph_runs, key=lambda k: graph_runs[k][0])
    batched_ms, clocks, best_sched = graph_runs[best_order]
    # the same path, each batch bracketed by its own events: the median over
    # steps x batches samples (the reference's timing protocol)
    check(lib.gs3d_set_flags(ctx, _lib.FLAG_CUDA_GRAPH))
    check(lib.gs3d_set_schedule(ctx, best_sched))
    run_step("batched")
    check(lib.gs3d_synchronize(ctx))
    marks = []
    for _ in range(max(args.steps, 3)):
        for arr in batches:
            ev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            ev[0].record(stream)
            check(lib.gs3d_rebin_batch(ctx, C.cast(arr, C.c_void_p), len(arr)))
            ev[1].record(stream)
            marks.append((ev, len(arr)))
    check(lib.gs3d_synchronize(ctx))
    torch.cuda.synchronize()
    per_view_ms = sorted(a.elapsed_time(b) / n for (a, b), n in marks)
    batch_median = {"ms_per_view": round(statistics.median(per_view_ms), 4),
                    "views_per_s": round(1e3 / statistics.median(per_view_ms), 1),
                    "samples": len(per_view_ms)}
    check(lib.gs3d_set_flags(ctx, 0))
    eager_ms, batched_stages, _ = timed("batched", best_sched)  # per-stage events
    # each work order on the tuned batched path (same image): graph-replay
    # views/s and the raster's eager per-stage time
    sched_batched = {}
    for name, sc in orders:
        ms_, st_, _ = timed("batched", sc)
        sched_batched[name] = {"raster_ms": round(st_["rasterize-tiles"][0], 4),
                               "views_per_s": round(views * world / (graph_runs[name][0] * 1e-3),
                                                    1)}

    # ---- e2e: the public batched entry point with host view tables in and
    # pinned host images out, every batch, under the same tuning ----
    img_bytes = WIDTH * HEIGHT * 8
    batch_bytes = img_bytes * B
    pinned = torch.empty(batch_bytes * 2, dtype=torch.uint8, pin_memory=True)
    check(lib.gs3d_set_flags(ctx, _lib.FLAG_CUDA_GRAPH))
    check(lib.gs3d_set_schedule(ctx, best_sched))
    for _ in range(2):  # warm-up: graph capture, and first copies into both pinned slots
        for bi, arr in enumerate(batches):
            check(lib.gs3d_rebin_batch(ctx, C.cast(arr, C.c_void_p), len(arr)))
            check(lib.gs3d_copy_buffer_async(
                ctx, 14, C.c_void_p(pinned.data_ptr() + (bi % 2) * batch_bytes),
                img_bytes * len(arr)))
    check(lib.gs3d_synchronize(ctx))
    if world > 1:
        torch.distributed.barrier()
    t0 = time.perf_counter()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for k in range(args.steps):
        for bi, arr in enumerate(batches):
            for i in range(len(arr)):  # host view table built per batch
                arr[i].camera = camera_struct(cams[bi * B + i])
            check(lib.gs3d_rebin_batch(ctx, C.cast(arr, C.c_void_p), len(arr)))
            check(lib.gs3d_copy_buffer_async(
                ctx, 14, C.c_void_p(pinned.data_ptr() + (bi % 2) * batch_bytes),
                img_bytes * len(arr)))
    e1.record(stream)
    check(lib.gs3d_synchronize(ctx))
    e2e_wall = max_over_ranks(time.perf_counter() - t0, world)
    e2e_ms = max_over_ranks(e0.elapsed_time(e1), world)
    check(lib.gs3d_set_flags(ctx, 0))

    # ---- reference tuning (16x16 tiles, 8-bit digits, one splat per pixel
    # per raster batch): single-view fused, the plain stage-wise path and the
    # raster under each work order ----
    set_tuning(TILE, 8, 0)
    sched16, model16 = install_cost_model(lib, ctx, TILE)
    fused_ms, fused_stages, _ = timed("fused", _lib.SCHEDULE_ROW_MAJOR)
    stagewise_ms, stagewise_stages, _ = timed("stagewise", _lib.SCHEDULE_ROW_MAJOR)
    sched_raster = {}
    for name, sc in (("row_major", _lib.SCHEDULE_ROW_MAJOR), ("key_count", _lib.SCHEDULE_KEY_COUNT),
                     ("learned", sched16)):
        ms_, st_, _ = timed("fused", sc)
        sched_raster[name] = {"raster_ms": round(st_["rasterize-tiles"][0], 4),
                              "views_per_s": round(views * world / (ms_ * 1e-3), 1)}

    # the small benchmark scene (100k splats, SH 0, 1280x720, 16x16 tiles):
    # single-view fused rebins replayed as a graph, beside the CPU C0 figures
    c0_data, c0_u, (c0_w, c0_h) = c0_workload()
    check(lib.gs3d_set_splats(ctx, c0_data.splatCount, ptr(c0_data.positions),
                              ptr(c0_data.scales), ptr(c0_data.rotations),
                              ptr(c0_data.colors), None, 0, 0))
    c0_cam = camera_struct(c0_u)
    check(lib.gs3d_set_flags(ctx, _lib.FLAG_CUDA_GRAPH))
    check(lib.gs3d_set_schedule(ctx, _lib.SCHEDULE_ROW_MAJOR))
    for _ in range(3):
        rc = lib.gs3d_rebin(ctx, C.byref(c0_cam), c0_w, c0_h)
        rc = lib.gs3d_synchronize(ctx) if rc == 0 else rc
        if rc != _lib.ERR_CAPACITY:
            check(rc)
            break
    c0_reps = 200
    for _ in range(20):
        check(lib.gs3d_rebin(ctx, C.byref(c0_cam), c0_w, c0_h))
    check(lib.gs3d_synchronize(ctx))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(c0_reps):
        check(lib.gs3d_rebin(ctx, C.byref(c0_cam), c0_w, c0_h))
    e1.record(stream)
    check(lib.gs3d_synchronize(ctx))
    torch.cuda.synchronize()
    c0_gpu = round(c0_reps / (e0.elapsed_time(e1) * 1e-3), 1)
    check(lib.gs3d_set_flags(ctx, 0))
    lib.gs3d_destroy(ctx)

    tiles16 = -(-WIDTH // TILE) * -(-HEIGHT // TILE)
    tile_passes16 = ((tiles16 - 1).bit_length() + 7) // 8
    tiles_t = -(-WIDTH // tuned.tile_w) * -(-HEIGHT // tuned.tile_h)
    mean_R = float(np.mean(refs))
    peak, peak_kind = peaks()

    def roof(stages, fused, R, tiles, passes, tile_px, views_per_scene=1):
        algo = algorithmic_bytes(N_SPLATS, R, tiles, passes, 45, fused, views_per_scene)
        out = {}
        for name, (ms, n) in stages.items():
            gbs = algo[name] / (ms * 1e-3) / 1e9
            out[name] = {"ms": round(ms, 4), "algo_bytes": int(algo[name]), "gbs": round(gbs, 1),
                         "frac_hbm": round(gbs / peak, 3)}
        return out

    batched_roof = roof(batched_stages, True, tuned_R, tiles_t, tuned_passes, tuned.tile_w, B)
    hbm = [s for s in batched_roof if s != "rasterize-tiles"]
    dom = max(hbm, key=lambda s: batched_roof[s]["ms"])
    learned_on = batched_schedule == _lib.SCHEDULE_LEARNED
    # kernels of one batched rebin: preprocess, depth sort (histogram + 4 passes), scan, emit,
    # tile-digit passes, identify, schedule (features + MLP + keys + split count + histogram
    # + 2 passes + gate for the learned order; keys + split count + histogram + 2 passes for
    # key counts; none for row-major), raster
    sched_kernels = {_lib.SCHEDULE_ROW_MAJOR: 0, _lib.SCHEDULE_KEY_COUNT: 5,
                     _lib.SCHEDULE_LEARNED: 8}[best_sched]
    launches_per_batch = 1 + 5 + 1 + 1 + tuned_passes + 1 + sched_kernels + 1
    return {
        "value": views * world / (batched_ms * 1e-3), "ms_per_step": batched_ms / args.steps,
        "views": views, "per_stage": batched_roof, "dominant": dom, "peak": peak,
        "fused_value": views * world / (fused_ms * 1e-3),
        "fused_stages": roof(fused_stages, True, mean_R, tiles16, tile_passes16, TILE),
        "batched_eager_value": views * world / (eager_ms * 1e-3),
        "peak_kind": peak_kind, "mean_refs": mean_R, "tuned_refs": tuned_R,
        "clocks": clocks,
        "stagewise_value": views * world / (stagewise_ms * 1e-3),
        "stagewise_stages": roof(stagewise_stages, False, mean_R, tiles16, tile_passes16, TILE),
        # the image copy-outs run on the library's copy stream: the host clock
        # around the loop, which ends in gs3d_synchronize, covers all of them
        "e2e_value": views * world / e2e_wall, "e2e_stream_value": views * world / (e2e_ms * 1e-3),
        "h2d": 416 * len(cam_structs), "d2h": img_bytes * len(cam_structs),
        "launches_per_step": launches_per_batch * len(batches),
        "schedules": sched_raster, "schedules_batched": sched_batched,
        "learned_active": learned_on, "best_order": best_order,
        "cost_model": {k: round(v, 4) for k, v in (tuned_model or {}).items()},
        "tuning": {"tile": [tuned.tile_w, tuned.tile_h], "digit_bits": tuned.digit_bits,
                   "raster_batch": tuned.raster_batch, "candidates": tune_table},
        "tile_passes_batched": tuned_passes,
        "traffic": dominant_traffic(dom, (tuned.tile_w, tuned.tile_h), tuned_R * B, N_SPLATS * B,
                                    N_SPLATS),
        "launch_units": {"refs": int(tuned_R * B), "splat_views": N_SPLATS * B},
        "batch_median": batch_median, "c0_gpu_views_per_s": c0_gpu,
        # bytes the sort moves per view: the reference's eight 8-bit passes over
        # 12-byte refs at its 16x16 tiles (one histogram read + 8 scatters)
        # against this path's 4 depth passes over splats + its tile-digit passes
        "sort_bytes_per_view": {
            "reference_8_pass_16x16": int(8 * mean_R + 8 * 24 * mean_R),
            "this_path": int(4 * N_SPLATS + 4 * 16 * N_SPLATS + tuned_passes * 24 * tuned_R)},
    }


SIZES_C2 = [(640, 360), (1280, 720), (1920, 1080), (2560, 1440), (3840, 2160)]


def c2_workload():
    """The batched configuration: 4 scenes of 0.5M, 1M, 3M and 6M splats
    (cluster distribution, seeds 1-4, SH 3) and one batch of 32 views at sizes
    drawn from 640x360 ... 3840x2160, random poses at radius 8-16."""
    from gs3d import scenes
    scs = [scenes.scene_clusters(n, seed=s, sh_degree=3)
           for n, s in ((500_000, 1), (1_000_000, 2), (3_000_000, 3), (6_000_000, 4))]
    rng = np.random.default_rng(11)
    eyes = scenes.random_eyes(32, 8.0, 16.0, seed=11)
    views = []
    for i in range(32):
        w, h = SIZES_C2[int(rng.integers(len(SIZES_C2)))]
        views.append((i % 4, scenes.camera_at(eyes[i], w, h).getUniformData(w, h), w, h))
    return scs, [views]


def c4_workload():
    """The skewed stress configuration: 10M splats (16 dense clusters + 20%
    background, heavy-tailed scales, SH 3), 8 close-up and 8 wide 3840x2160
    views; batches of 2 close-ups (about 1.1e9 refs each at 32x32 tiles) and
    one batch of the 8 wide views, within one rebin's 2^32 refs."""
    from gs3d import scenes
    data = scenes.scene_skewed(10_000_000, seed=0, sh_degree=3)
    W, H = 3840, 2160
    close = scenes.random_eyes(8, 3.0, 5.0, seed=21)
    wide = scenes.random_eyes(8, 28.0, 34.0, seed=22)
    cv = [(0, scenes.camera_at(e, W, H).getUniformData(W, H), W, H) for e in close]
    wv = [(0, scenes.camera_at(e, W, H).getUniformData(W, H), W, H) for e in wide]
    return [data], [cv[0:2], cv[2:4], cv[4:6], cv[6:8], wv]


def tail_workload():
    """A tail-bound workload: scene_opacity_mix (1.5M opaque splats in 12
    clusters beside 0.4M translucent ones in 6 dense clusters, SH 0), 1080p,
    16x16 tiles; the cost model is trained on 120 random poses and 16 held-out
    poses are rendered, as two batches of 8."""
    from gs3d import scenes
    data = scenes.scene_opacity_mix(1_500_000, 400_000, seed=3)
    W, H = 1920, 1080
    us = [scenes.camera_at(e, W, H).getUniformData(W, H)
          for e in scenes.random_eyes(136, 9.0, 16.0, seed=9)]
    views = [(0, u, W, H) for u in us[120:]]
    return [data], [views[:8], views[8:]], (us[:120], W, H)


def run_extra_config(name, scenes_data, batches, tuning, steps, warmup, train=None,
                     single_orders=False):
    """views/s of one configuration under the batched path (CUDA-graph replay)
    with each raster order, and of the plain single-view path (fused rebin,
    16x16 tiles, row-major; every order with single_orders), with per-stage
    times and the learned order's gate state.  Every step renders every view
    once.  train = (uniforms, width, height): the cost model is trained on
    those poses of the first scene by the library's kernels and installed,
    instead of the committed checkpoint."""
    import torch

    from gs3d import _lib
    from gs3d.camera import camera_struct

    lib = _lib.load()
    stream = torch.cuda.Stream()
    ctx = C.c_void_p()
    cfg = _lib.Config_t(int(os.environ.get("LOCAL_RANK", 0)), 16, 16, 16,
                        C.c_void_p(stream.cuda_stream), 0)
    if lib.gs3d_create(C.byref(ctx), C.byref(cfg)) != 0:
        raise RuntimeError("gs3d_create failed")

    def check(rc):
        if rc != 0:
            raise RuntimeError(f"{name}: " + lib.gs3d_last_error(ctx).decode())

    ptr = lambda a: None if a is None else a.ctypes.data_as(C.c_void_p)  # noqa: E731
    for i, d in enumerate(scenes_data):
        args = (d.splatCount, ptr(d.positions), ptr(d.scales), ptr(d.rotations), ptr(d.colors),
                ptr(d.sphericalHarmonics), d.sphericalHarmonicsDegree, 0)
        if i == 0:
            check(lib.gs3d_set_splats(ctx, *args))
        else:
            sid = C.c_uint32()
            check(lib.gs3d_add_scene(ctx, *args, C.byref(sid)))
    arrs = []
    for vs in batches:
        arr = (_lib.View_t * len(vs))()
        for i, (sid, u, w, h) in enumerate(vs):
            arr[i].camera = camera_struct(u)
            arr[i].scene, arr[i].width, arr[i].height = sid, w, h
        arrs.append(arr)
    n_views = sum(len(a) for a in arrs)
    if tuning is None:  # autotune on the first batch
        out = (_lib.TuneResult_t * 64)()
        n = C.c_uint32()
        check(lib.gs3d_autotune(ctx, C.cast(arrs[0], C.c_void_p), len(arrs[0]), 1, out, 64,
                                C.byref(n)))
    else:
        check(lib.gs3d_set_tuning(ctx, C.byref(_lib.Tuning_t(*tuning))))
    tuned = _lib.Tuning_t()
    check(lib.gs3d_get_tuning(ctx, C.byref(tuned)))

    def step(single):
        for arr in arrs:
            if single:
                for i in range(len(arr)):
                    at = C.c_void_p(C.addressof(arr) + i * C.sizeof(_lib.View_t))
                    check(lib.gs3d_rebin_batch(ctx, at, 1))
            else:
                check(lib.gs3d_rebin_batch(ctx, C.cast(arr, C.c_void_p), len(arr)))

    def settle(single):  # size the key buffers for this path
        for _ in range(3):
            step(single)
            rc = lib.gs3d_synchronize(ctx)
            if rc != _lib.ERR_CAPACITY:
                check(rc)
                return

    def timed(single, schedule, graph):
        check(lib.gs3d_set_schedule(ctx, schedule))
        check(lib.gs3d_set_flags(ctx, _lib.FLAG_CUDA_GRAPH if graph else 0))
        settle(single)
        for _ in range(warmup):
            step(single)
        check(lib.gs3d_synchronize(ctx))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            step(single)
        e1.record(stream)
        check(lib.gs3d_synchronize(ctx))
        torch.cuda.synchronize()
        views_s = steps * n_views / (e0.elapsed_time(e1) * 1e-3)
        # one eager step with stage events: per-view stage times
        check(lib.gs3d_set_flags(ctx, _lib.FLAG_STAGE_TIMING))
        check(lib.gs3d_read_stage_times(ctx, None, None))
        step(single)
        check(lib.gs3d_synchronize(ctx))
        ms = (C.c_double * 7)()
        cnt = (C.c_uint32 * 7)()
        check(lib.gs3d_read_stage_times(ctx, ms, cnt))
        st = _lib.ScheduleStatus_t()
        check(lib.gs3d_get_schedule_status(ctx, C.byref(st)))
        check(lib.gs3d_set_flags(ctx, 0))
        return {"views_per_s": round(views_s, 2),
                "stage_ms_per_view": {nm: round(ms[i] / n_views, 4)
                                      for i, nm in enumerate(_lib.STAGE_NAMES) if cnt[i]},
                "split_tiles_last_rebin": st.split_tiles,
                "gate": {"active": ["row_major", "key_count", "learned"][st.active],
                         "mae_log": round(st.mae_log, 4), "bound": st.bound,
                         "frames": st.frames, "fallbacks": st.fallbacks}
                if schedule == _lib.SCHEDULE_LEARNED else None}

    res = {"views": n_views, "batches": [len(a) for a in arrs],
           "tuning": {"tile": [tuned.tile_w, tuned.tile_h], "digit_bits": tuned.digit_bits,
                      "raster_batch": tuned.raster_batch}}
    if train is None:
        learned_sched, model = install_cost_model(lib, ctx, tuned.tile_w, tuned.tile_h)
        res["cost_model_checkpoint"] = "trained on the 3M-splat 1080p workload" if model else None
    else:
        from gs3d import learned
        tu, tw, th = train
        x, t, k = learned.collect(lib, ctx, tu, tw, th)
        n_fit = len(tu) * 5 // 6
        fit = learned.train(lib, x[:n_fit].reshape(-1, 16), t[:n_fit].reshape(-1), steps=2000,
                            batch=65536, lr=5e-3)
        res["cost_model_heldout"] = {k_: round(float(v), 4) for k_, v in
                                     learned.evaluate(lib, fit, x[n_fit:], t[n_fit:],
                                                      k[n_fit:]).items()}
        f32 = lambda a: np.ascontiguousarray(a, np.float32)  # noqa: E731
        check(lib.gs3d_set_cost_model(ctx, ptr(f32(fit.params)), ptr(f32(fit.mean)),
                                      ptr(f32(fit.std))))
        check(lib.gs3d_set_schedule_gate(ctx, C.c_float(learned.ERROR_BOUND)))
        learned_sched = _lib.SCHEDULE_LEARNED
        res["cost_model_checkpoint"] = (f"trained in this run on {len(tu)} poses of the "
                                        "workload (library kernels)")
        del x, t, k
    # CUDA-graph replay where every batch has one layout (a graph is captured
    # per layout; alternating layouts would re-capture every call)
    graph = len(arrs) == 1
    res["batched_path"] = "CUDA-graph replay" if graph else "eager launches"
    for label, sc in (("batched_row_major", _lib.SCHEDULE_ROW_MAJOR),
                      ("batched_key_count", _lib.SCHEDULE_KEY_COUNT),
                      ("batched_learned", learned_sched)):
        if label == "batched_learned" and sc != _lib.SCHEDULE_LEARNED:
            res[label] = None
            continue
        res[label] = timed(False, sc, graph)
    check(lib.gs3d_set_tuning(ctx, C.byref(_lib.Tuning_t(16, 16, 8, 0))))
    res["single_view_fused_16x16_row_major"] = timed(True, _lib.SCHEDULE_ROW_MAJOR, False)
    if single_orders:
        res["single_view_fused_16x16_key_count"] = timed(True, _lib.SCHEDULE_KEY_COUNT, False)
        res["single_view_fused_16x16_learned"] = timed(True, learned_sched, False)
    lib.gs3d_destroy(ctx)
    del stream
    torch.cuda.empty_cache()
    return res


def run_extras(args):
    """The batched and skewed-stress configurations beside the headline."""
    scs, batches = c2_workload()
    c2 = run_extra_config("batched (4 scenes, 32 mixed views)", scs, batches, None,
                          args.extra_steps, 1)
    del scs
    scs, batches = c4_workload()
    c4 = run_extra_config("skewed stress (10M, 16 4K views)", scs, batches, (32, 32, 8, 512),
                          args.extra_steps, 1)
    del scs
    scs, batches, train = tail_workload()
    tail = run_extra_config("tail-bound (opacity mix, 1080p)", scs, batches, (16, 16, 8, 0),
                            args.extra_steps, 1, train=train, single_orders=True)
    return {"batched_4_scenes_32_mixed_views": c2, "skewed_10M_16_views_4k": c4,
            "tail_bound_opacity_mix_1080p_16x16": tail}


def profile_run(args):
    """Renders the workload through the batched path for a profiler: each
    step = ceil(views / batch) launch sequences; nothing is timed."""
    from gs3d import _lib
    from gs3d.camera import camera_struct
    lib = _lib.load()
    ctx = C.c_void_p()
    if lib.gs3d_create(C.byref(ctx), None) != 0:
        raise RuntimeError("gs3d_create failed")
    data, cams = make_workload(args.views)
    ptr = lambda a: a.ctypes.data_as(C.c_void_p)  # noqa: E731
    assert lib.gs3d_set_splats(ctx, data.splatCount, ptr(data.positions), ptr(data.scales),
                               ptr(data.rotations), ptr(data.colors),
                               ptr(data.sphericalHarmonics), 3, 0) == 0
    tile_s, digit_s, batch_s = args.tuning.split(",")
    tile_w, tile_h = (int(x) for x in tile_s.split("x")) if "x" in tile_s else (int(tile_s),) * 2
    digit_bits, raster_batch = int(digit_s), int(batch_s)
    assert lib.gs3d_set_tuning(ctx, C.byref(_lib.Tuning_t(tile_w, tile_h, digit_bits,
                                                           raster_batch))) == 0
    if args.order == "learned":
        schedule, _ = install_cost_model(lib, ctx, tile_w, tile_h)
    else:
        schedule = {"row_major": _lib.SCHEDULE_ROW_MAJOR,
                    "key_count": _lib.SCHEDULE_KEY_COUNT}[args.order]
    assert lib.gs3d_set_schedule(ctx, schedule) == 0
    B = args.batch
    for step in range(args.profile):
        for b0 in range(0, len(cams), B):
            arr = (_lib.View_t * min(B, len(cams) - b0))()
            for i in range(len(arr)):
                arr[i].camera = camera_struct(cams[b0 + i])
                arr[i].width, arr[i].height = WIDTH, HEIGHT
            for _ in range(3):
                assert lib.gs3d_rebin_batch(ctx, C.cast(arr, C.c_void_p), len(arr)) == 0
                rc = lib.gs3d_synchronize(ctx)
                if rc != _lib.ERR_CAPACITY:
                    break
            assert rc == 0, lib.gs3d_last_error(ctx)
    lib.gs3d_destroy(ctx)


def cpu_view_seconds(n_views=1, threads=0):
    """Times the oracle's whole rebin on one full-size view (bounded sample)."""
    from oracle import Oracle
    o = Oracle()
    data, cams = make_workload(n_views)
    t = o.max_threads() if threads == 0 else threads
    times = []
    for u in cams:
        t0 = time.perf_counter()
        o.rebin(u, WIDTH, HEIGHT, TILE, TILE, data.positions, data.scales, data.rotations,
                data.colors, data.sphericalHarmonics, 3, threads=t,
                key_capacity=N_SPLATS * 16)
        times.append(time.perf_counter() - t0)
    return times, t


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--views", type=int, default=64)
    ap.add_argument("--batch", type=int, default=8, help="views per batched rebin")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the batched and skewed-stress configurations")
    ap.add_argument("--extra-steps", type=int, default=3,
                    help="timed steps of each extra configuration path")
    ap.add_argument("--profile", type=int, default=0, metavar="STEPS",
                    help="profiling run: render STEPS batched steps of --views views and exit "
                         "(no timing, no JSON)")
    ap.add_argument("--tuning", default=f"{TILE},8,0", metavar="TILE,DIGIT_BITS,RASTER_BATCH",
                    help="profiling run: the tuning to render with, TILE square or WxH "
                         "(the bench autotunes)")
    ap.add_argument("--order", default="key_count", choices=["row_major", "key_count", "learned"],
                    help="profiling run: the raster order")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))

    if args.impl == "reference":
        if rank != 0:
            return
        times, threads = cpu_view_seconds(args.warmup + args.steps)
        timed = times[args.warmup:]
        v = len(timed) / sum(timed)
        sample = f"one full 3M-splat SH3 1080p view per step ({len(timed)} views of the orbit)"
        print(json.dumps({
            "impl": "reference", "metric": METRIC, "value": v, "unit": "views/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * sum(timed) / len(timed), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "views_per_step": 1, "threads": threads},
            "cpu_baseline": {"value": v, "unit": "views/s", "cores": threads, "kind": "port",
                             "sample": sample},
            "e2e": {"value": v, "unit": "views/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
        }))
        return

    if args.profile:
        profile_run(args)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res = run_ours(args, rank, world)
    extras = None
    if rank == 0 and world == 1 and not args.no_extras:
        extras = run_extras(args)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        times, threads = cpu_view_seconds(1)
        from oracle import Oracle
        cpu = {"value": 1.0 / times[0], "unit": "views/s", "cores": threads, "kind": "port",
               "sample": "one full 3M-splat SH3 1080p view (orbit pose 0), oracle rebin",
               "c0_100k_720p": {"threads_1": cpu_c0_stages(1),
                                f"threads_{Oracle().max_threads()}":
                                    cpu_c0_stages(Oracle().max_threads()),
                                "gpu_single_view_fused_views_per_s": res["c0_gpu_views_per_s"]}}
    raster_roof = None
    if rank == 0:
        # the raster is issue-bound: its pipe use (ncu) and the reference
        # loop's work on view 0 against the headline path's raster time
        rms = res["per_stage"]["rasterize-tiles"]["ms"]
        raster_roof = dict(RASTER_NCU, bound="issue (FMA/ALU/SFU pipes)", ms_per_view=rms)
        if not args.no_cpu_baseline:
            pairs = raster_work(0, TILE)
            raster_roof.update(
                pairs_per_view=pairs, pairs_view="orbit pose 0, 16x16 tiles, oracle count",
                blended_pairs_per_s=round(pairs["blended"] / (rms * 1e-3), 1),
                evaluated_pairs_per_s=round(pairs["evaluated"] / (rms * 1e-3), 1))
    if rank == 0:
        dom = res["per_stage"][res["dominant"]]
        out = {
            "metric": METRIC, "value": res["value"], "unit": "views/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": res["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic",
            "config": {"workload": WORKLOAD,
                       "path": f"batched fused rebin, {args.batch} views per launch sequence, "
                               "autotuned, replayed as a CUDA graph",
                       "tuning": res["tuning"],
                       "mean_refs_per_view_tuned": res["tuned_refs"],
                       "batched_without_graph_views_per_s": res["batched_eager_value"],
                       "views_per_step": args.views, "l2": "inputs larger than L2 (no flush)",
                       "mean_refs_per_view_16x16": res["mean_refs"],
                       "tile_digit_passes": res["tile_passes_batched"],
                       "single_view_fused_views_per_s": res["fused_value"],
                       "raster_schedule": res["best_order"] + " (the fastest of the orders "
                                          "measured below; every order renders the same "
                                          "image)",
                       "cost_model_installed": res["learned_active"],
                       "schedules_single_view": res["schedules"],
                       "schedules_batched_tuned": res["schedules_batched"],
                       "cost_model_heldout": res["cost_model"],
                       "plain_stagewise_views_per_s": res["stagewise_value"],
                       "batch_median": res["batch_median"],
                       "sort_bytes_per_view": res["sort_bytes_per_view"]},
            "roofline": {"bound": "hbm", "kernel": res["dominant"], "achieved": dom["gbs"],
                         "peak": res["peak"], "unit": "GB/s", "frac": dom["frac_hbm"],
                         "peak_kind": res["peak_kind"], "traffic": res["traffic"],
                         "traffic_per": "launch (one pass over one batch), ncu DRAM "
                                        "bytes of a 2-view capture scaled by units",
                         "launch_units": res["launch_units"]},
            "roofline_raster": raster_roof,
            "stages": res["per_stage"],
            "stages_single_view_fused": res["fused_stages"],
            "stages_plain_stagewise": res["stagewise_stages"],
            "cpu_baseline": cpu,
            "e2e": {"value": res["e2e_value"], "unit": "views/s",
                    "h2d_bytes_per_step": res["h2d"], "d2h_bytes_per_step": res["d2h"],
                    "clock": "host wall clock from the first view-table build to "
                             "gs3d_synchronize after the last image copy-out",
                    "rebin_stream_events_value": res["e2e_stream_value"]},
            "gpu_launches": res["launches_per_step"] * args.steps,
            "clocks": res["clocks"],
            "configs_extra": extras,
        }
        print(json.dumps(out))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
