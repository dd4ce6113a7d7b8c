"""Benchmark of the per-step render path (one JSON line on stdout).

Workload: the 256^3 training step — a sparse band around the union of 8
spheres, SH degree 3, 8 shells, 4 cameras at 800x800 (synthetic stand-in for
the reference's datasets). A step is tessellation of all shells + fused render
of all cameras + MSE + backward into the grid SDF and SH, through the
package's public API.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``value`` is the device time of one step (CUDA events on the launching
stream, inputs resident in HBM, L2 flushed between steps); ``e2e`` is the same
step with the inputs copied from pinned host memory and the loss copied back
inside the timed region. ``--impl reference`` times the CPU restatement of the
reference algorithm (the reference's Slang kernels cannot run here) on the
host cores.

With N > 1 (torchrun), every rank runs an independent replica of the step on
its own GPU (the path needs no exchange); the reported time is the maximum
over ranks.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

METRIC = "fwd+bwd step ms & HBM GB/s at 256³×8 shells×4×800²; serve p99 ms vs plain"
CONFIG_NAME = "mid"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=None,
                   help="timed steps (default: 200 on the GPU, 5 for the host-core reference arm)")
    p.add_argument("--warmup", type=int, default=None, help="warm-up steps (default: 5 on the GPU, 3 on the host)")
    p.add_argument("--impl", choices=("ours", "reference"), default="ours")
    p.add_argument("--config", default=CONFIG_NAME)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-cameras", action="store_true", help="skip the uneven-camera batching comparison")
    p.add_argument("--no-serving", action="store_true", help="skip the serving sweep")
    p.add_argument("--serve-requests", type=int, default=2000, help="requests per arrival rate of the serving sweep")
    p.add_argument("--no-subdivision", action="store_true", help="skip the subdivision step measurement")
    p.add_argument("--no-large", action="store_true", help="skip the large-configuration step in both modes")
    p.add_argument("--no-band", action="store_true", help="skip the band-matched variant of the step")
    p.add_argument("--tile", default=None, help="tile shape HxW for the step (default: autotuned)")
    p.add_argument("--no-reference-cub", action="store_true",
                   help="skip timing the reference's CUB scan and sort extensions")
    return p.parse_args()


def dist_setup(n):
    import torch
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    local = int(os.environ.get("LOCAL_RANK", 0))
    if world > 1:
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.proc = None
        self.gpu = gpu_index
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={gpu_index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in out.strip().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {
            "sm_mhz": statistics.median(sm) if sm else None,
            "sm_max_mhz": max(smax) if smax else None,
            "reasons": sorted(reasons),
            "samples": len(sm),
        }


def profiled_traffic(entry: str):
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    of an entry point's kernels from the ncu capture summarised in
    profiles/traffic.json, used only while the kernels' sources are the ones
    captured (their SHA-256 is recorded beside the figure)."""
    import hashlib

    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            table = json.load(f)
    except (OSError, ValueError):
        return None, "no capture"
    rec = table.get(entry)
    if not isinstance(rec, dict):
        return None, "no capture of this entry point"
    digest = hashlib.sha256()
    for name in rec.get("sources", []):
        with open(os.path.join(ROOT, "meshtryoshka_gb300", "csrc", name), "rb") as f:
            digest.update(f.read())
    if digest.hexdigest() != rec.get("sha256"):
        return None, "capture predates the current kernel sources"
    return rec.get("bytes_per_launch"), rec.get("capture")


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# CPU leg: the oracle (restatement of the reference algorithm) on host cores.
# ---------------------------------------------------------------------------
def cpu_step(w, tile_shape=(16, 16)):
    """One whole training step of the workload on the host cores with the
    oracle (the restatement of the reference's kernels): tessellation of every
    shell, fused render of every camera, the MSE loss through the background
    blend and the clip, the compositing backward, the SH backward and the
    vertex-interpolation backward into the grid SDF and SH. Returns
    (seconds, sizes)."""
    import numpy as np

    from oracle import oracle

    vox = w.voxels
    np_vox = [t.detach().cpu().numpy() for t in (vox.vertices, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                                 vox.indices)]
    sdf = w.grid_sdf.detach().cpu().numpy()
    sh = w.grid_sh.detach().cpu().numpy()
    ls = w.level_sets.cpu().numpy()
    ext = w.extrinsics.cpu().numpy()
    intr = w.intrinsics.cpu().numpy()
    bg = w.background.cpu().numpy()
    target = w.target.detach().cpu().numpy()
    b = ext.shape[0]
    t0 = time.perf_counter()
    tri = oracle.tessellate_voxels(sdf, np_vox[0], sh, np_vox[1], np_vox[2], np_vox[3], np_vox[4], ls)
    verts = (np.float32(2.0) * tri.vertices - np.float32(1.0)).astype(np.float32)
    r = oracle.render_fused(ext, intr, w.image_shape, verts, tri.faces, tri.face_boundaries, tri.signed_distances,
                            tri.spherical_harmonics, w.sh_degree, float(w.sharpness), bg, tile_shape=tile_shape)
    bgc = bg[None, :, None, None]
    x = r.raw[:, :3] + r.raw[:, 3:4] * bgc
    grad = np.where((x >= 0) & (x <= 1), (2.0 / target.size) * (r.image - target), 0.0).astype(np.float32)
    graw = np.zeros_like(r.raw)
    graw[:, :3] = grad
    graw[:, 3] = (grad * bgc).sum(1)
    gcol, gsdf, _ = oracle.intersect_and_composite_backward(
        r.xy, r.colors, tri.signed_distances, tri.faces, float(w.sharpness), r.sorted_keys, r.sorted_tri,
        r.tile_boundaries.reshape(b, -1, 2), tri.face_boundaries.shape[0], tile_shape, w.image_shape,
        oracle.fused_key_defines(), r.raw, graw)
    gsh = oracle.evaluate_spherical_harmonics_backward(verts, tri.spherical_harmonics.shape, ext, w.sh_degree,
                                                       r.colors, gcol)
    oracle.create_triangle_vertices_backward(sdf, sh.shape, np_vox[2], ls, tri.vertex_offsets, None, gsdf, gsh)
    seconds = time.perf_counter() - t0
    h, wd = w.image_shape
    sizes = {"G": int(np_vox[2].shape[1]), "Nv": int(np_vox[3].shape[1]), "V": int(tri.vertices.shape[0]),
             "F": int(tri.faces.shape[0]), "P": int(b * h * wd)}
    return seconds, sizes


def workload_config(w, sizes: dict) -> dict:
    """The `config` object of both arms' bench lines (identical for the same
    workload): what is computed, on which sizes, and how L2 is handled."""
    h, wd = w.image_shape
    cfg = w.config
    return {
        "workload": f"{cfg.name}: {cfg.resolution}^3 band around {cfg.num_spheres} spheres, SH deg {cfg.sh_degree}, "
                    f"{len(cfg.level_sets)} shells, {w.extrinsics.shape[0]}x{h}x{wd}, fused fwd+bwd training step",
        "sizes": {k: int(sizes[k]) for k in ("G", "Nv", "V", "F", "P")},
        "l2": "GPU arm: flushed by a 256 MB write between timed steps; host arm: inputs far larger than the "
              "host caches",
    }


def cpu_threads():
    return int(os.environ.get("OMP_NUM_THREADS") or os.cpu_count() or 1)


def host_workload(name: str):
    """The benchmark scene built on the host with the oracle (same seeds and
    arrays as pipeline.build_workload, whose voxels come from the GPU path),
    so that the reference arm needs neither a GPU nor this library's kernels."""
    import numpy as np
    import torch

    from meshtryoshka_gb300 import pipeline, synthetic
    from meshtryoshka_gb300 import triangle_extraction as te
    from oracle import oracle

    cfg = synthetic.CONFIGS[name]
    occ = synthetic.make_occupancy(cfg, "cpu").numpy()
    v = oracle.extract_voxels(occ)
    voxels = te.Voxels(*(torch.from_numpy(np.ascontiguousarray(a)) for a in
                         (v.vertices, v.neighbors, v.lower_corners, v.upper_corners, v.indices)), v.grid_shape)
    sdf = synthetic.corner_sdf(cfg, voxels.vertices)
    sh = synthetic.corner_sh(cfg, voxels.vertices.shape[0], "cpu")
    cams = synthetic.make_cameras(cfg)
    shapes = [tuple(x) for x in cams.image_shapes]
    if len(set(shapes)) != 1:
        raise ValueError("the reference arm takes one image size per step")
    h, w = shapes[0]
    return pipeline.Workload(
        config=cfg, voxels=voxels, grid_sdf=sdf, grid_sh=sh, level_sets=synthetic.level_sets(cfg, "cpu"),
        extrinsics=torch.from_numpy(cams.extrinsics), intrinsics=torch.from_numpy(cams.intrinsics),
        image_shape=(h, w), target=synthetic.make_target(cfg.num_cameras, h, w, "cpu"),
        sharpness=torch.tensor(cfg.sharpness, dtype=torch.float32),
        background=torch.zeros(3, dtype=torch.float32))


def run_reference(args, rank, world):
    """CPU restatement of the reference path on the host cores (rank 0 only;
    under torchrun the other ranks return without work). Every timed step is
    one whole training step of the workload: all cameras, forward and
    backward."""
    if rank != 0:
        return
    w = host_workload(args.config)
    times = []
    sizes = None
    for i in range(args.warmup + args.steps):
        seconds, sizes = cpu_step(w)
        if i >= args.warmup:
            times.append(seconds)
    ms = 1000.0 * statistics.mean(times)
    b = w.extrinsics.shape[0]
    line = {
        "metric": METRIC, "value": ms, "unit": "ms", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(w, sizes),
        "impl": "reference",
        "parallelism": f"host threads ({cpu_threads()})",
        "tile_shape": [16, 16],
        "timed_region_s": sum(times),
        "cpu_baseline": {"value": ms, "unit": "ms", "cores": cpu_threads(), "kind": "port",
                         "sample": f"each step: the whole training step on the host (tessellation of every shell, "
                                   f"fused render of all {b} cameras, MSE through blend and clip, compositing, SH "
                                   f"and vertex-interpolation backward into the grid)"},
        "e2e": {"value": ms, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------
def run_ours(args, rank, world, local):
    import torch

    from meshtryoshka_gb300 import _native, autotune, graph, pipeline

    device = torch.device("cuda", local)
    torch.manual_seed(0)
    w = pipeline.build_workload(args.config, device)
    stream = torch.cuda.current_stream(device)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=device)  # > L2 (129 MB)
    # The tile shape only splits the work (every pixel walks the same
    # triangles in the same order, so images and gradients are the same):
    # the step uses the fastest of a few shapes, timed as captured steps.
    if args.tile:
        tile = tuple(int(x) for x in args.tile.lower().split("x"))
        w.tile_shape = tile
        tile_ms = {}
    else:
        tile, tile_ms = autotune.tune_tile_shape(w, repeats=5)

    def eager_step():
        w.grid_sdf.grad = None
        w.grid_sh.grad = None
        loss, stats = pipeline.forward(w)
        loss.backward()
        return loss, stats

    for _ in range(max(args.warmup, 3)):
        eager_step()
    torch.cuda.synchronize(device)

    # Eager steps (the reference's form: sizes read back to the host).
    eager_steps = min(args.steps, 50)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(eager_steps)]
    for i in range(eager_steps):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        loss, stats = eager_step()
        ev[i][1].record(stream)
    torch.cuda.synchronize(device)
    eager_ms = statistics.mean(a.elapsed_time(b) for a, b in ev)

    # The training step as one CUDA graph (capacity-sized buffers, no host
    # reads); the timed region. L2 flushed between steps, outside the events.
    step = graph.CapturedTrainingStep(w, input_sets=2)  # set 1: the e2e pipeline's second input buffer
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize(device)
    if not step.check():
        for _ in range(max(args.warmup, 3)):
            step()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier(world)
    torch.cuda.synchronize(device)
    clocks = ClockSampler(local) if rank == 0 else None
    wall0 = time.perf_counter()
    for i in range(args.steps):
        flush.fill_(float(i))
        torch.cuda.nvtx.range_push("step")
        ev[i][0].record(stream)
        step()
        ev[i][1].record(stream)
        torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize(device)
    wall = time.perf_counter() - wall0
    barrier(world)
    clock_info = clocks.stop() if clocks else None
    fits = step.check()
    step_ms = [a.elapsed_time(b) for a, b in ev]

    # The captured step's function run outside the graph with every library
    # entry point timed by CUDA events on its launching stream: the timed
    # step's per-kernel breakdown and the roofline's launch time.
    with _native.record_launches(timed=True) as rec:
        for i in range(eager_steps):
            with torch.cuda.stream(step.stream):
                flush.fill_(float(i))
            step.run_uncaptured()
    torch.cuda.synchronize(device)
    per_call = rec.times_ms()
    ms = max_over_ranks(statistics.mean(step_ms), world)
    launches_per_step = step.launches_per_replay

    # End to end through the public API: every step copies its batch (target
    # images and cameras) from pinned host memory into the inputs the step
    # reads, replays the step and reads its loss back, as a training loop
    # with an input pipeline does (the parameters stay resident on the
    # device, where an optimizer updates them in place). The step holds two
    # input sets (one graph each, both reading their set in place): the copy
    # of step i + 1's batch into one set (on a copy stream, once that set's
    # previous replay is done) overlaps step i's replay on the other; the
    # compute stream waits for the copy, flushes L2 and replays; each step's
    # loss is read on the host one step later. The wall clock runs from the
    # first copy to the last loss read.
    host = {k: step.inputs[0][k].detach().cpu().pin_memory() for k in graph.DATA}
    h2d = sum(t.numel() * t.element_size() for t in host.values())
    copy_stream = torch.cuda.Stream(device)
    copied = [torch.cuda.Event() for _ in range(2)]
    consumed = [torch.cuda.Event() for _ in range(2)]
    loss_host = [torch.empty((), dtype=torch.float32).pin_memory() for _ in range(2)]
    loss_ready = [torch.cuda.Event() for _ in range(2)]

    def issue_copy(b):
        with torch.cuda.stream(copy_stream):
            copy_stream.wait_event(consumed[b])
            with torch.no_grad():
                for k, t in host.items():
                    step.inputs[b][k].copy_(t, non_blocking=True)
            copied[b].record(copy_stream)

    def run_e2e(n):
        losses = []
        issue_copy(0)
        for i in range(n):
            b = i & 1
            if i + 1 < n:
                issue_copy(1 - b)
            stream.wait_event(copied[b])
            flush.fill_(float(i))
            loss_host[b].copy_(step(b), non_blocking=True)
            consumed[b].record(stream)
            loss_ready[b].record(stream)
            if i > 0:
                loss_ready[1 - b].synchronize()
                losses.append(float(loss_host[1 - b]))
        loss_ready[(n - 1) & 1].synchronize()
        losses.append(float(loss_host[(n - 1) & 1]))
        return losses

    run_e2e(3)
    barrier(world)
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    e2e_losses = run_e2e(args.steps)
    e2e_value = max_over_ranks(1000.0 * (time.perf_counter() - t0) / args.steps, world)
    assert len(e2e_losses) == args.steps and all(math.isfinite(x) for x in e2e_losses)

    if rank != 0:
        return

    # Roofline of the dominant entry point (largest share of device time).
    peak, peak_kind = measured_peaks()
    bytes_by_stage = pipeline.step_bytes(stats)
    # Library entry point -> the step_bytes stages its kernels cover.
    stages_of = {
        "mt_intersect_and_composite_backward": ("composite_bwd",),
        "mt_intersect_and_composite_forward": ("composite_fwd", "warp_masks"),
        "mt_sort_keys_by_tile": ("tile_sort",),
        "mt_bound_and_generate_keys": ("keys",),
        "mt_grid_sh_colors": ("grid_sh_colors",),
        "mt_create_triangle_faces": ("create_faces",),
    }
    totals = {k: sum(v) for k, v in per_call.items()}
    dominant = max(totals, key=totals.get)
    dom_ms = statistics.mean(per_call[dominant])
    dom_stages = stages_of.get(dominant)
    dom_bytes = sum(bytes_by_stage[x] for x in dom_stages) if dom_stages else None
    achieved = (dom_bytes / (dom_ms * 1e-3) / 1e9) if dom_bytes else None
    total_bytes = sum(bytes_by_stage.values())
    traffic, traffic_note = profiled_traffic(dominant)

    b = stats["B"]
    h, wd = w.image_shape
    line = {
        "metric": METRIC,
        "value": ms,
        "unit": "ms",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": workload_config(w, stats),
        "parallelism": "replicas" if world > 1 else "single GPU",
        "tile_shape": list(tile),
        "tile_autotune_ms": {"x".join(str(x) for x in k): v for k, v in tile_ms.items()},
        "keys": stats["K"],
        "hbm_gbs": total_bytes / (ms * 1e-3) / 1e9,
        "hbm_bytes_per_step": total_bytes,
        "hbm_bytes_form": "compulsory bytes of the kernels the captured step runs (pipeline.step_bytes)",
        "reference_algorithm_bytes_per_step": sum(pipeline.reference_algorithm_bytes(stats).values()),
        "step_ms_median": statistics.median(step_ms),
        "step_ms_p90": sorted(step_ms)[int(0.9 * (len(step_ms) - 1))],
        "wall_s_timed_region": wall,
        "step_form": "CUDA graph replay of the whole fused forward+backward (capacity-sized buffers)",
        "capacities_fit": fits,
        "eager_ms_per_step": eager_ms,
        "gpu_launches": int(round(launches_per_step * args.steps)),
        "gpu_launches_per_step": launches_per_step,
        "kernel_ms": {k: statistics.mean(v) for k, v in sorted(per_call.items(), key=lambda kv: -sum(kv[1]))},
        "roofline": {
            "kernel": dominant,
            "bound": "hbm",
            "achieved": achieved,
            "peak": peak,
            "peak_kind": peak_kind,
            "unit": "GB/s",
            "frac": (achieved / peak) if achieved else None,
            "traffic": traffic,
            "traffic_source": traffic_note,
            "algorithmic_bytes_per_launch": dom_bytes,
            "algorithmic_stages": list(dom_stages) if dom_stages else None,
            "launch_ms": dom_ms,
        },
        "e2e": {"value": e2e_value, "unit": "ms", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": 4,
                "form": "per step: pinned-host copy of the batch (target images and cameras) on a copy stream "
                        "into one of the step's two input sets (one graph per set, each reading its set in "
                        "place; parameters resident and shared; the copy overlaps the other set's replay), "
                        "L2 flush, graph replay, loss read on the host one step later; wall clock over all "
                        "steps"},
        "clocks": clock_info,
    }
    if not args.no_cameras and world == 1:
        line["cameras_batched"] = run_cameras(device, min(args.steps, 20))
    if not args.no_serving and world == 1:
        line["serving"] = run_serving(device, args.serve_requests)
    if not args.no_large and world == 1:
        line["large"] = run_large(device, min(args.steps, 10))
    if not args.no_band and world == 1:
        line["band_matched"] = run_band_matched(device, min(args.steps, 20))
    if not args.no_subdivision and world == 1:
        line["subdivision"] = run_subdivision(device, min(args.steps, 20), cpu=not args.no_cpu_baseline)
    if not args.no_reference_cub and world == 1:
        line["reference_cub"] = run_reference_cub(w)
    if not args.no_cpu_baseline and world == 1:
        cpu_s = [cpu_step(w)[0] for _ in range(3)]
        cpu_ms = 1000.0 * statistics.median(cpu_s[1:])
        line["cpu_baseline"] = {
            "value": cpu_ms, "unit": "ms", "cores": cpu_threads(), "kind": "port",
            "sample": f"3 whole training steps of the workload on the host (tessellation of every shell, fused "
                      f"render of all {b} cameras, MSE, every backward), median of the last 2",
        }
    print(json.dumps(line))


def run_cameras(device, steps):
    """Cameras of uneven size: the mid scene (256^3, 8 spheres, SH degree 3,
    8 shells) seen by 32 cameras of 200-1600 px per side on its orbit. One batched training step (render_cameras, tile
    shape autotuned over 8/16/32, as a CUDA graph) against the plain form that
    renders each camera with its own call (eager), plus the images' largest
    difference between the two."""
    import torch

    from meshtryoshka_gb300 import autotune, graph, pipeline
    from meshtryoshka_gb300 import triangle_extraction as te
    from meshtryoshka_gb300 import triangle_rasterization as tr

    w = pipeline.build_workload("uneven", device)
    tile, tile_ms = autotune.tune_tile_shape(w, repeats=max(3, min(steps, 10)))
    captured = graph.CapturedTrainingStep(w)
    batched_graph = autotune.time_ms(captured, repeats=steps)

    def batched_eager():
        w.grid_sdf.grad = None
        w.grid_sh.grad = None
        pipeline.training_step(w)

    def per_camera():
        w.grid_sdf.grad = None
        w.grid_sh.grad = None
        pipeline.per_camera_training_step(w)

    eager_ms = autotune.time_ms(batched_eager, repeats=steps)
    plain_ms = autotune.time_ms(per_camera, repeats=steps)
    with torch.no_grad():
        tri = te.tessellate_voxels(w.grid_sdf, w.voxels.vertices, w.grid_sh, w.voxels.neighbors,
                                   w.voxels.lower_corners, w.voxels.upper_corners, w.voxels.indices, w.level_sets)
        vertices = pipeline.uncontract_stand_in(tri.vertices)
        args = (vertices, tri.faces, tri.face_boundaries, tri.signed_distances, tri.spherical_harmonics, w.sh_degree,
                w.sharpness, w.background)
        images = tr.render_cameras(w.extrinsics, w.intrinsics, w.image_shapes, *args, tile_shape=tile)
        diff = 0.0
        for b, (h, wd) in enumerate(w.image_shapes):
            single = tr.render_fused(w.extrinsics[b:b + 1], w.intrinsics[b:b + 1], (h, wd), *args, tile_shape=tile)
            diff = max(diff, float((single[0] - images[b]).abs().max()))
    return {
        "workload": f"uneven: {w.config.resolution}^3 band around 8 spheres, SH deg 3, {w.level_sets.numel()} shells, "
                    f"{len(w.image_shapes)} cameras of 200-1600 px per side ({w.num_pixels} pixels), "
                    "fused fwd+bwd training step",
        "tile": list(tile),
        "tile_ms": {"x".join(str(x) for x in k): v for k, v in tile_ms.items()},
        "batched_graph_ms": batched_graph,
        "batched_eager_ms": eager_ms,
        "per_camera_eager_ms": plain_ms,
        "speedup_vs_per_camera": plain_ms / batched_graph,
        "max_image_diff_vs_per_camera": diff,
    }


def run_large(device, steps):
    """The large training step: 512^3 band around 32 spheres plus an
    inward-facing background sphere, SH degree 3, 16 shells, 4 cameras at
    1297x840 inside the background. Forward + backward in both render modes
    (eager; the fused mode also as a CUDA graph), each with its peak HBM
    above the resident scene, and the largest difference between the two
    modes' images."""
    import torch

    from meshtryoshka_gb300 import autotune, graph, pipeline
    from meshtryoshka_gb300 import triangle_extraction as te

    from meshtryoshka_gb300 import triangle_rasterization as tr

    w = pipeline.build_workload("large", device)
    out = {}
    for mode in ("fused", "explicit"):
        def step(mode=mode, defer_sh=False):
            w.grid_sdf.grad = None
            w.grid_sh.grad = None
            pipeline.training_step(w, mode, defer_sh=defer_sh)

        step()
        torch.cuda.synchronize(device)
        w.grid_sdf.grad = None
        w.grid_sh.grad = None
        torch.cuda.empty_cache()
        resident = torch.cuda.memory_allocated(device)
        torch.cuda.reset_peak_memory_stats(device)
        step()
        torch.cuda.synchronize(device)
        peak = torch.cuda.max_memory_allocated(device) - resident
        out[mode] = {"eager_ms": autotune.time_ms(step, repeats=steps), "peak_hbm_gb": peak / 1e9,
                     "resident_gb": resident / 1e9}
        if mode == "fused":  # the same step with no hit bits kept for the backward
            budget = tr.HIT_BITS_BYTES_PER_PIXEL
            tr.HIT_BITS_BYTES_PER_PIXEL = 0
            w.grid_sdf.grad = None
            w.grid_sh.grad = None
            torch.cuda.empty_cache()
            torch.cuda.reset_peak_memory_stats(device)
            step()
            torch.cuda.synchronize(device)
            out[mode]["peak_hbm_gb_without_hit_bits"] = (torch.cuda.max_memory_allocated(device) - resident) / 1e9
            tr.HIT_BITS_BYTES_PER_PIXEL = budget
        # The same step with vertex colours from the grid SH (no [C, V, 3]
        # rows, which dominate the peaks above): the two modes then differ by
        # the explicit mode's per-shell buffers.
        step(defer_sh=True)
        torch.cuda.synchronize(device)
        w.grid_sdf.grad = None
        w.grid_sh.grad = None
        torch.cuda.empty_cache()
        torch.cuda.reset_peak_memory_stats(device)
        step(defer_sh=True)
        torch.cuda.synchronize(device)
        out[mode]["peak_hbm_gb_deferred_sh"] = (torch.cuda.max_memory_allocated(device) - resident) / 1e9
    w.grid_sdf.grad = None
    w.grid_sh.grad = None
    with torch.no_grad():
        _, stats = pipeline.forward(w, "fused")
    # The captured step's footprint: the device memory its graph holds (its
    # private pool: capacity-sized buffers with a 1.25 margin, deferred SH,
    # the contribution list, the hit bits) plus the library workspace it
    # reads, above the resident scene.
    w.grid_sdf.grad = None
    w.grid_sh.grad = None
    torch.cuda.empty_cache()
    reserved = torch.cuda.memory_reserved(device)
    resident = torch.cuda.memory_allocated(device)
    torch.cuda.reset_peak_memory_stats(device)
    captured = graph.CapturedTrainingStep(w, capacities=pipeline.Capacities.around(stats))
    captured()
    torch.cuda.synchronize(device)
    out["fused"]["graph_construction_peak_hbm_gb"] = (torch.cuda.max_memory_allocated(device) - resident) / 1e9
    torch.cuda.empty_cache()
    out["fused"]["graph_held_hbm_gb"] = (torch.cuda.memory_reserved(device) - reserved) / 1e9
    out["fused"]["graph_ms"] = autotune.time_ms(captured, repeats=steps)
    del captured
    # The captured step at the fastest tile shape (same images; the eager and
    # memory figures above stay at the reference's 16x16 tiles).
    tile, tile_ms = autotune.tune_tile_shape(w, candidates=((8, 8, 256), (8, 8, 512), (16, 8, 256), (16, 16, 256)),
                                             repeats=steps)
    out["fused"]["graph_ms_tuned"] = tile_ms[tile]
    out["fused"]["graph_tile_shape"] = list(tile)
    w.tile_shape = (16, 16)
    with torch.no_grad():
        tri = te.tessellate_voxels(w.grid_sdf, w.voxels.vertices, w.grid_sh, w.voxels.neighbors,
                                   w.voxels.lower_corners, w.voxels.upper_corners, w.voxels.indices, w.level_sets)
        vertices = pipeline.uncontract_stand_in(tri.vertices)
        fused = pipeline._render(w, tri, vertices, None, "fused")
        explicit = pipeline._render(w, tri, vertices, None, "explicit")
        diff = float((fused - explicit).abs().max())
    h, wd = w.image_shape
    out.update({
        "workload": f"large: {w.config.resolution}^3 band around 32 spheres + background sphere, SH deg 3, "
                    f"{w.level_sets.numel()} shells, {w.extrinsics.shape[0]}x{h}x{wd}, fwd+bwd training step",
        "sizes": {k: stats[k] for k in ("G", "Nv", "V", "F", "K", "P")},
        "max_image_diff_fused_vs_explicit": diff,
    })
    return out


def run_band_matched(device, steps):
    """The mid step on a band wide enough for its shells ("mid_band": the
    same spheres, cameras and 8 level sets in [-0.03, 0.03] on a 4-voxel
    band, so that every shell has faces): the captured step at the
    autotuned tile, with its sizes."""
    import torch

    from meshtryoshka_gb300 import autotune, pipeline

    w = pipeline.build_workload("mid_band", device)
    tile, tile_ms = autotune.tune_tile_shape(w, candidates=((8, 8, 128), (8, 8, 256), (16, 8, 256)),
                                             repeats=steps)
    with torch.no_grad():
        _, stats = pipeline.forward(w, "fused")
    h, wd = w.image_shape
    cfg = w.config
    out = {
        "workload": f"mid_band: {cfg.resolution}^3, {cfg.band_voxels:g}-voxel band around {cfg.num_spheres} spheres, "
                    f"SH deg {cfg.sh_degree}, {len(cfg.level_sets)} shells in [-0.03, 0.03], "
                    f"{w.extrinsics.shape[0]}x{h}x{wd}, fused fwd+bwd training step",
        "sizes": {k: int(stats[k]) for k in ("G", "Nv", "V", "F", "K", "P")},
        "tile": list(tile),
        "graph_ms": tile_ms[tile],
        "tile_ms": {"x".join(str(x) for x in k): v for k, v in tile_ms.items()},
    }
    return out


def run_subdivision(device, steps, cpu=True, config="mid"):
    """Coarse-to-fine subdivision step (subdivision.subdivide: canonical
    vertex copy, triangle-voxel mask, dilation by 4, occupancy and parameter
    upscaling) of a scene to twice its resolution (the mid scene: 256^3 ->
    512^3 with SH degree 3), against the oracle on the host cores; the two
    results are compared bit for bit."""
    import time

    import numpy as np
    import torch

    from meshtryoshka_gb300 import _native as nt
    from meshtryoshka_gb300 import subdivision, synthetic
    from meshtryoshka_gb300 import triangle_extraction as te

    cfg = synthetic.CONFIGS[config]
    occ = synthetic.make_occupancy(cfg, device)
    vox = te.extract_voxels(occ)
    sdf = synthetic.corner_sdf(cfg, vox.vertices)
    sh = synthetic.corner_sh(cfg, vox.num_vertices, device)
    with torch.no_grad():
        tri = te.tessellate_voxels(sdf, vox.vertices, sh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                   vox.indices, synthetic.level_sets(cfg, device))
    target = (2 * cfg.resolution,) * 3

    def step():
        return subdivision.subdivide(vox, sdf, sh, occ, tri.voxel_indices, target)

    for _ in range(3):
        step()
    torch.cuda.synchronize(device)
    times = []
    for _ in range(max(steps, 5)):
        t0 = time.perf_counter()
        out = step()
        torch.cuda.synchronize(device)
        times.append(1000.0 * (time.perf_counter() - t0))
    with nt.record_launches(timed=True) as rec:
        step()
        torch.cuda.synchronize(device)
    kernels = {name: round(sum(v), 4) for name, v in rec.times_ms().items()}
    result = {
        "workload": f"{config} scene {cfg.resolution}^3 ({vox.num_voxels} voxels, {vox.num_vertices} vertices, SH "
                    f"C={sh.shape[0]}, {tri.voxel_indices.numel()} triangles) -> {target[0]}^3, dilation 4",
        "new_vertices": int(out.signed_distances.numel()),
        "gpu_ms_median": float(np.median(times)),
        "gpu_ms_min": float(np.min(times)),
        "kernel_ms": kernels,
    }
    if cpu:
        from oracle import oracle

        args = (vox.vertices.cpu().numpy(), sdf.cpu().numpy(), sh.cpu().numpy(), occ.cpu().numpy(),
                tri.voxel_indices.cpu().numpy(), target)
        t0 = time.perf_counter()
        want = oracle.subdivide(*args)
        cpu_ms = 1000.0 * (time.perf_counter() - t0)
        identical = all(np.array_equal(a, b.cpu().numpy()) for a, b in
                        zip(want, (out.signed_distances, out.spherical_harmonics, out.occupancy)))
        result.update({"cpu_ms": cpu_ms, "cpu_cores": cpu_threads(), "cpu_kind": "port",
                       "identical_to_oracle": bool(identical)})
    return result


def run_reference_cub(w, repeats=20):
    """The reference's own CUB extensions (oracle/cub_ref.py: its
    compute_exclusive_cumsum.cu and sort_keys.cu built as they are) against
    this library's scan and sorts on the same GPU, on the step's sizes: the
    vertex-count scan (S * G + 1 int32, in place) and the fused-layout keys of
    the step's cameras at the reference's 16x16 tiles (stable signed 64-bit
    pair sort). Device time per call, CUDA events, median of ``repeats``."""
    import torch

    from meshtryoshka_gb300 import _native as nt
    from meshtryoshka_gb300 import pipeline
    from meshtryoshka_gb300 import triangle_extraction as te
    from meshtryoshka_gb300 import triangle_rasterization as tr
    from oracle import cub_ref

    try:
        modules = cub_ref.load()
    except Exception as exc:  # a build failure is reported, not fatal
        return {"unavailable": f"reference CUB extensions did not build: {type(exc).__name__}: {exc}"[:300]}
    if modules is None:
        return {"unavailable": "reference CUB sources not staged (no reference checkout where this was built)"}
    ref_scan, ref_sort = modules
    device = w.grid_sdf.device
    stream = torch.cuda.current_stream(device)
    lib = nt.library()

    def timed(fn, prepare):
        # A device-side sleep ahead of the start event keeps the host's
        # enqueue overhead (pybind for the reference, ctypes here) out of the
        # device time of both.
        times = []
        for i in range(repeats + 3):
            prepare()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda._sleep(200_000)
            a.record(stream)
            fn()
            b.record(stream)
            b.synchronize()
            if i >= 3:
                times.append(a.elapsed_time(b))
        return statistics.median(times)

    with torch.no_grad():
        v = w.voxels
        counts = te.count_triangle_vertices(w.grid_sdf, v.lower_corners, w.level_sets)
        tri = te.tessellate_voxels(w.grid_sdf, v.vertices, w.grid_sh, v.neighbors, v.lower_corners, v.upper_corners,
                                   v.indices, w.level_sets)
        verts = pipeline.uncontract_stand_in(tri.vertices)
        b = w.extrinsics.shape[0]
        grid = tr.TileGrid((16, 16), w.image_shape, b, w.level_sets.numel())
        kd = tr.create_key_defines(("camera", 6), ("tile", 20), ("depth", 32), ("shell", 6))
        xy, depth = tr.project_vertices(verts, w.extrinsics, w.intrinsics)
        bounds = tr.bound_triangles(xy, depth, tri.faces, grid, 0.2)
        paired = tr.generate_keys(depth, tri.faces, tri.face_boundaries, bounds.tile_minima, bounds.tile_maxima,
                                  bounds.num_tiles_overlapped, grid, kd)
    n = counts.numel()
    k = paired.keys.numel()
    x = torch.empty_like(counts)
    ws_ptr, ws_bytes = nt.workspace(device).get(lib.mt_scan_workspace_bytes(n))
    refill = lambda: x.copy_(counts)  # noqa: E731
    out = {"scan_elements": n, "sort_keys": k}
    out["reference_scan_ms"] = timed(lambda: ref_scan.compute_exclusive_cumsum(x), refill)
    out["ours_scan_ms"] = timed(lambda: nt.call("mt_exclusive_scan_i32", x.data_ptr(), n, ws_ptr, ws_bytes,
                                                nt.stream(device)), refill)
    want = x.clone()
    ref_scan.compute_exclusive_cumsum(want.copy_(counts))
    nt.call("mt_exclusive_scan_i32", x.copy_(counts).data_ptr(), n, ws_ptr, ws_bytes, nt.stream(device))
    out["scan_identical"] = bool(torch.equal(x, want))
    keys, idx = paired.keys.contiguous(), paired.triangle_indices.contiguous()
    out["reference_sort_ms"] = timed(lambda: ref_sort.sort_keys(keys, idx, k), lambda: None)
    ours = {}
    out["ours_radix_sort_ms"] = timed(lambda: ours.update(p=tr.sort_keys(paired, grid)), lambda: None)
    out["ours_tile_sort_and_delineate_ms"] = timed(
        lambda: ours.update(t=tr._sort_and_delineate(paired, grid, kd, False)), lambda: None)
    rk, rt = ref_sort.sort_keys(keys, idx, k)
    out["sort_identical"] = bool(torch.equal(rk, ours["p"].keys) and torch.equal(rt, ours["p"].triangle_indices)
                                 and torch.equal(rk, ours["t"][0].keys))
    out["note"] = ("the reference sort is followed by its delineate_tiles kernel (Slang, not runnable here); the "
                   "tile sort produces the sorted keys and the tile ranges in one entry point")
    return out


SERVE_RATES = (50, 200, 500, 1000, 2000)
SERVE_REQUESTS = 2000


def run_serving(device, requests_per_rate=SERVE_REQUESTS):
    """Serving sweep: four resident scenes (mid layout at 256^3 x2 and 128^3,
    large layout at 512^3; SH degree 3, 8 shells), Poisson arrivals at each
    rate for ``requests_per_rate`` requests, 80 % render-only and 20 % render
    + gradient, images of 256-1920 x 256-1080 px. Continuous batching
    (serving.Server) against the plain per-request form at the same arrival
    times; p50 / p99 latency and throughput for both, and the server's peak
    estimated bytes in flight against its budget."""
    import torch

    from meshtryoshka_gb300 import serving

    scenes = serving.default_scenes(device)
    server = serving.Server(scenes)
    warm = serving.poisson_requests(scenes, 500.0, 0.05, seed=99)
    server.run(warm)
    serving.run_plain(scenes, warm[:10])
    torch.cuda.synchronize(device)
    rows = []
    for rate in SERVE_RATES:
        requests = serving.poisson_requests(scenes, float(rate), requests_per_rate / rate, seed=4 + rate)
        server = serving.Server(scenes)
        # Responses are released as they complete (the client here needs only
        # their timing), in both forms.
        batched = serving.latency_summary(server.run(requests, keep_results=False))
        torch.cuda.synchronize(device)
        plain = serving.latency_summary(serving.run_plain(scenes, requests, keep_results=False))
        rows.append({"rate_rps": rate, "batched": batched, "plain": plain,
                     "p99_ratio_plain_over_batched": plain["p99_ms"] / batched["p99_ms"],
                     "peak_inflight_gb": server.peak_inflight_bytes / 1e9, "hbm_budget_gb": server.hbm_budget / 1e9})
        del requests
        torch.cuda.empty_cache()
    return {
        "workload": "4 resident scenes (mid layout at 256^3 x2 and 128^3, large layout at 512^3; 8 shells, SH deg "
                    f"3); Poisson arrivals, {requests_per_rate} requests per rate; 80 % render, 20 % render+gradient "
                    "(MSE vs U[0,1] target); images 256-1920 x 256-1080, fov 40-70; the server back-propagates "
                    "gradient requests through each scene's resident tessellation, the plain form tessellates per "
                    "gradient request",
        "rates": rows,
    }


def main():
    args = parse()
    if args.steps is None:
        args.steps = 5 if args.impl == "reference" else 200
    if args.warmup is None:
        args.warmup = 3 if args.impl == "reference" else 5
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
