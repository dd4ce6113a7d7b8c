"""Tile-shape and threads-per-CTA autotuning for the fused training step.

Times the CUDA-graph training step (``graph.CapturedTrainingStep``) of a
workload for each candidate (tile height, tile width, threads per CTA of the
compositing kernels) with CUDA events and keeps the fastest; results are
cached per workload shape so a trainer or server tunes once per scene/camera
configuration. The reference fixes one tile of TILE_H x TILE_W threads per
CTA at compile time (triangle_rasterization/intersect_and_composite.py:11-21);
here the tile (8, 16 or 32 pixels a side) sets the key lists and the CTA size
(128, 256 or 512 threads of persistent warps) the launch. Every candidate
renders the same images (both only change the work decomposition), so tuning
never changes results beyond atomic summation order in the gradients.
"""

from __future__ import annotations

import statistics

import torch

from . import graph, pipeline

CANDIDATES = ((8, 8, 128), (8, 8, 256), (8, 8, 512), (16, 8, 256), (16, 16, 256), (16, 16, 512), (32, 32, 256))
_CACHE: dict = {}


def time_ms(fn, repeats: int = 10, warmup: int = 3) -> float:
    """Median CUDA-event time of fn() on the current stream, in ms."""
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    stream = torch.cuda.current_stream()
    for _ in range(repeats):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        times.append(a.elapsed_time(b))
    return statistics.median(times)


def _key(w: pipeline.Workload):
    shapes = w.image_shapes or ((w.image_shape,) * w.extrinsics.shape[0])
    return (w.config.name, tuple(shapes), int(w.voxels.lower_corners.shape[1]), int(w.level_sets.numel()))


def tune_tile_shape(w: pipeline.Workload, candidates=CANDIDATES, repeats: int = 10,
                    use_cache: bool = True) -> tuple[tuple[int, int], dict]:
    """Sets ``w.tile_shape`` to the fastest candidate; returns it and the
    per-candidate step times (ms)."""
    key = _key(w)
    if use_cache and key in _CACHE:
        w.tile_shape = _CACHE[key][0]
        return _CACHE[key]
    results = {}
    for tile in candidates:
        w.tile_shape = tuple(tile)
        step = graph.CapturedTrainingStep(w)
        results[tuple(tile)] = time_ms(step, repeats)
        del step
    best = min(results, key=results.get)
    w.tile_shape = best
    _CACHE[key] = (best, results)
    return best, results
