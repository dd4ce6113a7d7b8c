"""The per-step render path as the trainer composes it (meshtryoshka/model/
model_meshtryoshka.py:240-258, ModelMeshtryoshka.fit): tessellate the voxel
SDF at every level set, render all cameras, MSE against the targets, and
backpropagate into the grid signed distances and spherical harmonics.

Used by ``bench.py`` and the smoke test; a trainer calls the two package
functions directly.
"""

from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch
from torch import Tensor

from . import _native as nt
from . import synthetic
from . import triangle_extraction as te
from . import triangle_rasterization as tr


@dataclass
class Workload:
    config: synthetic.SceneConfig
    voxels: te.Voxels
    grid_sdf: Tensor  # [G] leaf, requires grad
    grid_sh: Tensor  # [C, G, 3] leaf, requires grad
    level_sets: Tensor  # [S] descending
    extrinsics: Tensor  # [B, 4, 4]
    intrinsics: Tensor  # [B, 3, 3]
    image_shape: tuple[int, int]
    target: Tensor  # [B, 3, H, W]; cameras of different sizes: every camera's [3, h, w] back to back
    sharpness: Tensor  # [] constant, as the trainer rebuilds it every call
    background: Tensor  # [3]
    image_shapes: tuple[tuple[int, int], ...] | None = None  # cameras of different sizes
    tile_shape: tuple[int, int] = (16, 16)
    fused_loss: bool = True  # fused render: blend, clip and MSE inside the compositing kernels
    ssaa: int = 1  # supersampling factor of the render (the trainer's train_ssaa)

    @property
    def sh_degree(self) -> int:
        return self.config.sh_degree

    def targets(self) -> list[Tensor]:
        """Per-camera [3, h, w] targets."""
        if self.image_shapes is None:
            return list(self.target)
        views, start = [], 0
        for h, w in self.image_shapes:
            views.append(self.target[start:start + 3 * h * w].view(3, h, w))
            start += 3 * h * w
        return views

    @property
    def num_pixels(self) -> int:
        shapes = self.image_shapes or ((self.image_shape,) * self.extrinsics.shape[0])
        return sum(h * w for h, w in shapes)


def build_workload(name: str, device: torch.device) -> Workload:
    """Synthetic scene of one of the benchmark configurations, resident on `device`."""
    cfg = synthetic.CONFIGS[name]
    occ = synthetic.make_occupancy(cfg, device)
    voxels = te.extract_voxels(occ)
    sdf = synthetic.corner_sdf(cfg, voxels.vertices)
    sh = synthetic.corner_sh(cfg, voxels.vertices.shape[0], device)
    cams = synthetic.make_cameras(cfg)
    shapes = tuple(tuple(x) for x in cams.image_shapes)
    ragged = len(set(shapes)) != 1
    if ragged:
        h, w = max(x[0] for x in shapes), max(x[1] for x in shapes)
        rng = np.random.default_rng(3)
        target = torch.from_numpy(rng.uniform(0.0, 1.0, 3 * sum(a * b for a, b in shapes)).astype(np.float32))
        target = target.to(device)
    else:
        h, w = shapes[0]
        target = synthetic.make_target(cfg.num_cameras, h, w, device)
    return Workload(
        config=cfg,
        voxels=voxels,
        grid_sdf=sdf.requires_grad_(True),
        grid_sh=sh.requires_grad_(True),
        level_sets=synthetic.level_sets(cfg, device),
        extrinsics=torch.from_numpy(cams.extrinsics).to(device),
        intrinsics=torch.from_numpy(cams.intrinsics).to(device),
        image_shape=(h, w),
        target=target,
        sharpness=torch.tensor(cfg.sharpness, dtype=torch.float32, device=device),
        background=torch.tensor([0.0, 0.0, 0.0], dtype=torch.float32, device=device),
        image_shapes=shapes if ragged else None,
    )


def _loss(w: Workload, images) -> Tensor:
    """Mean squared error over every pixel and channel of every camera."""
    if w.image_shapes is None:
        return ((images - w.target) ** 2).mean()
    total = sum(((img - tgt) ** 2).sum() for img, tgt in zip(images, w.targets()))
    return total / (3 * w.num_pixels)


def _fused_loss(w: Workload, tri, vertices, gradient_mode, **counted) -> Tensor:
    return tr.render_fused_loss(w.extrinsics, w.intrinsics, w.image_shape, vertices, tri.faces, tri.face_boundaries,
                                tri.signed_distances, tri.spherical_harmonics, w.sh_degree, w.sharpness,
                                w.background, w.target, tile_shape=w.tile_shape, gradient_mode=gradient_mode,
                                camera_shapes=w.image_shapes, ssaa=w.ssaa, **counted)


def _render(w: Workload, tri, vertices, gradient_mode, mode="fused", **counted):
    if w.image_shapes is not None:
        return tr.render_cameras(w.extrinsics, w.intrinsics, w.image_shapes, vertices, tri.faces, tri.face_boundaries,
                                 tri.signed_distances, tri.spherical_harmonics, w.sh_degree, w.sharpness, w.background,
                                 tile_shape=w.tile_shape, gradient_mode=gradient_mode, **counted)
    if counted:
        return tr.render_fused(w.extrinsics, w.intrinsics, w.image_shape, vertices, tri.faces, tri.face_boundaries,
                               tri.signed_distances, tri.spherical_harmonics, w.sh_degree, w.sharpness, w.background,
                               tile_shape=w.tile_shape, gradient_mode=gradient_mode, **counted)
    return tr.render(w.extrinsics, w.intrinsics, w.image_shape, vertices, tri.faces, tri.face_boundaries,
                     tri.signed_distances, tri.spherical_harmonics, w.sh_degree, w.sharpness, w.background,
                     tile_shape=w.tile_shape, mode=mode, gradient_mode=gradient_mode, ssaa=w.ssaa)


@dataclass(frozen=True)
class Capacities:
    """Row capacities of the per-step vertex, face and key buffers."""

    vertices: int
    faces: int
    keys: int

    @staticmethod
    def around(stats: dict, margin: float = 1.25, minimum: int = 4096) -> "Capacities":
        grow = lambda n: max(int(n * margin) + minimum, minimum)  # noqa: E731
        return Capacities(grow(stats["V"]), grow(stats["F"]), grow(stats["K"]))


_AFFINE: dict = {}


def uncontract_stand_in(vertices: Tensor) -> Tensor:
    """2 v - 1, the linear stand-in for the trainer's uncontract(), as one
    elementwise kernel (-1 + v * 2: v * 2 is exact, so the value is that of
    2.0 * v - 1.0)."""
    key = str(vertices.device)
    consts = _AFFINE.get(key)
    if consts is None:
        consts = (torch.tensor(-1.0, device=vertices.device), torch.tensor(2.0, device=vertices.device))
        _AFFINE[key] = consts
    return torch.addcmul(consts[0], vertices, consts[1])


def forward_counted(w: Workload, caps: Capacities, gradient_mode: str | None = None,
                    grid_sdf: Tensor | None = None, grid_sh: Tensor | None = None,
                    defer_sh: bool = True) -> tuple[Tensor, Tensor]:
    """The fused step's forward with capacity-sized buffers and no
    device->host reads (capturable in a CUDA graph). Returns the loss and a
    device flag that is true when a live vertex, face or key count exceeded
    its capacity (the step's result is then incomplete). ``defer_sh``: vertex
    colours straight from the grid SH (no per-vertex SH rows; same values)."""
    grid_sdf = w.grid_sdf if grid_sdf is None else grid_sdf
    grid_sh = w.grid_sh if grid_sh is None else grid_sh
    tri, counts = te.tessellate_voxels_counted(
        grid_sdf, w.voxels.vertices, grid_sh, w.voxels.neighbors, w.voxels.lower_corners,
        w.voxels.upper_corners, w.voxels.indices, w.level_sets, caps.vertices, caps.faces, defer_sh=defer_sh)
    with torch.no_grad():
        vertices = uncontract_stand_in(tri.vertices)
    counted = dict(num_faces=counts.num_faces, key_capacity=caps.keys)
    if w.fused_loss:
        loss = _fused_loss(w, tri, vertices, gradient_mode, **counted)
    else:
        loss = _loss(w, _render(w, tri, vertices, gradient_mode, **counted))
    key_count = tr.LAST_RENDER_STATS["key_count"]
    overflow = torch.empty((), dtype=torch.bool, device=loss.device)
    nt.call("mt_capacity_overflow", counts.num_vertices.data_ptr(), caps.vertices, counts.num_faces.data_ptr(),
            caps.faces, key_count.data_ptr(), caps.keys, overflow.data_ptr(), nt.stream(loss.device))
    return loss, overflow


def forward(w: Workload, mode: str = "fused", gradient_mode: str | None = None,
            grid_sdf: Tensor | None = None, grid_sh: Tensor | None = None,
            target: Tensor | None = None, defer_sh: bool = False) -> tuple[Tensor, dict]:
    """The eager step's forward in either render mode. ``defer_sh``: vertex
    colours straight from the grid SH (no per-vertex SH rows; same values)."""
    grid_sdf = w.grid_sdf if grid_sdf is None else grid_sdf
    grid_sh = w.grid_sh if grid_sh is None else grid_sh
    target = w.target if target is None else target
    tri = te.tessellate_voxels(grid_sdf, w.voxels.vertices, grid_sh, w.voxels.neighbors, w.voxels.lower_corners,
                               w.voxels.upper_corners, w.voxels.indices, w.level_sets, defer_sh=defer_sh)
    with torch.no_grad():
        vertices = uncontract_stand_in(tri.vertices)
    if mode == "fused" and w.fused_loss and target is w.target:
        loss = _fused_loss(w, tri, vertices, gradient_mode)
    else:
        image = _render(w, tri, vertices, gradient_mode, mode)
        loss = _loss(w, image) if target is w.target else ((image - target) ** 2).mean()
    stats = {
        "G": int(w.voxels.lower_corners.shape[1]),
        "Nv": int(w.voxels.upper_corners.shape[1]),
        "V": int(tri.vertices.shape[0]),
        "F": int(tri.faces.shape[0]),
        "C": int(grid_sh.shape[0]),
        "S": int(w.level_sets.shape[0]),
        "B": int(w.extrinsics.shape[0]),
        "P": int(w.num_pixels),
        "K": int(tr.LAST_RENDER_STATS.get("num_keys", 0)),
        "T": int(tr.LAST_RENDER_STATS.get("num_tiles", 0)),
    }
    return loss, stats


def training_step(w: Workload, mode: str = "fused", **kw) -> Tensor:
    """One forward + backward; gradients accumulate into w.grid_sdf / w.grid_sh."""
    loss, _ = forward(w, mode, **kw)
    loss.backward()
    return loss


def per_camera_training_step(w: Workload, gradient_mode: str | None = None) -> Tensor:
    """The plain form of a multi-camera step: one tessellation, then every
    camera rendered by its own ``render_fused`` call (the reference renders
    one image size per call), one backward. Gives the batched step's loss and
    gradients; used as its comparison baseline."""
    tri = te.tessellate_voxels(w.grid_sdf, w.voxels.vertices, w.grid_sh, w.voxels.neighbors, w.voxels.lower_corners,
                               w.voxels.upper_corners, w.voxels.indices, w.level_sets)
    with torch.no_grad():
        vertices = uncontract_stand_in(tri.vertices)
    shapes = w.image_shapes or ((w.image_shape,) * w.extrinsics.shape[0])
    total = 0.0
    for b, ((h, wd), target) in enumerate(zip(shapes, w.targets())):
        image = tr.render_fused(w.extrinsics[b:b + 1], w.intrinsics[b:b + 1], (h, wd), vertices, tri.faces,
                                tri.face_boundaries, tri.signed_distances, tri.spherical_harmonics, w.sh_degree,
                                w.sharpness, w.background, tile_shape=w.tile_shape, gradient_mode=gradient_mode)[0]
        total = total + ((image - target) ** 2).sum()
    loss = total / (3 * w.num_pixels)
    loss.backward()
    return loss


def reference_algorithm_bytes(stats: dict) -> dict[str, float]:
    """Compulsory traffic per stage of the reference's algorithm (eight radix
    passes over 24-byte key pairs, per-vertex SH rows formed and read back,
    delineation as its own pass), from the measured sizes. Each input read
    once, each output written once, gathers counted once per consumer."""
    G, Nv, V, F, C, S, B, P, K, T = (stats[k] for k in ("G", "Nv", "V", "F", "C", "S", "B", "P", "K", "T"))
    passes = 8
    return {
        "count_vertices": G * (16 + 16) + 4 * S * G,
        "scans": 8 * S * G + 8 * S * Nv,
        "create_vertices": G * (16 + 4 * (4 + 12 + 12 * C)) + V * (16 + 12 * C + 1),
        "count_faces": Nv * (32 + 32) + 5 * S * Nv,
        "create_faces": Nv * (28 + 4 + S) + 8 * S * Nv + 16 * F,
        "project_sh": V * (12 + 12 * C) + 24 * B * V,
        "bound": F * (12 + 36 * B) + 20 * B * F,
        "keys": B * F * (20 + 12) + 8 * B * F + 12 * K,
        "sort": 24 * K * passes,
        "delineate": 8 * K + 16 * B * T,
        "composite_fwd": K * (4 + 8 + 12 + 72) + 16 * P,
        "composite_bwd": K * 96 + 32 * P + 16 * V * B,
        "sh_bwd": 12 * B * V + 24 * C * V,
        "create_vertices_bwd": V * (16 + 12 * C) + G * 4 * (4 + 12 + 12 * C),
    }


def step_bytes(stats: dict) -> dict[str, float]:
    """Compulsory traffic of the kernels the captured training step runs
    (``graph.CapturedTrainingStep``: deferred SH, the contribution list, the
    capacity-mode keys, the tile-bucketed sort, warp masks, the compositing
    kernels with the MSE epilogue), from the measured sizes. Each input read
    once, each output written once, gathers counted once per consumer;
    scratch that only speeds a kernel up (stored hit bits) is not counted."""
    G, Nv, V, F, C, S, B, P, K, T = (stats[k] for k in ("G", "Nv", "V", "F", "C", "S", "B", "P", "K", "T"))
    return {
        # tessellation
        "count_vertices": G * (16 + 16) + 4 * S * G,
        "scans": 8 * S * G + 8 * S * Nv,
        # per entry: 4 corner ids, 4 SDFs, 4 positions, its offsets; per
        # vertex: position, SDF, type, source record (origin, corner, t)
        "create_vertices": G * (16 + 4 * (4 + 12) + 4 * S) + V * (12 + 4 + 1 + 12),
        # corner inverse, per-entry list counts, their scan, list fill
        "contribution_list": G * (16 + 16) + G * (16 + 4) + 8 * G + G * 16 + 16 * V,
        "count_faces": Nv * (32 + 32) + 5 * S * Nv,
        "create_faces": Nv * (28 + 4 + S) + 8 * S * Nv + 16 * F,
        # render front end
        "uncontract": 24 * V,
        "project": 12 * V + 12 * B * V,
        "grid_sh_colors": V * (12 + 12) + 2 * 12 * C * V + 12 * B * V,
        "keys": B * F * (12 + 36 + 20) + B * F * 20 + 12 * K,
        "tile_sort": 60 * K + 16 * B * T,
        "warp_masks": K * (8 + 4 + 12 + 24) + 4 * K,
        # compositing with the MSE epilogue (target read, output written)
        "composite_fwd": K * 96 + 16 * P + 12 * P,
        "gradient_zero_fill": 12 * B * V + 4 * V,
        "composite_bwd": K * 96 + 16 * P + 12 * P + 16 * V * B,
        # grid SH gradient: per-vertex SH gradient once, then per grid vertex
        # the weighted sum over its list entries
        "grid_sh_bwd": 12 * B * V + 24 * V + 12 * C * V + 16 * V + 2 * 12 * C * V + 12 * C * G,
        "grid_sdf_bwd": 16 * V + 4 * V + 16 * G,
    }


def numpy_inputs(w: Workload) -> dict[str, np.ndarray]:
    return {k: getattr(w, k).detach().cpu().numpy() for k in ("grid_sdf", "grid_sh", "target")}
