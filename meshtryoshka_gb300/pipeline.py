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
    target: Tensor  # [B, 3, H, W]
    sharpness: Tensor  # [] constant, as the trainer rebuilds it every call
    background: Tensor  # [3]

    @property
    def sh_degree(self) -> int:
        return self.config.sh_degree


def build_workload(name: str, device: torch.device) -> Workload:
    """Synthetic scene of one of the benchmark configurations, resident on `device`."""
    cfg = synthetic.CONFIGS[name]
    occ = synthetic.make_occupancy(cfg, device)
    voxels = te.extract_voxels(occ)
    sdf = synthetic.corner_sdf(cfg, voxels.vertices)
    sh = synthetic.corner_sh(cfg, voxels.vertices.shape[0], device)
    cams = synthetic.make_cameras(cfg)
    if len(set(cams.image_shapes)) != 1:
        raise ValueError("build_workload needs one image size per camera set")
    h, w = cams.image_shapes[0]
    return Workload(
        config=cfg,
        voxels=voxels,
        grid_sdf=sdf.requires_grad_(True),
        grid_sh=sh.requires_grad_(True),
        level_sets=synthetic.level_sets(cfg, device),
        extrinsics=torch.from_numpy(cams.extrinsics).to(device),
        intrinsics=torch.from_numpy(cams.intrinsics).to(device),
        image_shape=(h, w),
        target=synthetic.make_target(cfg.num_cameras, h, w, device),
        sharpness=torch.tensor(cfg.sharpness, dtype=torch.float32, device=device),
        background=torch.tensor([0.0, 0.0, 0.0], dtype=torch.float32, device=device),
    )


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


def forward_counted(w: Workload, caps: Capacities, gradient_mode: str | None = None,
                    grid_sdf: Tensor | None = None, grid_sh: Tensor | None = None) -> tuple[Tensor, Tensor]:
    """The fused step's forward with capacity-sized buffers and no
    device->host reads (capturable in a CUDA graph). Returns the loss and a
    device flag that is true when a live vertex, face or key count exceeded
    its capacity (the step's result is then incomplete)."""
    grid_sdf = w.grid_sdf if grid_sdf is None else grid_sdf
    grid_sh = w.grid_sh if grid_sh is None else grid_sh
    tri, counts = te.tessellate_voxels_counted(
        grid_sdf, w.voxels.vertices, grid_sh, w.voxels.neighbors, w.voxels.lower_corners,
        w.voxels.upper_corners, w.voxels.indices, w.level_sets, caps.vertices, caps.faces)
    with torch.no_grad():
        vertices = 2.0 * tri.vertices - 1.0  # linear stand-in for uncontract()
    image = tr.render_fused(w.extrinsics, w.intrinsics, w.image_shape, vertices, tri.faces, tri.face_boundaries,
                            tri.signed_distances, tri.spherical_harmonics, w.sh_degree, w.sharpness, w.background,
                            gradient_mode=gradient_mode, num_faces=counts.num_faces, key_capacity=caps.keys)
    key_count = tr.LAST_RENDER_STATS["key_count"]
    loss = ((image - w.target) ** 2).mean()
    with torch.no_grad():
        overflow = ((counts.num_vertices > caps.vertices) | (counts.num_faces > caps.faces)
                    | (key_count > caps.keys))
    return loss, overflow


def forward(w: Workload, mode: str = "fused", gradient_mode: str | None = None,
            grid_sdf: Tensor | None = None, grid_sh: Tensor | None = None,
            target: Tensor | None = None) -> tuple[Tensor, dict]:
    grid_sdf = w.grid_sdf if grid_sdf is None else grid_sdf
    grid_sh = w.grid_sh if grid_sh is None else grid_sh
    target = w.target if target is None else target
    tri = te.tessellate_voxels(grid_sdf, w.voxels.vertices, grid_sh, w.voxels.neighbors, w.voxels.lower_corners,
                               w.voxels.upper_corners, w.voxels.indices, w.level_sets)
    with torch.no_grad():
        vertices = 2.0 * tri.vertices - 1.0  # linear stand-in for uncontract()
    image = tr.render(w.extrinsics, w.intrinsics, w.image_shape, vertices, tri.faces, tri.face_boundaries,
                      tri.signed_distances, tri.spherical_harmonics, w.sh_degree, w.sharpness, w.background,
                      mode=mode, gradient_mode=gradient_mode)
    loss = ((image - target) ** 2).mean()
    stats = {
        "G": int(w.voxels.lower_corners.shape[1]),
        "Nv": int(w.voxels.upper_corners.shape[1]),
        "V": int(tri.vertices.shape[0]),
        "F": int(tri.faces.shape[0]),
        "C": int(grid_sh.shape[0]),
        "S": int(w.level_sets.shape[0]),
        "B": int(w.extrinsics.shape[0]),
        "P": int(w.extrinsics.shape[0] * w.image_shape[0] * w.image_shape[1]),
        "K": int(tr.LAST_RENDER_STATS.get("num_keys", 0)),
        "T": int(tr.LAST_RENDER_STATS.get("num_tiles", 0)),
    }
    return loss, stats


def training_step(w: Workload, mode: str = "fused", **kw) -> Tensor:
    """One forward + backward; gradients accumulate into w.grid_sdf / w.grid_sh."""
    loss, _ = forward(w, mode, **kw)
    loss.backward()
    return loss


def algorithmic_bytes(stats: dict) -> dict[str, float]:
    """Compulsory traffic per stage (each input read once, each output
    written once, gathers counted once per consumer), from the measured sizes."""
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


def numpy_inputs(w: Workload) -> dict[str, np.ndarray]:
    return {k: getattr(w, k).detach().cpu().numpy() for k in ("grid_sdf", "grid_sh", "target")}
