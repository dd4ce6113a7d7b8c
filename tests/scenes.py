"""Small seeded scenes for parity tests, built on the CPU oracle so GPU and
oracle consume identical input arrays."""

from __future__ import annotations

import dataclasses
from dataclasses import dataclass

import numpy as np
import torch

from meshtryoshka_gb300 import synthetic
from oracle import oracle
from tests import semantics


@dataclass
class Scene:
    vertices: np.ndarray  # [V, 3] renderer positions (2 v - 1)
    faces: np.ndarray
    face_boundaries: np.ndarray
    sdf: np.ndarray  # [V]
    sh: np.ndarray  # [C, V, 3]
    sh_degree: int
    extrinsics: np.ndarray
    intrinsics: np.ndarray
    image_shape: tuple[int, int]
    sharpness: float
    background: np.ndarray


def sphere_mesh(n=64, levels=(0.02, 0.0, -0.02), sh_degree=0, seed=0, radius=0.5, centre=(0.0, 0.0, 0.0)):
    coords = -1 + (np.arange(n) + 0.5) * 2 / n
    z, y, x = np.meshgrid(coords, coords, coords, indexing="ij")
    d = np.sqrt((x - centre[0]) ** 2 + (y - centre[1]) ** 2 + (z - centre[2]) ** 2) - radius
    occ = semantics.pack(np.abs(d) < 2.5 * 2 / n)
    vox = oracle.extract_voxels(occ)
    p = 2 * vox.vertices.astype(np.float64) - 1
    rng = np.random.default_rng(seed)
    gsdf = (np.linalg.norm(p - np.array(centre), axis=1) - radius + rng.normal(0, 0.002, len(p))).astype(np.float32)
    c = (sh_degree + 1) ** 2
    gsh = np.empty((c, len(p), 3), np.float32)
    gsh[0] = rng.uniform(0, 1, (len(p), 3))
    if c > 1:
        gsh[1:] = rng.normal(0, 0.05, (c - 1, len(p), 3))
    ls = np.array(levels, np.float32)
    tri = oracle.tessellate_voxels(gsdf, vox.vertices, gsh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                   vox.indices, ls)
    return tri


def multi_sphere_mesh(n=64, levels=(0.02, 0.0, -0.02), sh_degree=0, seed=0, spheres=6):
    """The large configuration's layout at resolution n: a band around the
    union of `spheres` spheres and an inward-facing background sphere."""
    cfg = dataclasses.replace(synthetic.CONFIGS["large"], resolution=n, num_spheres=spheres, radius_range=(0.15, 0.3))
    occ = synthetic.make_occupancy(cfg, "cpu").numpy()
    vox = oracle.extract_voxels(occ)
    centres, radii = synthetic.sphere_layout(cfg)
    p = torch.from_numpy(2 * vox.vertices - 1)
    d = synthetic.analytic_sdf(p, torch.from_numpy(centres), torch.from_numpy(radii), cfg.background_radius).numpy()
    rng = np.random.default_rng(seed)
    gsdf = (d + rng.normal(0, 0.002, len(d))).astype(np.float32)
    c = (sh_degree + 1) ** 2
    gsh = np.empty((c, len(d), 3), np.float32)
    gsh[0] = rng.uniform(0, 1, (len(d), 3))
    if c > 1:
        gsh[1:] = rng.normal(0, 0.05, (c - 1, len(d), 3))
    return oracle.tessellate_voxels(gsdf, vox.vertices, gsh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                    vox.indices, np.array(levels, np.float32))


def make_scene(n=64, levels=(0.02, 0.0, -0.02), sh_degree=0, cameras=((0.0, 0.0, 2.0),), image_shape=(128, 128),
               fov=60.0, sharpness=50.0, seed=0, spheres=0) -> Scene:
    if spheres:
        tri = multi_sphere_mesh(n, levels, sh_degree, seed, spheres)
    else:
        tri = sphere_mesh(n, levels, sh_degree, seed)
    ext = np.stack([synthetic.look_at(np.array(c)) for c in cameras])
    intr = np.stack([synthetic.pinhole(image_shape[0], image_shape[1], fov) for _ in cameras])
    return Scene(
        vertices=(2.0 * tri.vertices - 1.0).astype(np.float32),
        faces=tri.faces,
        face_boundaries=tri.face_boundaries,
        sdf=tri.signed_distances,
        sh=tri.spherical_harmonics,
        sh_degree=sh_degree,
        extrinsics=ext,
        intrinsics=intr,
        image_shape=image_shape,
        sharpness=sharpness,
        background=np.array([0.2, 0.4, 0.6], np.float32),
    )


SCENES = {
    "front_128": dict(),
    "three_cams_odd": dict(cameras=((0.0, 0.0, 2.0), (1.2, 0.8, 1.3), (-1.5, -0.3, 1.1)), image_shape=(75, 101),
                           fov=55.0, sh_degree=3, levels=(0.03, 0.01, -0.01, -0.03)),
    "close_up": dict(cameras=((0.3, 0.2, 0.9),), image_shape=(96, 64), fov=70.0, levels=(0.01, -0.01),
                     sh_degree=1),
    # Several objects and a background seen from inside, 16 shells: shells of
    # different objects interleave in depth, where the fused walk and the
    # per-shell explicit mode give different images.
    "multi_inside": dict(spheres=6, cameras=((0.6, 0.1, 0.0), (0.0, 0.2, 0.6)), image_shape=(48, 64), fov=55.0,
                         levels=tuple(float(x) for x in np.linspace(0.02, -0.02, 16)), sh_degree=1),
}
