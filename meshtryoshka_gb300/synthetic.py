"""Seeded synthetic scenes with the shapes and value distributions of the
benchmark workloads (the reference trains on Mip-NeRF 360 / NeRF-Synthetic
captures, which are not available here).

A scene is an analytic SDF (a union of spheres, optionally with an
inward-facing background sphere) sampled on the corners of a sparse voxel
band, plus per-corner spherical-harmonic colours, a set of level sets
(shells) in descending order (shell 0 outermost, as the trainer produces with
``logit(cdf) / sharpness`` for descending CDFs), pinhole cameras looking at
the origin, and a random target image.

Axis convention (triangle_extraction/create_voxels.slang:44-46): voxel
(i, j, k) has its corner at (k, j, i) / extent, i.e. x <-> k (the packed
axis), y <-> j, z <-> i. Renderer positions are ``2 * v - 1`` in [-1, 1]^3,
a linear stand-in for the trainer's ``uncontract``.

Random draws use numpy's PCG64 (platform independent); geometry is evaluated
with torch on the requested device. Seeds: 0 grid noise, 1 colours,
2 cameras, 3 target, 5 sphere layout.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch


@dataclass(frozen=True)
class SceneConfig:
    name: str
    resolution: int  # voxels per side (multiple of 32)
    num_spheres: int  # 0 = the single centred sphere of radius 0.5
    centre_range: float
    radius_range: tuple[float, float]
    background_radius: float | None  # inward-facing background sphere
    band_voxels: float  # keep voxels with |sdf(centre)| < band * voxel width
    noise_sigma: float
    sh_degree: int
    level_sets: tuple[float, ...]  # descending
    sharpness: float
    cameras: str  # "front", "orbit", "uneven", "ring"
    num_cameras: int
    image_shape: tuple[int, int]  # (H, W) for fixed-size camera sets
    fov_degrees: float | tuple[float, float]


def _even(lo: float, hi: float, n: int) -> tuple[float, ...]:
    if n == 1:
        return (0.5 * (lo + hi),)
    return tuple(float(hi - (hi - lo) * i / (n - 1)) for i in range(n))


CONFIGS: dict[str, SceneConfig] = {
    # 64^3 sphere, 3 shells, one 128^2 camera (the CPU-runnable configuration).
    "small": SceneConfig("small", 64, 0, 0.0, (0.5, 0.5), None, 2.0, 0.002, 0, (0.02, 0.0, -0.02), 50.0,
                         "front", 1, (128, 128), 60.0),
    # 256^3, union of 8 spheres, SH degree 3, 8 shells, 4 x 800^2 cameras.
    "mid": SceneConfig("mid", 256, 8, 0.6, (0.1, 0.3), None, 2.0, 0.001, 3, _even(-0.03, 0.03, 8), 50.0,
                       "orbit", 4, (800, 800), 50.0),
    # The mid scene with a band wide enough for its shells: a 4-voxel band
    # (|sdf| < 0.031 at the voxel centres) holds all 8 level sets in
    # [-0.03, 0.03], where the 2-voxel band of "mid" leaves two shells empty
    # and two nearly empty.
    "mid_band": SceneConfig("mid_band", 256, 8, 0.6, (0.1, 0.3), None, 4.0, 0.001, 3, _even(-0.03, 0.03, 8), 50.0,
                            "orbit", 4, (800, 800), 50.0),
    # The mid scene seen by 32 cameras of uneven resolution (200-1600 px per
    # side, fov 40-70 degrees) placed on the mid scene's orbit.
    "uneven": SceneConfig("uneven", 256, 8, 0.6, (0.1, 0.3), None, 2.0, 0.001, 3, _even(-0.03, 0.03, 8), 50.0,
                          "uneven", 32, (0, 0), (40.0, 70.0)),
    # 512^3, 32 spheres + background sphere, SH degree 3, 16 shells, 4 x 1297x840.
    "large": SceneConfig("large", 512, 32, 0.7, (0.05, 0.25), 0.95, 2.0, 0.001, 3, _even(-0.02, 0.02, 16), 50.0,
                         "ring", 4, (840, 1297), 55.0),
    # Resident scenes of the serving workload, 8 shells each; cameras come with
    # the requests: the mid scene's layout at 256^3 (two, different noise) and
    # at 128^3, and the large scene's layout (inside a background sphere) at
    # 512^3.
    "serve_256": SceneConfig("serve_256", 256, 8, 0.6, (0.1, 0.3), None, 2.0, 0.001, 3, _even(-0.03, 0.03, 8),
                             50.0, "orbit", 1, (256, 256), 50.0),
    "serve_128": SceneConfig("serve_128", 128, 8, 0.6, (0.1, 0.3), None, 2.0, 0.001, 3, _even(-0.03, 0.03, 8),
                             50.0, "orbit", 1, (256, 256), 50.0),
    "serve_512": SceneConfig("serve_512", 512, 32, 0.7, (0.05, 0.25), 0.95, 2.0, 0.001, 3, _even(-0.02, 0.02, 8),
                             50.0, "ring", 1, (256, 256), 55.0),
}


def sphere_layout(cfg: SceneConfig) -> tuple[np.ndarray, np.ndarray]:
    if cfg.num_spheres == 0:
        return np.zeros((1, 3), np.float32), np.array([cfg.radius_range[0]], np.float32)
    rng = np.random.default_rng(5)
    centres = rng.uniform(-cfg.centre_range, cfg.centre_range, (cfg.num_spheres, 3)).astype(np.float32)
    radii = rng.uniform(cfg.radius_range[0], cfg.radius_range[1], cfg.num_spheres).astype(np.float32)
    return centres, radii


def analytic_sdf(points: torch.Tensor, centres: torch.Tensor, radii: torch.Tensor,
                 background_radius: float | None) -> torch.Tensor:
    """Union (min) of spheres; optional inward-facing background sphere."""
    d = None
    for c, r in zip(centres, radii):
        di = torch.linalg.vector_norm(points - c, dim=-1) - r
        d = di if d is None else torch.minimum(d, di)
    if background_radius is not None:
        d = torch.minimum(d, background_radius - torch.linalg.vector_norm(points, dim=-1))
    return d


def make_occupancy(cfg: SceneConfig, device: torch.device | str = "cpu") -> torch.Tensor:
    """Packed int32 occupancy [n, n, n // 32] of the band around the surface."""
    n = cfg.resolution
    assert n % 32 == 0
    centres, radii = sphere_layout(cfg)
    centres_t = torch.from_numpy(centres).to(device)
    radii_t = torch.from_numpy(radii).to(device)
    width = 2.0 / n
    coords = (-1.0 + (torch.arange(n, device=device, dtype=torch.float32) + 0.5) * width)
    powers = (1 << torch.arange(32, device=device, dtype=torch.int64))
    packed = torch.empty((n, n, n // 32), dtype=torch.int32, device=device)
    # Slabs of i keep memory bounded at 512^3 with few launches.
    slab = max(1, (1 << 22) // (n * n))
    for i0 in range(0, n, slab):
        i1 = min(n, i0 + slab)
        z = coords[i0:i1, None, None].expand(i1 - i0, n, n)
        y = coords[None, :, None].expand(i1 - i0, n, n)
        x = coords[None, None, :].expand(i1 - i0, n, n)
        pts = torch.stack((x, y, z), dim=-1)
        d = analytic_sdf(pts, centres_t, radii_t, cfg.background_radius)
        occ = (d.abs() < cfg.band_voxels * width).reshape(i1 - i0, n, n // 32, 32)
        packed[i0:i1] = (occ.to(torch.int64) * powers).sum(-1).to(torch.uint32).view(torch.int32)
    return packed


def corner_sdf(cfg: SceneConfig, grid_vertices: torch.Tensor) -> torch.Tensor:
    """Analytic SDF at the grid corners (positions 2v - 1) plus N(0, sigma^2)."""
    centres, radii = sphere_layout(cfg)
    device = grid_vertices.device
    pts = 2.0 * grid_vertices - 1.0
    d = analytic_sdf(pts, torch.from_numpy(centres).to(device), torch.from_numpy(radii).to(device),
                     cfg.background_radius)
    noise = np.random.default_rng(0).normal(0.0, cfg.noise_sigma, grid_vertices.shape[0]).astype(np.float32)
    return (d + torch.from_numpy(noise).to(device)).contiguous()


def corner_sh(cfg: SceneConfig, num_vertices: int, device: torch.device | str = "cpu") -> torch.Tensor:
    """[C, G, 3]: DC terms U[0,1], higher orders N(0, 0.05^2)."""
    c = (cfg.sh_degree + 1) ** 2
    rng = np.random.default_rng(1)
    sh = np.empty((c, num_vertices, 3), np.float32)
    sh[0] = rng.uniform(0.0, 1.0, (num_vertices, 3))
    if c > 1:
        sh[1:] = rng.normal(0.0, 0.05, (c - 1, num_vertices, 3))
    return torch.from_numpy(sh).to(device)


def look_at(eye: np.ndarray, target=(0.0, 0.0, 0.0), up=(0.0, 1.0, 0.0)) -> np.ndarray:
    """OpenCV world->camera matrix (+Z forward, -Y up, +X right)."""
    eye = np.asarray(eye, np.float64)
    forward = np.asarray(target, np.float64) - eye
    forward /= np.linalg.norm(forward)
    right = np.cross(forward, np.asarray(up, np.float64))
    if np.linalg.norm(right) < 1e-8:
        right = np.cross(forward, np.array([0.0, 0.0, 1.0]))
    right /= np.linalg.norm(right)
    down = np.cross(forward, right)
    r = np.stack((right, down, forward), axis=0)  # rows: camera axes in world
    w2c = np.eye(4)
    w2c[:3, :3] = r
    w2c[:3, 3] = -r @ eye
    return w2c.astype(np.float32)


def pinhole(h: int, w: int, fov_degrees: float) -> np.ndarray:
    f = (w / 2.0) / math.tan(math.radians(fov_degrees) / 2.0)
    return np.array([[f, 0.0, w / 2.0], [0.0, f, h / 2.0], [0.0, 0.0, 1.0]], np.float32)


@dataclass
class CameraSet:
    extrinsics: np.ndarray  # [B, 4, 4] world->camera
    intrinsics: np.ndarray  # [B, 3, 3]
    image_shapes: list[tuple[int, int]]  # per camera (H, W)


def make_cameras(cfg: SceneConfig) -> CameraSet:
    rng = np.random.default_rng(2)
    ext, intr, shapes = [], [], []
    for b in range(cfg.num_cameras):
        if cfg.cameras == "front":
            eye = np.array([0.0, 0.0, 2.0])
            h, w = cfg.image_shape
            fov = cfg.fov_degrees
        elif cfg.cameras == "orbit":
            az = math.radians(rng.uniform(0.0, 360.0))
            el = math.radians(rng.uniform(10.0, 60.0))
            eye = 2.5 * np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
            h, w = cfg.image_shape
            fov = cfg.fov_degrees
        elif cfg.cameras == "uneven":
            az = math.radians(rng.uniform(0.0, 360.0))
            el = math.radians(rng.uniform(10.0, 60.0))
            eye = 2.5 * np.array([math.cos(el) * math.cos(az), math.sin(el), math.cos(el) * math.sin(az)])
            w = int(rng.integers(200, 1601))
            h = int(rng.integers(200, 1601))
            fov = float(rng.uniform(*cfg.fov_degrees))
        elif cfg.cameras == "ring":
            az = 2.0 * math.pi * b / cfg.num_cameras
            eye = 0.6 * np.array([math.cos(az), 0.0, math.sin(az)])
            h, w = cfg.image_shape
            fov = cfg.fov_degrees
        else:
            raise ValueError(cfg.cameras)
        ext.append(look_at(eye))
        intr.append(pinhole(h, w, fov))
        shapes.append((h, w))
    return CameraSet(np.stack(ext), np.stack(intr), shapes)


def make_target(num_cameras: int, h: int, w: int, device: torch.device | str = "cpu") -> torch.Tensor:
    rng = np.random.default_rng(3)
    return torch.from_numpy(rng.uniform(0.0, 1.0, (num_cameras, 3, h, w)).astype(np.float32)).to(device)


def level_sets(cfg: SceneConfig, device: torch.device | str = "cpu") -> torch.Tensor:
    return torch.tensor(cfg.level_sets, dtype=torch.float32, device=device)
