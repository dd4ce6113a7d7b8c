"""Scenes from the reference trainer's checkpoints.

The reference trainer saves ``torch.save({"model": state_dict, ...})``
(meshtryoshka/trainer.py:111-120). The scene lives in the model's
``tesseract`` module (meshtryoshka/model/tesseract.py:151-256):

* ``tesseract.occupancy``: int32 words of every component's packed occupancy
  grid, back to back (the central cube, then six arms when the tesseract has
  arms);
* ``tesseract.signed_distances_raw`` [G] and ``tesseract.sh_rgb`` [1, G, 3],
  ``tesseract.sh_rest`` [C - 1, G, 3] (a 0-d placeholder at SH degree 0): one
  entry per grid vertex of the concatenated components;
* ``tesseract.step``: the training step, which selects the resolutions of the
  trainer's schedules.

The grid's geometry (the components' resolutions at that step, the central
cube's share of the contracted volume, whether the arms are disabled) and the
contraction come from the trainer's configuration, not from the checkpoint;
``TesseractLayout`` and ``Contraction`` carry them.

The voxels are assembled as the reference's ``Tesseract.extract_voxels``
does (tesseract.py:347-377): each component's slice of the occupancy goes
through ``extract_voxels`` (the CUDA path), its [0, 1]^3 vertices are mapped
trilinearly onto the component's eight corners (tesseract.py:29-41, 72-142),
the components' voxels are concatenated with their neighbour and corner
indices offset (tesseract.py:262-327), and the corners of duplicate vertices
are pointed at the first copy (``index_vertices`` at tolerance 1e-6,
tesseract.py:520-526). Renderer positions are the contraction's inverse of
the tessellated vertices (contraction.py:65-108).
"""

from __future__ import annotations

from dataclasses import dataclass
from math import exp, prod

import torch
from torch import Tensor

from . import triangle_extraction as te


@dataclass(frozen=True)
class TesseractLayout:
    """Grid geometry of a tesseract at one training step."""

    center_resolution: int  # the central cube's resolution at the step
    arm_resolution: int  # the arms' resolution at the step (0: no arms)
    center_extent: float  # the central cube's share of the contracted [0, 1]^3 cube
    disable_tesseract: bool = False  # one cube over the whole volume (no arms)

    def components(self) -> list[tuple[str, int, int]]:
        """(kind, dimension, direction) of each component, in storage order."""
        out = [("center", -1, -1)]
        if self.arm_resolution > 0 and not self.disable_tesseract:
            out += [("arm", d, s) for d in range(3) for s in range(2)]
        return out

    def shape(self, component: tuple[str, int, int]) -> tuple[int, int, int]:
        kind, dim, _ = component
        c = self.center_resolution
        if kind == "center":
            if self.disable_tesseract:
                c += 2 * self.arm_resolution
            return (c, c, c)
        shape = [c, c, c]
        shape[dim] = self.arm_resolution
        return tuple(shape)

    @property
    def extent(self) -> tuple[int, int, int]:
        e = self.center_resolution + 2 * self.arm_resolution
        return (e, e, e)


def unit_corners(device) -> Tensor:
    """int32 [2, 2, 2, 3]: corner (i, j, k) of the unit cube at (x, y, z) = (k, j, i)."""
    r = torch.arange(2, dtype=torch.int32, device=device)
    i, j, k = torch.meshgrid(r, r, r, indexing="ij")
    return torch.stack((k, j, i), dim=-1)


def component_corners(layout: TesseractLayout, component: tuple[str, int, int], device) -> Tensor:
    """float32 [2, 2, 2, 3]: where the component's unit-cube corners sit in the
    contracted [0, 1]^3 volume (tesseract.py:94-142). The central cube spans
    [0.5 - e / 2, 0.5 + e / 2]^3; an arm is the frustum between one face of
    the central cube and the matching face of the unit cube."""
    extent = torch.tensor(1.0 if layout.disable_tesseract else layout.center_extent)
    low = 0.5 - 0.5 * extent
    high = 0.5 + 0.5 * extent
    unit = unit_corners(extent.device)
    corners = low + (high - low) * unit
    kind, dim, direction = component
    if kind == "arm":
        corners = corners.flip(dim)
        index = [slice(None)] * 3
        index[dim] = direction
        corners[tuple(index)] = unit[tuple(index)].to(corners.dtype)
    return corners.to(device)


def map_to_component(xyz: Tensor, corners: Tensor) -> Tensor:
    """Trilinear map of points in [0, 1]^3 onto a component's corners
    (tesseract.py:29-41, 72-79): the weight of corner c is
    prod_axis (c_axis xyz_axis + (1 - xyz_axis)(1 - c_axis))."""
    unit = unit_corners(xyz.device)
    p = xyz[..., None, None, None, :]
    weights = (unit * p + (1 - p) * (1 - unit)).prod(dim=-1)
    return torch.einsum("...ijk,ijkx->...x", weights, corners.to(xyz.device))


def concatenate_voxels(parts: list[te.Voxels]) -> te.Voxels:
    """The components' voxels as one grid (tesseract.py:262-327): every
    component's voxels, then every component's subvoxels; neighbour indices
    (voxel or subvoxel ids) and corner indices (vertex ids) offset to match,
    grid indices offset by the preceding components' cell counts."""
    num_voxels = sum(v.num_voxels for v in parts)
    vertex_offset = voxel_offset = subvoxel_offset = grid_offset = 0
    neighbors, voxel_lower, subvoxel_lower, upper, indices = [], [], [], [], []
    for v in parts:
        is_sub = v.neighbors >= v.num_voxels
        n = v.neighbors.clone()
        n[is_sub] += subvoxel_offset + num_voxels - v.num_voxels
        n[~is_sub] += voxel_offset
        neighbors.append(n)
        voxel_lower.append(v.lower_corners[:, : v.num_voxels] + vertex_offset)
        subvoxel_lower.append(v.lower_corners[:, v.num_voxels:] + vertex_offset)
        upper.append(v.upper_corners + vertex_offset)
        indices.append(v.indices + grid_offset)
        vertex_offset += v.num_vertices
        voxel_offset += v.num_voxels
        subvoxel_offset += v.num_subvoxels
        grid_offset += prod(v.grid_shape)
    return te.Voxels(torch.cat([v.vertices for v in parts], dim=0), torch.cat(neighbors, dim=1),
                     torch.cat((*voxel_lower, *subvoxel_lower), dim=1), torch.cat(upper, dim=1),
                     torch.cat(indices, dim=0), (0, 0, 0))


def tesseract_voxels(occupancy: Tensor, layout: TesseractLayout) -> tuple[te.Voxels, tuple[int, ...]]:
    """The tesseract's voxels from its flat occupancy words (on a CUDA
    device): the assembled grid and each component's first vertex index."""
    parts, counts = [], [0]
    start = 0
    for component in layout.components():
        i, j, k = layout.shape(component)
        words = i * j * k // 32
        occ = occupancy[start:start + words].view(i, j, k // 32)
        start += words
        v = te.extract_voxels(occ)
        v = v._replace(vertices=map_to_component(v.vertices, component_corners(layout, component, occ.device)))
        parts.append(v)
        counts.append(counts[-1] + v.num_vertices)
    if start != occupancy.numel():
        raise ValueError(f"occupancy holds {occupancy.numel()} words, the layout {start}")
    voxels = concatenate_voxels(parts)._replace(grid_shape=layout.extent)
    first = te.index_vertices(voxels.vertices, 1e-6).to(torch.int32)
    # As in the reference, the corner tables index the representative table
    # directly: a missing corner's -64 marker indexes from the end
    # (tesseract.py:522-525).
    voxels = voxels._replace(lower_corners=first[voxels.lower_corners.long()].contiguous(),
                             upper_corners=first[voxels.upper_corners.long()].contiguous())
    return voxels, tuple(counts)


@dataclass(frozen=True)
class Contraction:
    """The reference's scene contraction (contraction.py:9-108): points within
    [-center_radius, center_radius]^3 scale linearly into the central cube,
    the rest are compressed exponentially along their largest axis."""

    center_radius: float
    arm_ratio: float
    center_extent: float
    disable_exponential: bool = False

    @torch.no_grad()
    def uncontract(self, xyz: Tensor) -> Tensor:
        """Contracted [0, 1]^3 positions -> world positions (contraction.py:65-108)."""
        xyz = xyz.clip(min=0, max=1) * 2 - 1
        if self.disable_exponential:
            return xyz * exp(2 * self.arm_ratio)
        e = self.center_extent
        inside = (xyz.abs() <= e).all(dim=-1)
        t_c = (xyz.abs().max(dim=-1).values - e) / (1 - e)
        far_ratio = exp(2 * self.arm_ratio)
        t_u = ((2 * t_c * self.arm_ratio).exp() - 1) / (far_ratio - 1)
        far_u = far_ratio * self.center_radius
        outer = xyz * ((far_u * t_u + self.center_radius * (1 - t_u)) / (t_c + e * (1 - t_c)))[..., None]
        return torch.where(inside[..., None], xyz * self.center_radius / e, outer)


@dataclass
class CheckpointScene:
    voxels: te.Voxels
    signed_distances: Tensor  # [G] float32
    spherical_harmonics: Tensor  # [C, G, 3] float32
    sh_degree: int
    step: int
    vertex_boundaries: tuple[int, ...]


def load_tesseract_checkpoint(path, layout: TesseractLayout, device, sdf_offset=None) -> CheckpointScene:
    """Loads a reference trainer checkpoint's scene onto ``device``.

    ``sdf_offset``: optional callable (raw SDF [G], grid vertices [G, 3] in
    [0, 1]^3) -> SDF, the initializer's modification that the reference adds
    on every read (e.g. ``sphere_initializer(radius)``; the point-cloud
    initializer adds nothing once its steps are over). None: the raw values.
    """
    content = torch.load(path, map_location="cpu", weights_only=True)
    state = content["model"] if "model" in content else content
    prefix = "tesseract."
    occupancy = state[prefix + "occupancy"].to(device=device, dtype=torch.int32).contiguous()
    voxels, boundaries = tesseract_voxels(occupancy, layout)
    sdf = state[prefix + "signed_distances_raw"].to(device=device, dtype=torch.float32)
    if sdf.shape[0] != voxels.num_vertices:
        raise ValueError(f"{sdf.shape[0]} signed distances for {voxels.num_vertices} grid vertices: the layout "
                         "does not match the checkpoint")
    if sdf_offset is not None:
        sdf = sdf_offset(sdf, voxels.vertices)
    rgb = state[prefix + "sh_rgb"].to(device=device, dtype=torch.float32)
    rest = state.get(prefix + "sh_rest")
    sh = rgb if rest is None or rest.dim() != 3 or rest.shape[0] == 0 else torch.cat(
        (rgb, rest.to(device=device, dtype=torch.float32)), dim=0)
    c = sh.shape[0]
    degree = {1: 0, 4: 1, 9: 2, 16: 3}.get(c)
    if degree is None:
        raise ValueError(f"{c} SH coefficients per vertex is not a full degree")
    step = int(state.get(prefix + "step", torch.tensor(0)))
    return CheckpointScene(voxels, sdf.contiguous(), sh.contiguous(), degree, step, boundaries)


def sphere_initializer(radius: float):
    """The sphere initializer's modification (initializer/initializer_sphere.py:25-31):
    raw + |x - 0.5| - radius."""
    def offset(sdf: Tensor, xyz: Tensor) -> Tensor:
        return sdf + (xyz - 0.5).norm(dim=-1) - radius

    return offset
