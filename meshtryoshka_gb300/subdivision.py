"""Coarse-to-fine subdivision of a voxel grid's parameters.

The reference subdivides inside ``Tesseract.set_step``
(meshtryoshka/model/tesseract.py:396-486). For each grid component it

1. copies every vertex's parameters from its canonical duplicate
   (``index_vertices(voxels.vertices, 1e-6)``, :432-434),
2. marks the voxels that hold a triangle of the current mesh
   (``write_occupancy(scene.voxel_indices, ...)``, :443-448),
3. dilates that mask by 4 voxels (:464-466), and
4. upscales the occupancy inside the mask and resamples the signed
   distances and SH onto the finer grid (``upscale_parameters``, :469-475).

``subdivide`` is that sequence for one component, on the library's kernels;
the trainer-side bookkeeping (optimizer state, SH degree schedule, component
boundaries) stays with the caller.
"""

from __future__ import annotations

import torch
from torch import Tensor

from . import triangle_extraction as te


@torch.no_grad()
def subdivide(voxels: te.Voxels, signed_distances: Tensor, spherical_harmonics: Tensor, occupancy: Tensor,
              triangle_voxel_indices: Tensor, new_resolution: tuple[int, int, int], dilation: int = 4,
              disable_sparsity: bool = False, tol: float = 1e-6) -> te.UpscaledParameters:
    """One component's subdivision step (tesseract.py:432-475).

    ``voxels`` / ``occupancy`` describe the current grid, ``signed_distances``
    [V] and ``spherical_harmonics`` [C, V, 3] its vertex parameters, and
    ``triangle_voxel_indices`` the voxel of every triangle of the current
    mesh (``Triangles.voxel_indices``)."""
    canonical = te.index_vertices(voxels.vertices, tol).long()
    signed_distances = signed_distances[canonical]
    spherical_harmonics = spherical_harmonics[:, canonical, :]
    to_upscale = te.write_occupancy(triangle_voxel_indices, tuple(occupancy.shape), 0, 1)
    if disable_sparsity:
        to_upscale = torch.full_like(to_upscale, -1)
    to_upscale = te.dilate_occupancy(to_upscale, dilation)
    return te.upscale_parameters(signed_distances, spherical_harmonics, occupancy, to_upscale, new_resolution)
