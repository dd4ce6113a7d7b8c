"""GB300 drop-in for the reference's ``triangle_extraction`` package.

Same public names, argument meanings, return types and autograd behaviour as
``triangle_extraction/__init__.py`` of dcharatan/meshtryoshka; every kernel is
a hand-written sm_103a CUDA kernel behind the C ABI (``libmtgb.so``).

Differences that do not change results:

* ``tessellate_voxels`` runs the vertex and face counting passes before any
  output is allocated and reads both totals in one device->host copy (the
  reference synchronises four times, ``__init__.py:93-142``).
* Scans are single-pass decoupled look-back kernels on caller-owned scratch.
"""

from __future__ import annotations

import logging
from typing import NamedTuple

import numpy as np
import torch
from torch import Tensor
from torch.profiler import record_function

from .. import _native as nt
from ..record import note

__all__ = [
    "Voxels",
    "Triangles",
    "DeferredSH",
    "extract_voxels",
    "tessellate_voxels",
    "compute_sdf_regularizers",
    "SDFRegularizerLosses",
    "pack_occupancy",
    "unpack_occupancy",
    "dilate_occupancy",
    "compute_exclusive_cumsum",
    "compute_vertex_occupancy",
    "count_occupancy",
    "create_voxels",
    "count_triangle_vertices",
    "create_triangle_vertices",
    "count_triangle_faces",
    "create_triangle_faces",
    "CreateTriangleVertices",
    "CreateTriangleVerticesResult",
    "CountTriangleFacesResult",
    "CreateTriangleFacesResult",
    "VertexOccupancyFnResult",
    "write_occupancy",
    "upscale_occupancy",
    "upscale_parameters",
    "UpscaledParameters",
    "get_occupancy_mesh",
    "Mesh",
    "index_vertices",
    "index_keys",
]


def _i32(t: Tensor, name: str) -> Tensor:
    if t.dtype != torch.int32:
        raise TypeError(f"{name} must be int32, got {t.dtype}")
    return t.contiguous()


def _f32(t: Tensor, name: str) -> Tensor:
    if t.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {t.dtype}")
    return t.contiguous()


# ---------------------------------------------------------------------------
# Packed occupancy (triangle_extraction/common.py:17-35). Elementwise tensor
# reshuffles; they are not on the per-step path.
# ---------------------------------------------------------------------------
def pack_occupancy(occupancy: Tensor) -> Tensor:
    """bool [i, j, k] -> int32 [i, j, k // 32]; bit b of word kp is voxel 32*kp + b."""
    assert occupancy.shape[-1] % 32 == 0
    i, j, k = occupancy.shape
    occupancy = occupancy.reshape(i, j, k // 32, 32)
    powers = 1 << torch.arange(32, device=occupancy.device, dtype=torch.int64)
    return (occupancy * powers).sum(dim=-1).type(torch.uint32).view(torch.int32)


def unpack_occupancy(packed_occupancy: Tensor) -> Tensor:
    """int32 [i, j, kp] -> bool [i, j, 32 * kp]."""
    occupancy = packed_occupancy.view(torch.int32)
    powers = 1 << torch.arange(32, device=occupancy.device, dtype=torch.int32)
    occupancy = occupancy[..., None] & powers
    i, j, kp, _ = occupancy.shape
    return occupancy.reshape(i, j, kp * 32).type(torch.bool)


# ---------------------------------------------------------------------------
# Scan (triangle_extraction/compute_exclusive_cumsum.py:19-21).
# ---------------------------------------------------------------------------
@record_function("compute_exclusive_cumsum")
def compute_exclusive_cumsum(x: Tensor) -> None:
    """In-place exclusive prefix sum of a contiguous int32 CUDA tensor."""
    if x.dtype != torch.int32 or not x.is_contiguous():
        raise TypeError("compute_exclusive_cumsum expects a contiguous int32 tensor")
    device = nt.require_cuda(x)
    n = x.numel()
    if n == 0:
        return
    ws_ptr, ws_bytes = nt.workspace(device).get(nt.library().mt_scan_workspace_bytes(n))
    nt.call("mt_exclusive_scan_i32", x.data_ptr(), n, ws_ptr, ws_bytes, nt.stream(device))


# ---------------------------------------------------------------------------
# Voxel extraction (triangle_extraction/__init__.py:31-62 and helpers).
# ---------------------------------------------------------------------------
class VertexOccupancyFnResult(NamedTuple):
    vertex_occupancy: Tensor  # [i+1, j+1, kp+1] int32
    vertex_counts: Tensor  # [(i+1)(j+1)(kp+1)+1] int32


class Voxels(NamedTuple):
    vertices: Tensor  # [vertex, 3] float32 in [0, 1]^3, ordered (k, j, i) / extent
    neighbors: Tensor  # [7, voxel] int32 (+x, +y, +z, +xy, +yz, +xz, +xyz)
    lower_corners: Tensor  # [4, voxel_and_subvoxel] int32 (origin, +x, +y, +z); -64 = invalid
    upper_corners: Tensor  # [4, voxel] int32 (+xyz, +yz, +xz, +xy)
    indices: Tensor  # [voxel] int32 linear grid index
    grid_shape: tuple[int, int, int]

    @property
    def num_vertices(self) -> int:
        return self.vertices.shape[0]

    @property
    def num_voxels(self) -> int:
        return self.upper_corners.shape[1]

    @property
    def num_subvoxels(self) -> int:
        return self.lower_corners.shape[1] - self.upper_corners.shape[1]


@record_function("compute_vertex_occupancy")
def compute_vertex_occupancy(occupancy: Tensor) -> VertexOccupancyFnResult:
    occupancy = _i32(occupancy, "occupancy")
    device = nt.require_cuda(occupancy)
    i, j, kp = occupancy.shape
    shape = (i + 1, j + 1, kp + 1)
    vertex_occupancy = torch.empty(shape, dtype=torch.int32, device=device)
    vertex_counts = torch.empty(((i + 1) * (j + 1) * (kp + 1) + 1,), dtype=torch.int32, device=device)
    nt.call(
        "mt_compute_vertex_occupancy",
        nt.ptr(occupancy), i, j, kp,
        vertex_occupancy.data_ptr(), vertex_counts.data_ptr(), nt.stream(device),
    )
    return VertexOccupancyFnResult(vertex_occupancy, vertex_counts)


@record_function("count_occupancy")
def count_occupancy(occupancy: Tensor) -> Tensor:
    occupancy = _i32(occupancy, "occupancy")
    device = nt.require_cuda(occupancy)
    i, j, kp = occupancy.shape
    counts = torch.empty(((i + 1) * (j + 1) * (kp + 1) + 1,), dtype=torch.int32, device=device)
    nt.call("mt_count_occupancy", nt.ptr(occupancy), i, j, kp, counts.data_ptr(), nt.stream(device))
    return counts


@record_function("create_voxels")
def create_voxels(
    occupancy: Tensor,
    voxel_offsets: Tensor,
    num_voxels: int,
    vertex_occupancy: Tensor,
    vertex_offsets: Tensor,
    num_vertices: int,
) -> Voxels:
    occupancy = _i32(occupancy, "occupancy")
    device = nt.require_cuda(occupancy)
    i, j, kp = occupancy.shape
    kw = dict(device=device)
    vertices = torch.empty((num_vertices, 3), dtype=torch.float32, **kw)
    neighbors = torch.empty((7, num_voxels), dtype=torch.int32, **kw)
    lower_corners = torch.empty((4, num_vertices), dtype=torch.int32, **kw)
    upper_corners = torch.empty((4, num_voxels), dtype=torch.int32, **kw)
    indices = torch.empty((num_voxels,), dtype=torch.int32, **kw)
    if num_voxels > 0:
        # Converted inputs are bound to names so they outlive the launch.
        voxel_offsets = _i32(voxel_offsets, "voxel_offsets")
        vertex_occupancy = _i32(vertex_occupancy, "vertex_occupancy")
        vertex_offsets = _i32(vertex_offsets, "vertex_offsets")
        nt.call(
            "mt_create_voxels",
            occupancy.data_ptr(),
            voxel_offsets.data_ptr(),
            vertex_occupancy.data_ptr(),
            vertex_offsets.data_ptr(),
            i, j, kp, num_voxels, num_vertices,
            vertices.data_ptr(), neighbors.data_ptr(), lower_corners.data_ptr(),
            upper_corners.data_ptr(), indices.data_ptr(), nt.stream(device),
        )
    return Voxels(vertices, neighbors, lower_corners, upper_corners, indices, (i, j, kp * 32))


@record_function("extract_voxels")
def extract_voxels(occupancy: Tensor) -> Voxels:
    """Packed occupancy [i, j, kp] -> sparse voxel topology (one host sync)."""
    occupancy = _i32(occupancy, "occupancy")
    i, j, kp = occupancy.shape
    logging.debug(f"Extracting voxels for grid with shape ({i}, {j}, {kp * 32}).")
    vertex_occupancy, vertex_counts = compute_vertex_occupancy(occupancy)
    voxel_counts = count_occupancy(occupancy)
    compute_exclusive_cumsum(vertex_counts)
    compute_exclusive_cumsum(voxel_counts)
    totals = torch.stack((vertex_counts[-1], voxel_counts[-1])).cpu()
    num_vertices, num_voxels = int(totals[0]), int(totals[1])
    shape = vertex_occupancy.shape
    return create_voxels(
        occupancy,
        voxel_counts[:-1].view(shape),
        num_voxels,
        vertex_occupancy,
        vertex_counts[:-1].view(shape),
        num_vertices,
    )


@record_function("dilate_occupancy")
def dilate_occupancy(occupancy: Tensor, dilation: int) -> Tensor:
    if dilation == 0:
        return occupancy.clone()
    assert 0 < dilation < 32
    occupancy = _i32(occupancy, "occupancy")
    device = nt.require_cuda(occupancy)
    out = torch.empty_like(occupancy)
    i, j, kp = occupancy.shape
    if out.numel() > 0:
        nt.call("mt_dilate_occupancy", occupancy.data_ptr(), i, j, kp, dilation, out.data_ptr(), nt.stream(device))
    return out


# ---------------------------------------------------------------------------
# Coarse-to-fine subdivision (tesseract.py:396-486), occupancy mesh and
# vertex de-duplication. These run at subdivision steps and in the viewer.
# ---------------------------------------------------------------------------
@record_function("write_occupancy")
def write_occupancy(voxel_indices: Tensor, packed_occupancy_shape: tuple[int, ...], min_shell: int,
                    max_shell: int) -> Tensor:
    """Packed occupancy with the bit of every triangle's voxel set
    (write_occupancy.py:22-46). ``min_shell`` / ``max_shell`` are accepted
    and unused, as in the reference kernel."""
    voxel_indices = _i32(voxel_indices, "voxel_indices")
    device = nt.require_cuda(voxel_indices)
    occupancy = torch.zeros(packed_occupancy_shape, dtype=torch.int32, device=device)
    n = voxel_indices.numel()
    if n > 0 and occupancy.numel() > 0:
        nt.call("mt_write_occupancy", voxel_indices.data_ptr(), n, occupancy.data_ptr(), occupancy.numel(),
                nt.stream(device))
    return occupancy


def _upscale_occupancy(occupancy: Tensor, mask: Tensor | None, target_shape: tuple[int, int, int]) -> Tensor:
    occupancy = _i32(occupancy, "occupancy")
    device = nt.require_cuda(occupancy)
    i, j, k_packed = occupancy.shape
    i_target, j_target, k_target = target_shape
    assert k_target % 32 == 0
    k_packed_target = k_target // 32
    assert i_target >= i and j_target >= j and k_packed_target >= k_packed
    out = torch.empty((i_target, j_target, k_packed_target), dtype=torch.int32, device=device)
    if out.numel() > 0:
        if mask is not None:
            mask = _i32(mask, "occupancy_to_upscale")
            if mask.shape != occupancy.shape:
                raise ValueError(f"occupancy_to_upscale shape {tuple(mask.shape)} != {tuple(occupancy.shape)}")
        nt.call("mt_upscale_occupancy", occupancy.data_ptr(), nt.ptr(mask), i, j, k_packed, i_target, j_target,
                k_packed_target, out.data_ptr(), nt.stream(device))
    return out


@record_function("upscale_occupancy")
def upscale_occupancy(occupancy: Tensor, target_shape: tuple[int, int, int]) -> Tensor:
    """[i, j, kp] -> [i', j', k'/32] with every extent at least the old one
    (upscale_occupancy.py:24-54)."""
    return _upscale_occupancy(occupancy, None, target_shape)


class UpscaledParameters(NamedTuple):
    signed_distances: Tensor  # [vertex] float32
    spherical_harmonics: Tensor  # [sh, vertex, 3]; a DeferredSH from tessellate_voxels_counted(defer_sh=True) float32
    occupancy: Tensor  # [i, j, k_packed] int32


@record_function("upscale_parameters")
@torch.no_grad()
def upscale_parameters(old_signed_distances: Tensor, old_spherical_harmonics: Tensor, old_occupancy: Tensor,
                       occupancy_to_upscale: Tensor, new_resolution: tuple[int, int, int]) -> UpscaledParameters:
    """Upscaled occupancy of ``old_occupancy & occupancy_to_upscale`` and the
    old vertices' parameters resampled trilinearly onto its vertices
    (upscale_parameters.py:35-99). One host read (the new vertex count)."""
    old_signed_distances = _f32(old_signed_distances, "old_signed_distances")
    old_spherical_harmonics = _f32(old_spherical_harmonics, "old_spherical_harmonics")
    old_occupancy = _i32(old_occupancy, "old_occupancy")
    device = nt.require_cuda(old_signed_distances, old_spherical_harmonics, old_occupancy)
    num_sh, num_old, _ = old_spherical_harmonics.shape
    if old_signed_distances.shape[0] != num_old:
        raise ValueError("old_signed_distances and old_spherical_harmonics disagree on the vertex count")

    # The AND of upscale_parameters.py:49 is applied to every word the
    # upscaling kernel reads.
    new_occupancy = _upscale_occupancy(old_occupancy, occupancy_to_upscale, new_resolution)

    old_vertex_occupancy, old_vertex_offsets = compute_vertex_occupancy(old_occupancy)
    compute_exclusive_cumsum(old_vertex_offsets)
    new_vertex_occupancy, new_vertex_offsets = compute_vertex_occupancy(new_occupancy)
    compute_exclusive_cumsum(new_vertex_offsets)
    num_vertices = int(new_vertex_offsets[-1].item())

    new_signed_distances = torch.empty((num_vertices,), dtype=torch.float32, device=device)
    new_spherical_harmonics = torch.empty((num_sh, num_vertices, 3), dtype=torch.float32, device=device)
    if num_vertices > 0:
        i1, j1, k1 = old_vertex_occupancy.shape
        i1n, j1n, k1n = new_vertex_occupancy.shape
        nt.call("mt_upscale_parameters", old_vertex_occupancy.data_ptr(), old_vertex_offsets.data_ptr(),
                nt.ptr(old_signed_distances), nt.ptr(old_spherical_harmonics), num_sh, num_old, i1, j1, k1,
                new_vertex_occupancy.data_ptr(), new_vertex_offsets.data_ptr(), i1n, j1n, k1n, num_vertices,
                new_signed_distances.data_ptr(), new_spherical_harmonics.data_ptr(), nt.stream(device))
    return UpscaledParameters(new_signed_distances, new_spherical_harmonics, new_occupancy)


class Mesh(NamedTuple):
    vertices: Tensor  # [triangle, 3, 3] float32 (xyz)
    colors: Tensor  # [triangle, 3] float32


@record_function("get_occupancy_mesh")
def get_occupancy_mesh(occupancy: Tensor, colors: Tensor) -> Mesh:
    """Two triangles per face between occupied and free voxels, coloured by
    ``colors[axis, side]`` (get_occupancy_mesh.py:32-80). One host read."""
    occupancy = _i32(occupancy, "occupancy")
    colors = _f32(colors, "colors")
    device = nt.require_cuda(occupancy, colors)
    if tuple(colors.shape) != (3, 2, 3):
        raise ValueError(f"colors must be [3, 2, 3], got {tuple(colors.shape)}")
    i, j, k_packed = occupancy.shape
    counts = torch.empty(((i + 1) * (j + 1) * (k_packed + 1) + 1,), dtype=torch.int32, device=device)
    nt.call("mt_count_occupancy_mesh_triangles", nt.ptr(occupancy), i, j, k_packed, counts.data_ptr(),
            nt.stream(device))
    compute_exclusive_cumsum(counts)
    num_triangles = int(counts[-1].item())
    vertices = torch.empty((num_triangles, 3, 3), dtype=torch.float32, device=device)
    triangle_colors = torch.empty((num_triangles, 3), dtype=torch.float32, device=device)
    if num_triangles > 0:
        nt.call("mt_create_occupancy_mesh_triangles", occupancy.data_ptr(), i, j, k_packed, counts.data_ptr(),
                num_triangles, colors.data_ptr(), vertices.data_ptr(), triangle_colors.data_ptr(),
                nt.stream(device))
    return Mesh(vertices, triangle_colors)


def _index_pairs(keys: Tensor, values: Tensor) -> Tensor:
    """Stable sort of (key, original index), then every index mapped to the
    first original index of its run of equal keys."""
    device = keys.device
    n = keys.numel()
    sorted_keys = torch.empty_like(keys)
    order = torch.empty_like(values)
    out = torch.empty((n,), dtype=torch.int32, device=device)
    ws_ptr, ws_bytes = nt.workspace(device).get(nt.library().mt_sort_pairs_workspace_bytes(n))
    nt.call("mt_sort_pairs_i64_i32", keys.data_ptr(), values.data_ptr(), sorted_keys.data_ptr(), order.data_ptr(), n,
            None, 0, 64, ws_ptr, ws_bytes, nt.stream(device))
    nt.call("mt_index_sorted_runs", sorted_keys.data_ptr(), order.data_ptr(), n, out.data_ptr(), nt.stream(device))
    return out


def index_keys(keys: Tensor) -> Tensor:
    """int32 [n]: for every key, the index of the first equal key
    (index_vertices.py:30-51)."""
    if keys.dtype != torch.int64:
        raise TypeError(f"keys must be int64, got {keys.dtype}")
    keys = keys.contiguous()
    device = nt.require_cuda(keys)
    (n,) = keys.shape
    if n == 0:
        return torch.empty((0,), dtype=torch.int32, device=device)
    if n > 2**31 - 1:
        raise ValueError("index_keys handles at most 2^31 - 1 keys")
    values = torch.empty((n,), dtype=torch.int32, device=device)
    nt.call("mt_iota_i32", n, values.data_ptr(), nt.stream(device))
    return _index_pairs(keys, values)


def index_vertices(points: Tensor, tol: float = 1e-5) -> Tensor:
    """int32 [vertex]: for every point, the index of the first point with the
    same quantized position round(points / tol) (index_vertices.py:6-27).

    Quantization is that of the reference on its CUDA device: the division
    by the Python scalar ``tol`` is a multiplication by the float32
    reciprocal of float32(tol), rounded half to even."""
    points = _f32(points, "points")
    device = nt.require_cuda(points)
    v, _ = points.shape
    if v == 0:
        raise RuntimeError("index_vertices: max() of an empty tensor (no points)")
    if v > 2**31 - 1:
        raise ValueError("index_vertices handles at most 2^31 - 1 points")
    inv_tol = float(np.float32(1.0) / np.float32(tol))
    quantized = torch.empty((v, 3), dtype=torch.int64, device=device)
    max_abs = torch.empty((1,), dtype=torch.int64, device=device)
    nt.call("mt_quantize_points", points.data_ptr(), v, inv_tol, quantized.data_ptr(), max_abs.data_ptr(),
            nt.stream(device))
    bits = (int(max_abs.item()) & 0xFFFFFFFFFFFFFFFF).bit_length() + 1
    if bits * 3 > 63:
        raise RuntimeError(f"need {bits*3} bits, exceed 63 bits total")
    keys = torch.empty((v,), dtype=torch.int64, device=device)
    values = torch.empty((v,), dtype=torch.int32, device=device)
    nt.call("mt_pack_point_keys", quantized.data_ptr(), v, bits, keys.data_ptr(), values.data_ptr(),
            nt.stream(device))
    return _index_pairs(keys, values)


# ---------------------------------------------------------------------------
# Per-step marching cubes.
# ---------------------------------------------------------------------------
@record_function("count_triangle_vertices")
def count_triangle_vertices(signed_distances: Tensor, lower_corners: Tensor, level_sets: Tensor) -> Tensor:
    signed_distances = _f32(signed_distances, "signed_distances")
    lower_corners = _i32(lower_corners, "lower_corners")
    level_sets = _f32(level_sets, "level_sets")
    device = nt.require_cuda(signed_distances, lower_corners, level_sets)
    (s,) = level_sets.shape
    _, g = lower_corners.shape
    counts = torch.empty((s * g + 1,), dtype=torch.int32, device=device)
    nt.call(
        "mt_count_triangle_vertices",
        nt.ptr(signed_distances), nt.ptr(lower_corners), g, nt.ptr(level_sets), s,
        counts.data_ptr(), nt.stream(device),
    )
    return counts


# The grid SH backward forms each vertex's SH gradient once into scratch
# (48 floats per vertex) and then gathers it per grid vertex; above this many
# bytes of scratch (2.8 M vertices) it runs its one-pass form instead, which
# forms a vertex's gradient once per list entry and needs no scratch (same
# values): at the 512^3 / 16-shell scene the scratch would hold 3.5 GB.
GRID_SH_BACKWARD_SCRATCH_LIMIT = 512 << 20


class DeferredSH:
    """Per-vertex SH coefficients that are never formed (not in the
    reference): stands where ``Triangles.spherical_harmonics`` holds the
    [C, V, 3] rows, and renders evaluate vertex colours straight from the
    grid coefficients through it (``evaluate``), forward and backward, with
    the same bits as the rows would give. Filled by ``CreateTriangleVertices``
    with ``defer_sh``: the vertices' source records and the per-grid-vertex
    contribution list that both backward passes use."""

    def __init__(self, grid_spherical_harmonics: Tensor):
        self.grid_spherical_harmonics = grid_spherical_harmonics
        self.vertex_sources: Tensor | None = None  # [3, V] int32 (origin, axis corner, bits of t)
        self.num_vertices: Tensor | None = None  # device int32 live count (capacity mode) or None
        self.list_offsets: Tensor | None = None  # [G + 1] int32
        self.contributions: Tensor | None = None  # [2V, 2] int32

    @property
    def shape(self) -> tuple[int, int, int]:
        c = self.grid_spherical_harmonics.shape[0]
        v = self.vertex_sources.shape[1] if self.vertex_sources is not None else 0
        return (c, v, 3)

    def evaluate(self, vertices: Tensor, extrinsics: Tensor, sh_degree: int) -> Tensor:
        """evaluate_spherical_harmonics(vertices, rows, extrinsics, sh_degree)."""
        return GridSHColors.apply(self.grid_spherical_harmonics, vertices, extrinsics, sh_degree, self)


class GridSHColors(torch.autograd.Function):
    """Vertex colours [B, V, 3] from the grid SH (create_triangle_vertices.py's
    SH interpolation followed by evaluate_spherical_harmonics.py:23-111, fused);
    the gradient goes straight to the grid SH."""

    @staticmethod
    def forward(ctx, grid_spherical_harmonics, vertices, extrinsics, sh_degree, deferred):
        with record_function("grid_sh_colors_forward"):
            gsh = _f32(grid_spherical_harmonics, "grid_spherical_harmonics")
            vertices = _f32(vertices, "vertices")
            extrinsics = _f32(extrinsics, "extrinsics")
            device = nt.require_cuda(gsh, vertices, extrinsics)
            c, g, _ = gsh.shape
            b = extrinsics.shape[0]
            v = vertices.shape[0]
            if deferred.vertex_sources.shape[1] != v:
                raise ValueError("vertices must have one row per deferred SH vertex")
            campos = torch.empty((b, 3), dtype=torch.float32, device=device)
            nt.call("mt_camera_positions", nt.ptr(extrinsics), b, nt.ptr(campos), nt.stream(device))
            colors = torch.empty((b, v, 3), dtype=torch.float32, device=device)
            nt.call("mt_grid_sh_colors", nt.ptr(gsh), c, g, nt.ptr(deferred.vertex_sources), v,
                    nt.ptr(deferred.num_vertices), nt.ptr(vertices), int(sh_degree), nt.ptr(campos), b,
                    nt.ptr(colors), nt.stream(device))
            ctx.save_for_backward(vertices, campos, colors)
            ctx.deferred = deferred
            ctx.gsh_shape = gsh.shape
            ctx.sh_degree = int(sh_degree)
            return colors

    @staticmethod
    def backward(ctx, grad_colors):
        with record_function("grid_sh_colors_backward"):
            vertices, campos, colors = ctx.saved_tensors
            d = ctx.deferred
            c, g, _ = ctx.gsh_shape
            device = vertices.device
            grad_gsh = torch.empty(ctx.gsh_shape, dtype=torch.float32, device=device)  # fully written
            v = vertices.shape[0]
            need = nt.library().mt_grid_sh_colors_backward_workspace_bytes(v)
            if need <= GRID_SH_BACKWARD_SCRATCH_LIMIT:
                ws_ptr, ws_bytes = nt.workspace(device).get(need)
            else:
                ws_ptr, ws_bytes = None, 0  # the one-pass form: no scratch
            nt.call("mt_grid_sh_colors_backward", nt.ptr(d.list_offsets), nt.ptr(d.contributions), g, v,
                    nt.ptr(vertices), c, ctx.sh_degree, nt.ptr(campos), campos.shape[0], nt.ptr(colors),
                    nt.ptr(grad_colors.contiguous()), nt.ptr(grad_gsh), nt.ptr(d.num_vertices), ws_ptr, ws_bytes,
                    nt.stream(device))
            return grad_gsh, None, None, None, None


class CreateTriangleVerticesResult(NamedTuple):
    vertices: Tensor
    signed_distances: Tensor
    spherical_harmonics: Tensor
    vertex_types: Tensor


class CreateTriangleVertices(torch.autograd.Function):
    """create_triangle_vertices.py:30-170: vertices on crossing edges, with the
    MC weight t detached (gradients reach both edge corners with (1-t, t)).

    ``live_t`` (not in the reference): t = (iso - d0) / (d1 - d0) is
    differentiated too, so the positions and SH of a vertex also depend on
    its corner SDFs through t, and its SDF (= the level set) on nothing."""

    @staticmethod
    def forward(ctx, grid_vertices, grid_signed_distances, grid_spherical_harmonics, voxel_lower_corners,
                level_sets, vertex_offsets, num_vertices=None, capacity=None, deferred=None, live_t=False):
        with record_function("create_triangle_vertices_forward"):
            grid_vertices = _f32(grid_vertices, "grid_vertices")
            grid_signed_distances = _f32(grid_signed_distances, "grid_signed_distances")
            grid_spherical_harmonics = _f32(grid_spherical_harmonics, "grid_spherical_harmonics")
            voxel_lower_corners = _i32(voxel_lower_corners, "voxel_lower_corners")
            level_sets = _f32(level_sets, "level_sets")
            vertex_offsets = _i32(vertex_offsets, "vertex_offsets")
            device = nt.require_cuda(grid_vertices, grid_signed_distances, grid_spherical_harmonics,
                                     voxel_lower_corners, level_sets, vertex_offsets)
            (s,) = level_sets.shape
            _, g = voxel_lower_corners.shape
            c = grid_spherical_harmonics.shape[0]
            if capacity is not None:
                # Buffers of `capacity` rows; the live count stays on the device
                # (the last vertex offset), so nothing is read back.
                v = int(capacity)
                count_ptr = vertex_offsets.data_ptr() + 4 * (vertex_offsets.numel() - 1)
            else:
                v = int(vertex_offsets[-1].item()) if num_vertices is None else int(num_vertices)
                count_ptr = None
            kw = dict(dtype=torch.float32, device=device)
            vertices = torch.empty((v, 3), **kw)
            sdf = torch.empty((v,), **kw)
            # Deferred SH: no rows (a [C, 0, 3] placeholder); colours come from
            # the grid through `deferred`.
            sh = torch.empty((c, 0 if deferred is not None else v, 3), **kw)
            types = torch.empty((v,), dtype=torch.uint8, device=device)
            sources = torch.empty((3, v), dtype=torch.int32, device=device)
            nt.call(
                "mt_create_triangle_vertices",
                nt.ptr(grid_vertices), nt.ptr(grid_signed_distances), nt.ptr(grid_spherical_harmonics), c,
                nt.ptr(voxel_lower_corners), g, nt.ptr(level_sets), s, nt.ptr(vertex_offsets), v, count_ptr,
                nt.ptr(vertices), nt.ptr(sdf), None if deferred is not None else nt.ptr(sh), nt.ptr(types),
                nt.ptr(sources), nt.stream(device), launches=1 if deferred is not None else None,
            )
            ctx.deferred = deferred is not None
            if deferred is not None:
                # The contribution list of the backward gather, built now so that
                # the colour backward and this Function's backward share it.
                inverse = torch.empty((4, g), dtype=torch.int32, device=device)
                offsets = torch.empty((g + 1,), dtype=torch.int32, device=device)
                contributions = torch.empty((2 * v, 2), dtype=torch.int32, device=device)
                ws_ptr, ws_bytes = nt.workspace(device).get(nt.library().mt_build_vertex_grad_list_workspace_bytes(g))
                nt.call("mt_build_vertex_grad_list", nt.ptr(grid_signed_distances), nt.ptr(voxel_lower_corners), g,
                        nt.ptr(level_sets), s, nt.ptr(vertex_offsets), v, nt.ptr(inverse), nt.ptr(offsets),
                        nt.ptr(contributions), ws_ptr, ws_bytes, nt.stream(device))
                deferred.vertex_sources = sources
                deferred.num_vertices = (vertex_offsets[-1:].view(()) if capacity is not None else None)
                deferred.list_offsets = offsets
                deferred.contributions = contributions
                ctx.list = (offsets, contributions)
                ctx.mark_non_differentiable(sh)
            ctx.save_for_backward(grid_signed_distances, voxel_lower_corners, level_sets, vertex_offsets)
            ctx.shapes = (grid_vertices.shape, grid_spherical_harmonics.shape, v)
            ctx.live_t = None
            if live_t:
                if deferred is not None:
                    raise ValueError("a live marching-cubes weight needs the per-vertex SH rows (no deferred SH)")
                ctx.live_t = (grid_vertices, grid_spherical_harmonics, sources, count_ptr is not None)
            ctx.mark_non_differentiable(types)
            ctx.set_materialize_grads(False)
            return vertices, sdf, sh, types

    @staticmethod
    def backward(ctx, grad_vertices, grad_signed_distances, grad_spherical_harmonics, grad_types):
        with record_function("create_triangle_vertices_backward"):
            grid_signed_distances, lower_corners, level_sets, vertex_offsets = ctx.saved_tensors
            gv_shape, gsh_shape, v = ctx.shapes
            device = grid_signed_distances.device
            g = lower_corners.shape[1]
            (s,) = level_sets.shape
            c = gsh_shape[0]
            # The kernel writes every entry of the grid gradients: one per grid
            # vertex, and every grid vertex is the origin of exactly one entry.
            if grid_signed_distances.shape[0] != g:
                raise ValueError("grid_signed_distances must have one value per voxel-lower-corner entry")
            grad_grid_vertices = torch.empty(gv_shape, dtype=torch.float32, device=device)
            grad_grid_sdf = torch.empty_like(grid_signed_distances)
            if ctx.deferred:
                # The SH gradient comes from the colour Function (GridSHColors).
                offsets, contributions = ctx.list
                gv = grad_vertices.contiguous() if grad_vertices is not None else None
                gd = grad_signed_distances.contiguous() if grad_signed_distances is not None else None
                nt.call("mt_vertex_grads_from_list", nt.ptr(offsets), nt.ptr(contributions), g, nt.ptr(gv),
                        nt.ptr(gd), nt.ptr(grad_grid_vertices), nt.ptr(grad_grid_sdf), nt.stream(device))
                return grad_grid_vertices, grad_grid_sdf, None, None, None, None, None, None, None, None
            grad_grid_sh = torch.empty(gsh_shape, dtype=torch.float32, device=device)
            inverse = torch.empty((4, g), dtype=torch.int32, device=device)
            gv = grad_vertices.contiguous() if grad_vertices is not None else None
            gd = grad_signed_distances.contiguous() if grad_signed_distances is not None else None
            gs = grad_spherical_harmonics.contiguous() if grad_spherical_harmonics is not None else None
            if ctx.live_t is not None:
                gd = None  # with t live, the vertex SDF is the level set: no gradient reaches the corners
            ws_ptr, ws_bytes = nt.workspace(device).get(
                nt.library().mt_create_triangle_vertices_backward_workspace_bytes(g, v))
            nt.call(
                "mt_create_triangle_vertices_backward",
                nt.ptr(grid_signed_distances), c, nt.ptr(lower_corners), g, nt.ptr(level_sets), s,
                nt.ptr(vertex_offsets), nt.ptr(gv), nt.ptr(gd), nt.ptr(gs), v, nt.ptr(inverse),
                nt.ptr(grad_grid_vertices), nt.ptr(grad_grid_sdf), nt.ptr(grad_grid_sh), ws_ptr, ws_bytes,
                nt.stream(device),
            )
            if ctx.live_t is not None:
                grid_vertices, grid_sh, sources, counted = ctx.live_t
                count_ptr = vertex_offsets.data_ptr() + 4 * (vertex_offsets.numel() - 1) if counted else None
                nt.call("mt_create_triangle_vertices_live_t_backward", nt.ptr(grid_vertices),
                        nt.ptr(grid_signed_distances), nt.ptr(grid_sh), c, g, nt.ptr(sources), v, count_ptr,
                        nt.ptr(gv), nt.ptr(gs), nt.ptr(grad_grid_sdf), nt.stream(device))
            return grad_grid_vertices, grad_grid_sdf, grad_grid_sh, None, None, None, None, None, None, None


def create_triangle_vertices(
    grid_vertices: Tensor,
    grid_signed_distances: Tensor,
    grid_spherical_harmonics: Tensor,
    voxel_lower_corners: Tensor,
    level_sets: Tensor,
    vertex_offsets: Tensor,
    num_vertices: int | None = None,
    capacity: int | None = None,
    deferred: DeferredSH | None = None,
    t_gradient: str = "detached",
) -> CreateTriangleVerticesResult:
    """``num_vertices`` (optional, not in the reference signature) skips the
    device->host read of ``vertex_offsets[-1]`` when the caller knows it.
    ``capacity`` (optional) sizes the outputs to a fixed row count instead and
    keeps the live count on the device; rows past it are unused.
    ``deferred`` (optional): the SH rows are not formed; ``deferred`` is filled
    for colour evaluation from the grid, and the result's
    ``spherical_harmonics`` is a [C, 0, 3] placeholder.
    ``t_gradient`` (not in the reference): "detached" (the reference's
    gradients) or "live" (the marching-cubes weight is differentiated as a
    function of the edge's two corner SDFs; needs the SH rows)."""
    if t_gradient not in ("detached", "live"):
        raise ValueError(f"t_gradient must be 'detached' or 'live', not {t_gradient!r}")
    result = CreateTriangleVertices.apply(
        grid_vertices, grid_signed_distances, grid_spherical_harmonics, voxel_lower_corners, level_sets,
        vertex_offsets, num_vertices, capacity, deferred, t_gradient == "live",
    )
    return CreateTriangleVerticesResult(*result)


class CountTriangleFacesResult(NamedTuple):
    # Field names and positional order are kept as in the reference
    # (count_triangle_faces.py:23-25, filled positionally at :63): the first
    # field holds the face counts, the second the cube codes.
    cell_codes: Tensor
    face_counts: Tensor


@record_function("count_triangle_faces")
def count_triangle_faces(
    signed_distances: Tensor, lower_corners: Tensor, upper_corners: Tensor, level_sets: Tensor
) -> CountTriangleFacesResult:
    signed_distances = _f32(signed_distances, "signed_distances")
    lower_corners = _i32(lower_corners, "lower_corners")
    upper_corners = _i32(upper_corners, "upper_corners")
    level_sets = _f32(level_sets, "level_sets")
    device = nt.require_cuda(signed_distances, lower_corners, upper_corners, level_sets)
    _, nv = upper_corners.shape
    _, g = lower_corners.shape
    (s,) = level_sets.shape
    codes = torch.empty((s, nv), dtype=torch.uint8, device=device)
    counts = torch.empty((s * nv + 1,), dtype=torch.int32, device=device)
    nt.call(
        "mt_count_triangle_faces",
        nt.ptr(signed_distances), nt.ptr(lower_corners), g, nt.ptr(upper_corners), nv, nt.ptr(level_sets), s,
        counts.data_ptr(), nt.ptr(codes), nt.stream(device),
    )
    return CountTriangleFacesResult(counts, codes)


class CreateTriangleFacesResult(NamedTuple):
    faces: Tensor
    voxel_indices: Tensor | None


@record_function("create_triangle_faces")
def create_triangle_faces(
    signed_distances: Tensor,
    neighbors: Tensor,
    indices: Tensor,
    vertex_offsets: Tensor,
    triangle_vertex_types: Tensor,
    voxel_cell_codes: Tensor,
    level_sets: Tensor,
    face_offsets: Tensor,
    num_faces: int | None = None,
    capacity: int | None = None,
) -> CreateTriangleFacesResult:
    """``capacity`` (optional) sizes the outputs to a fixed row count; faces
    past it are not written and nothing is read back."""
    device = nt.require_cuda(signed_distances, neighbors, indices, vertex_offsets, face_offsets)
    _, nv = neighbors.shape
    (s,) = level_sets.shape
    g = (vertex_offsets.shape[0] - 1) // s if s > 0 else 0
    if capacity is not None:
        f = int(capacity)
    else:
        f = int(face_offsets[-1].item()) // 3 if num_faces is None else int(num_faces)
    faces = torch.empty((f, 3), dtype=torch.int32, device=device)
    voxel_indices = torch.empty((f,), dtype=torch.int32, device=device)
    neighbors, indices = _i32(neighbors, "neighbors"), _i32(indices, "indices")
    vertex_offsets, face_offsets = _i32(vertex_offsets, "vertex_offsets"), _i32(face_offsets, "face_offsets")
    types, codes = triangle_vertex_types.contiguous(), voxel_cell_codes.contiguous()
    nt.call(
        "mt_create_triangle_faces",
        nt.ptr(neighbors), nt.ptr(indices), nv, g, types.shape[0], nt.ptr(vertex_offsets), nt.ptr(types),
        nt.ptr(codes), s,
        nt.ptr(face_offsets), f, nt.ptr(faces), nt.ptr(voxel_indices), nt.stream(device),
    )
    return CreateTriangleFacesResult(faces, voxel_indices)


class Triangles(NamedTuple):
    vertices: Tensor  # [vertex, 3]
    signed_distances: Tensor  # [vertex]
    spherical_harmonics: Tensor  # [sh, vertex, 3]
    faces: Tensor  # [face, 3] int32
    voxel_indices: Tensor  # [face] int32
    vertex_boundaries: Tensor  # [level_set] int32 (cumulative ends)
    face_boundaries: Tensor  # [level_set] int32 (cumulative ends)


# ---------------------------------------------------------------------------
# SDF regularizers (triangle_extraction/compute_sdf_regularizers.py:21-150)
# ---------------------------------------------------------------------------
class SDFRegularizerLosses(NamedTuple):
    eikonal_loss_pos: Tensor  # [voxel]
    eikonal_loss_neg: Tensor  # [voxel]
    curvature_loss: Tensor  # [voxel]


class ComputeSDFRegularizers(torch.autograd.Function):
    @staticmethod
    def forward(ctx, grid_signed_distances, voxel_neighbors, voxel_lower_corners, voxel_upper_corners, grid_size):
        with record_function("compute_sdf_regularizers_forward"):
            sdf = _f32(grid_signed_distances, "grid_signed_distances")
            neighbors = _i32(voxel_neighbors, "voxel_neighbors")
            lower, upper = _i32(voxel_lower_corners, "voxel_lower_corners"), _i32(voxel_upper_corners,
                                                                                 "voxel_upper_corners")
            device = nt.require_cuda(sdf, neighbors, lower, upper)
            _, g = lower.shape
            _, nv = upper.shape
            i, j, k = (int(x) for x in grid_size)
            kw = dict(dtype=torch.float32, device=device)
            pos, neg, curv = torch.empty((nv,), **kw), torch.empty((nv,), **kw), torch.empty((nv,), **kw)
            nt.call("mt_compute_sdf_regularizers", nt.ptr(sdf), nt.ptr(neighbors), nt.ptr(lower), g, nt.ptr(upper),
                    nv, k, j, i, nt.ptr(pos), nt.ptr(neg), nt.ptr(curv), nt.stream(device))
            ctx.save_for_backward(sdf, neighbors, lower, upper)
            ctx.grid_size = (i, j, k)
            ctx.set_materialize_grads(False)
            return pos, neg, curv

    @staticmethod
    def backward(ctx, grad_pos, grad_neg, grad_curv):
        with record_function("compute_sdf_regularizers_backward"):
            sdf, neighbors, lower, upper = ctx.saved_tensors
            i, j, k = ctx.grid_size
            _, g = lower.shape
            _, nv = upper.shape
            grad = torch.empty_like(sdf)  # fully written
            gp = grad_pos.contiguous() if grad_pos is not None else None
            gn = grad_neg.contiguous() if grad_neg is not None else None
            gc = grad_curv.contiguous() if grad_curv is not None else None
            nt.call("mt_compute_sdf_regularizers_backward", nt.ptr(sdf), nt.ptr(neighbors), nt.ptr(lower), g,
                    nt.ptr(upper), nv, k, j, i, nt.ptr(gp), nt.ptr(gn), nt.ptr(gc), nt.ptr(grad),
                    nt.stream(sdf.device))
            return grad, None, None, None, None


def compute_sdf_regularizers(grid_signed_distances: Tensor, voxel_neighbors: Tensor, voxel_lower_corners: Tensor,
                             voxel_upper_corners: Tensor, grid_size: tuple[int, int, int]) -> SDFRegularizerLosses:
    """Eikonal (split by sign) and curvature regularizers per voxel; grid_size
    is the voxel grid's (i, j, k) extent (the Eikonal gradient is scaled by
    (k, j, i) along (x, y, z))."""
    return SDFRegularizerLosses(*ComputeSDFRegularizers.apply(
        grid_signed_distances, voxel_neighbors, voxel_lower_corners, voxel_upper_corners, grid_size))


class TessellationCounts(NamedTuple):
    """Live sizes of a capacity-sized tessellation, as device scalars."""

    num_vertices: Tensor  # [] int32
    num_faces: Tensor  # [] int32


@record_function("tessellate_voxels")
def tessellate_voxels(
    signed_distances: Tensor,
    vertices: Tensor,
    spherical_harmonics: Tensor,
    neighbors: Tensor,
    lower_corners: Tensor,
    upper_corners: Tensor,
    indices: Tensor,
    level_sets: Tensor,
    t_gradient: str = "detached",
    defer_sh: bool = False,
) -> Triangles:
    """Marching cubes over every level set (triangle_extraction/__init__.py:75-157).

    Differentiable with respect to ``signed_distances`` and
    ``spherical_harmonics`` (and ``vertices``) through the triangle vertices'
    signed distances / colours, exactly as the reference.

    ``t_gradient`` (not in the reference): "live" also differentiates each
    vertex's edge-crossing weight t = (iso - d0) / (d1 - d0) as a function of
    its two corner SDFs (topology stays fixed); the default "detached" gives
    the reference's gradients.

    ``defer_sh`` (not in the reference): ``Triangles.spherical_harmonics`` is
    a ``DeferredSH`` instead of the [C, V, 3] rows, as in
    ``tessellate_voxels_counted`` (same colours and gradients; the rows are
    neither written nor read). Applies when the level sets are at most
    ``mt_vertex_grad_list_max_shells()``.
    """
    defer = defer_sh and level_sets.shape[0] <= nt.library().mt_vertex_grad_list_max_shells()
    triangles, _ = _tessellate(signed_distances, vertices, spherical_harmonics, neighbors, lower_corners,
                               upper_corners, indices, level_sets, None, defer, t_gradient=t_gradient)
    return triangles


def tessellate_voxels_counted(
    signed_distances: Tensor,
    vertices: Tensor,
    spherical_harmonics: Tensor,
    neighbors: Tensor,
    lower_corners: Tensor,
    upper_corners: Tensor,
    indices: Tensor,
    level_sets: Tensor,
    vertex_capacity: int,
    face_capacity: int,
    defer_sh: bool = False,
) -> tuple[Triangles, TessellationCounts]:
    """tessellate_voxels without any device->host read, for CUDA-graph capture.

    Not in the reference. The outputs have ``vertex_capacity`` / ``face_capacity``
    rows; the live counts are returned as device scalars. Rows past the live
    counts are unused (faces never name them). When a live count exceeds its
    capacity the extra vertices / faces are dropped; callers compare the counts
    with the capacities (see ``meshtryoshka_gb300.graph``).

    ``defer_sh``: ``Triangles.spherical_harmonics`` is a ``DeferredSH`` instead
    of the [C, V, 3] rows; the render entry points evaluate colours from the
    grid through it (same values, no rows written or read). Applies when the
    level sets are at most ``mt_vertex_grad_list_max_shells()``; otherwise the
    rows are formed as usual.
    """
    defer = defer_sh and level_sets.shape[0] <= nt.library().mt_vertex_grad_list_max_shells()
    return _tessellate(signed_distances, vertices, spherical_harmonics, neighbors, lower_corners, upper_corners,
                       indices, level_sets, (int(vertex_capacity), int(face_capacity)), defer)


def _tessellate(signed_distances, vertices, spherical_harmonics, neighbors, lower_corners, upper_corners, indices,
                level_sets, capacity, defer_sh=False, t_gradient="detached"):
    (num_level_sets,) = level_sets.shape
    device = nt.require_cuda(signed_distances, lower_corners, level_sets)
    logging.debug(f"Tessellating {neighbors.shape[1]} voxels with {num_level_sets} level sets.")
    _, g = lower_corners.shape
    _, nv = upper_corners.shape

    with torch.no_grad():
        vertex_offsets = count_triangle_vertices(signed_distances, lower_corners, level_sets)
        compute_exclusive_cumsum(vertex_offsets)
        face_offsets, voxel_cell_codes = count_triangle_faces(signed_distances, lower_corners, upper_corners,
                                                              level_sets)
        compute_exclusive_cumsum(face_offsets)
        if capacity is None:
            # One device->host read for both totals (and the scan status word).
            totals = torch.stack((vertex_offsets[-1], face_offsets[-1])).cpu()
            nt.workspace(device).check()
            num_vertices, num_faces = int(totals[0]), int(totals[1]) // 3
            counts = None
        else:
            num_vertices, num_faces = capacity
            counts = TessellationCounts(vertex_offsets[-1], torch.empty((), dtype=torch.int32, device=device))

    deferred = DeferredSH(spherical_harmonics) if defer_sh else None
    triangle_vertices, triangle_sdf, triangle_sh, triangle_types = create_triangle_vertices(
        vertices, signed_distances, spherical_harmonics, lower_corners, level_sets, vertex_offsets,
        num_vertices if capacity is None else None, None if capacity is None else num_vertices, deferred,
        t_gradient=t_gradient,
    )
    if deferred is not None:
        triangle_sh = deferred

    with torch.no_grad():
        faces, voxel_indices = create_triangle_faces(
            signed_distances, neighbors, indices, vertex_offsets, triangle_types, voxel_cell_codes, level_sets,
            face_offsets, num_faces if capacity is None else None, None if capacity is None else num_faces,
        )
        # vertex_offsets[1:].view(S, -1)[:, -1] and face_offsets[...] // 3 (and
        # the counted face total) in one launch.
        vertex_boundaries = torch.empty((num_level_sets,), dtype=torch.int32, device=device)
        face_boundaries = torch.empty((num_level_sets,), dtype=torch.int32, device=device)
        nt.call("mt_shell_boundaries", vertex_offsets.data_ptr(), g, face_offsets.data_ptr(), nv, num_level_sets,
                vertex_boundaries.data_ptr(), face_boundaries.data_ptr(),
                counts.num_faces.data_ptr() if counts is not None else None, nt.stream(device))

    logging.debug(f"Created {num_vertices} vertices and {num_faces} faces.")
    note(vertex_offsets=vertex_offsets, face_offsets=face_offsets, faces=faces, voxel_indices=voxel_indices,
         vertex_boundaries=vertex_boundaries, face_boundaries=face_boundaries, triangle_vertices=triangle_vertices,
         triangle_signed_distances=triangle_sdf)
    return Triangles(triangle_vertices, triangle_sdf, triangle_sh, faces, voxel_indices, vertex_boundaries,
                     face_boundaries), counts
