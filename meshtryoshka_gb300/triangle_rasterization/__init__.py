"""GB300 drop-in for the reference's ``triangle_rasterization`` package.

Same public names, argument meanings, return types and autograd behaviour as
``triangle_rasterization/__init__.py`` of dcharatan/meshtryoshka (``render``,
``render_fused``, ``render_explicit``, ``rasterize`` and the per-stage
functions), backed by hand-written sm_103a kernels through the C ABI.

Gradient routing. The reference's adjoints route two gradients differently
from the exact derivative of its forward pass (the fused compositor scatters
the outer hit's deferred gradient with the current hit's barycentric weights;
the explicit compositor writes the outer / last shell's signed-distance
gradient to slots ``shell_index - 1`` / ``num_shells - 1``). The default,
``"reference"``, reproduces those routings bit-for-bit in structure so
gradients match the reference; ``"exact"`` uses the true adjoint (checked
against finite differences). Select with :func:`set_gradient_mode` or the
``gradient_mode=`` keyword of :func:`render`.
"""

from __future__ import annotations

import contextlib
import ctypes
from collections import OrderedDict
from dataclasses import dataclass
from math import prod
from typing import Literal, NamedTuple

import torch
from torch import Tensor
from torch.profiler import record_function

from .. import _native as nt
from ..record import note

__all__ = [
    "render",
    "render_fused",
    "render_cameras",
    "split_cameras",
    "render_fused_loss",
    "IntersectCompositeLoss",
    "render_explicit",
    "rasterize",
    "TileGrid",
    "create_key_defines",
    "ProjectedVertices",
    "project_vertices",
    "TriangleBounds",
    "bound_triangles",
    "PairedKeys",
    "generate_keys",
    "bound_and_generate_keys",
    "sort_keys",
    "delineate_tiles",
    "evaluate_spherical_harmonics",
    "EvaluateSphericalHarmonics",
    "intersect_and_composite",
    "IntersectAndComposite",
    "RenderedImages",
    "intersect",
    "interpolate",
    "Interpolate",
    "composite",
    "Composite",
    "set_gradient_mode",
    "gradient_mode",
]

_GRADIENT_MODE = "reference"

# Sizes of the most recent render (host integers already known to the
# wrapper; no extra synchronisation).
LAST_RENDER_STATS: dict[str, int] = {}


def set_gradient_mode(mode: Literal["reference", "exact"]) -> None:
    """Select the compositors' gradient routing (see the module docstring)."""
    global _GRADIENT_MODE
    if mode not in ("reference", "exact"):
        raise ValueError(f"unknown gradient mode {mode!r}")
    _GRADIENT_MODE = mode


@contextlib.contextmanager
def gradient_mode(mode: Literal["reference", "exact"]):
    previous = _GRADIENT_MODE
    set_gradient_mode(mode)
    try:
        yield
    finally:
        set_gradient_mode(previous)


def ceildiv(numerator, denominator):
    return (numerator + denominator - 1) // denominator


# ---------------------------------------------------------------------------
# Tiling and key layout (triangle_rasterization/common.py:15-44, keys.py:4-22)
# ---------------------------------------------------------------------------
@dataclass(frozen=True)
class TileGrid:
    tile_shape: tuple[int, int]  # (height, width) of one tile in pixels
    image_shape: tuple[int, int]  # (height, width) of the image (the largest, with camera_shapes)
    num_cameras: int
    num_shells: int
    # Not in the reference: per-camera image shapes for a batch of cameras of
    # different sizes. Each camera gets its own grid of tiles; keys carry the
    # camera-local tile index and tile ranges keep the [B, rows*cols, 2] shape
    # of the largest grid.
    camera_shapes: tuple[tuple[int, int], ...] | None = None
    # Not in the reference: threads per CTA of the compositing kernels'
    # persistent warps (128, 256 or 512; the reference runs one tile of
    # TILE_H x TILE_W threads per CTA). A third element of ``tile_shape``
    # sets it: (height, width, threads). Results do not depend on it.
    cta_threads: int = 256

    def __post_init__(self):
        shape = tuple(int(x) for x in self.tile_shape)
        if len(shape) == 3:
            object.__setattr__(self, "cta_threads", shape[2])
            shape = shape[:2]
        if len(shape) != 2 or self.cta_threads not in (128, 256, 512):
            raise ValueError(f"tile_shape must be (height, width) or (height, width, 128 | 256 | 512 threads), "
                             f"not {self.tile_shape}")
        object.__setattr__(self, "tile_shape", shape)

    @staticmethod
    def for_cameras(tile_shape, camera_shapes, num_shells) -> "TileGrid":
        shapes = tuple((int(h), int(w)) for h, w in camera_shapes)
        image = (max(h for h, _ in shapes), max(w for _, w in shapes))
        return TileGrid(tuple(tile_shape), image, len(shapes), num_shells, shapes)  # cta_threads from tile_shape

    @property
    def grid_shape(self) -> tuple[int, int]:
        return tuple(ceildiv(i, t) for i, t in zip(self.image_shape, self.tile_shape))

    @property
    def num_tiles_per_image(self) -> int:
        return prod(self.grid_shape)

    @property
    def tile_numel(self) -> int:
        h, w = self.tile_shape
        return h * w

    @property
    def ragged(self) -> bool:
        return self.camera_shapes is not None

    def camera_grids(self) -> list[tuple[int, int]]:
        shapes = self.camera_shapes or ((self.image_shape,) * self.num_cameras)
        return [(ceildiv(h, self.tile_shape[0]), ceildiv(w, self.tile_shape[1])) for h, w in shapes]

    @property
    def camera_tiles(self) -> int:
        return sum(r * c for r, c in self.camera_grids())

    @property
    def output_numel(self) -> int:
        shapes = self.camera_shapes or ((self.image_shape,) * self.num_cameras)
        return sum(4 * h * w for h, w in shapes)


_CAMERA_TABLES: "OrderedDict" = OrderedDict()
_CAMERA_TABLES_MAX = 256


def _camera_table(grid: TileGrid, device) -> Tensor | None:
    """Device table [B, 6] int64 (rows, cols, height, width, first tile, first
    output element) of a ragged grid; None for a uniform one. Built once per
    grid and device and kept in a bounded most-recently-used cache, so repeated
    calls (and CUDA-graph capture) copy nothing; whoever captures a graph keeps
    its own reference to the tables the graph reads (see graph.py)."""
    if not grid.ragged:
        return None
    key = (grid, str(device))
    table = _CAMERA_TABLES.get(key)
    if table is not None:
        _CAMERA_TABLES.move_to_end(key)
    else:
        rows = []
        tile = out = 0
        for (h, w), (r, c) in zip(grid.camera_shapes, grid.camera_grids()):
            rows.append((r, c, h, w, tile, out))
            tile += r * c
            out += 4 * h * w
        table = torch.tensor(rows, dtype=torch.int64).to(device)
        _CAMERA_TABLES[key] = table
        while len(_CAMERA_TABLES) > _CAMERA_TABLES_MAX:
            _CAMERA_TABLES.popitem(last=False)
    return table


def create_key_defines(*sequence: tuple[str, int]) -> tuple[tuple[str, int], ...]:
    """Bit layout of the 64-bit sort key, most significant field first."""
    offset = 0
    defines = []
    for key, length in reversed(sequence):
        if key == "depth" and length != 32:
            raise ValueError("Depth must have 32 bits.")
        upper = key.upper()
        defines.append((f"{upper}_BIT_OFFSET", offset))
        defines.append((f"{upper}_BIT_LENGTH", length))
        offset += length
    assert offset == 64
    return tuple(defines)


def _layout(key_defines) -> ctypes.Array:
    d = dict(key_defines)
    return (ctypes.c_int32 * 7)(
        d["CAMERA_BIT_OFFSET"], d["CAMERA_BIT_LENGTH"], d["SHELL_BIT_OFFSET"], d["SHELL_BIT_LENGTH"],
        d["TILE_BIT_OFFSET"], d["TILE_BIT_LENGTH"], d["DEPTH_BIT_OFFSET"],
    )


def _check_key_budget(grid: TileGrid, key_defines) -> None:
    d = dict(key_defines)
    for what, n, bits in (
        ("cameras", grid.num_cameras, d["CAMERA_BIT_LENGTH"]),
        ("shells", grid.num_shells, d["SHELL_BIT_LENGTH"]),
        ("tiles per image", grid.num_tiles_per_image, d["TILE_BIT_LENGTH"]),
    ):
        if n > (1 << bits):
            raise ValueError(f"{n} {what} do not fit in {bits} key bits")


def _f32(t: Tensor) -> Tensor:
    if t.dtype != torch.float32:
        raise TypeError(f"expected float32, got {t.dtype}")
    return t.contiguous()


def _numel(t: Tensor | None) -> int:
    return 0 if t is None else t.numel() * t.element_size()


def _i32(t: Tensor) -> Tensor:
    if t.dtype != torch.int32:
        raise TypeError(f"expected int32, got {t.dtype}")
    return t.contiguous()


def _sharpness(sharpness, device) -> Tensor:
    if not torch.is_tensor(sharpness):
        # A device fill, not a host->device copy, so it can be graph-captured.
        return torch.full((), float(sharpness), dtype=torch.float32, device=device)
    return sharpness.to(device=device, dtype=torch.float32).reshape(())


# ---------------------------------------------------------------------------
# Front end
# ---------------------------------------------------------------------------
class ProjectedVertices(NamedTuple):
    positions: Tensor  # [B, V, 2] pixels
    depths: Tensor  # [B, V]


@record_function("project_vertices")
def project_vertices(vertices: Tensor, extrinsics: Tensor, intrinsics: Tensor) -> ProjectedVertices:
    vertices, extrinsics, intrinsics = _f32(vertices), _f32(extrinsics), _f32(intrinsics)
    device = nt.require_cuda(vertices, extrinsics, intrinsics)
    b = extrinsics.shape[0]
    v = vertices.shape[0]
    xy = torch.empty((b, v, 2), dtype=torch.float32, device=device)
    depths = torch.empty((b, v), dtype=torch.float32, device=device)
    nt.call("mt_project_vertices", nt.ptr(vertices), v, nt.ptr(extrinsics), nt.ptr(intrinsics), b, nt.ptr(xy),
            nt.ptr(depths), nt.stream(device))
    return ProjectedVertices(xy, depths)


@dataclass
class TriangleBounds:
    tile_minima: Tensor  # [B, F, 2] (row, col), inclusive
    tile_maxima: Tensor  # [B, F, 2] (row, col), exclusive
    num_tiles_overlapped: Tensor  # [B, F]


@record_function("bound_triangles")
def bound_triangles(vertices: Tensor, depths: Tensor, faces: Tensor, grid: TileGrid,
                    near_plane: float, num_faces: Tensor | None = None) -> TriangleBounds:
    """``num_faces`` (optional, not in the reference signature): a device
    int32 scalar; face rows at or past it touch no tile."""
    assert near_plane >= 0
    vertices, depths, faces = _f32(vertices), _f32(depths), _i32(faces)
    device = nt.require_cuda(vertices, depths, faces)
    c, v, _ = vertices.shape
    f = faces.shape[0]
    kw = dict(dtype=torch.int32, device=device)
    tmin = torch.empty((c, f, 2), **kw)
    tmax = torch.empty((c, f, 2), **kw)
    count = torch.empty((c, f), **kw)
    rows, cols = grid.grid_shape
    nf = _i32(num_faces) if num_faces is not None else None
    table = _camera_table(grid, device)
    nt.call("mt_bound_triangles", nt.ptr(vertices), nt.ptr(depths), v, nt.ptr(faces), f, nt.ptr(nf), c,
            grid.tile_shape[0], grid.tile_shape[1], rows, cols, nt.ptr(table), float(near_plane), nt.ptr(tmin),
            nt.ptr(tmax), nt.ptr(count), nt.stream(device))
    return TriangleBounds(tmin, tmax, count)


@dataclass
class PairedKeys:
    keys: Tensor  # [K] int64
    triangle_indices: Tensor  # [K] int32
    # Capacity mode only: device int64 scalar with the live key count (the
    # buffers then have capacity rows and the rows past the count are unused).
    count: Tensor | None = None

    @property
    def num_keys(self) -> int:
        return self.keys.shape[0]


@record_function("generate_keys")
def generate_keys(depths: Tensor, faces: Tensor, shell_face_boundaries: Tensor, tile_minima: Tensor,
                  tile_maxima: Tensor, num_tiles_overlapped: Tensor, grid: TileGrid,
                  key_defines, capacity: int | None = None) -> PairedKeys:
    """``capacity`` (optional, not in the reference signature): allocate that
    many key slots and keep the live count on the device instead of reading
    it back; keys past the capacity are dropped (the caller checks the count)."""
    depths, faces, sfb = _f32(depths), _i32(faces), _i32(shell_face_boundaries)
    device = nt.require_cuda(depths, faces)
    _check_key_budget(grid, key_defines)
    counts = _i32(num_tiles_overlapped).view(-1)
    n = counts.numel()
    offsets = torch.empty((n,), dtype=torch.int64, device=device)
    if n > 0:
        ws_ptr, ws_bytes = nt.workspace(device).get(nt.library().mt_scan_workspace_bytes(n))
        nt.call("mt_inclusive_scan_i32_to_i64", counts.data_ptr(), offsets.data_ptr(), n, ws_ptr, ws_bytes,
                nt.stream(device))
    live = None
    if capacity is not None:
        num_keys = int(capacity)
        live = offsets[-1] if n > 0 else torch.zeros((), dtype=torch.int64, device=device)
    else:
        num_keys = int(offsets[-1].item()) if n > 0 else 0
    keys = torch.empty(num_keys, dtype=torch.int64, device=device)
    tri = torch.empty(num_keys, dtype=torch.int32, device=device)
    b, v = depths.shape
    tile_minima, tile_maxima = _i32(tile_minima), _i32(tile_maxima)
    nt.call("mt_generate_keys", nt.ptr(depths), v, nt.ptr(faces), faces.shape[0], nt.ptr(sfb), sfb.shape[0],
            nt.ptr(tile_minima), nt.ptr(tile_maxima), nt.ptr(offsets), b, grid.grid_shape[1],
            nt.ptr(_camera_table(grid, device)), _layout(key_defines), num_keys, nt.ptr(keys), nt.ptr(tri),
            nt.stream(device))
    return PairedKeys(keys, tri, live)


@record_function("bound_and_generate_keys")
def bound_and_generate_keys(vertices: Tensor, depths: Tensor, faces: Tensor, shell_face_boundaries: Tensor,
                            grid: TileGrid, near_plane: float, key_defines, capacity: int,
                            num_faces: Tensor | None = None) -> PairedKeys:
    """``bound_triangles`` followed by ``generate_keys(..., capacity)`` in one
    three kernels (not in the reference): the same keys in the same order,
    with no per-item offsets materialised. The live key count stays
    on the device (``PairedKeys.count``); keys past the capacity are dropped."""
    assert near_plane >= 0
    vertices, depths, faces, sfb = _f32(vertices), _f32(depths), _i32(faces), _i32(shell_face_boundaries)
    device = nt.require_cuda(vertices, depths, faces)
    _check_key_budget(grid, key_defines)
    c, v, _ = vertices.shape
    f = faces.shape[0]
    num_keys = int(capacity)
    keys = torch.empty(num_keys, dtype=torch.int64, device=device)
    tri = torch.empty(num_keys, dtype=torch.int32, device=device)
    live = torch.empty((), dtype=torch.int64, device=device)
    rows, cols = grid.grid_shape
    nf = _i32(num_faces) if num_faces is not None else None
    ws_ptr, ws_bytes = nt.workspace(device).get(nt.library().mt_bound_and_generate_keys_workspace_bytes(c * f))
    nt.call("mt_bound_and_generate_keys", nt.ptr(vertices), nt.ptr(depths), v, nt.ptr(faces), f, nt.ptr(nf),
            nt.ptr(sfb), sfb.shape[0], c, grid.tile_shape[0], grid.tile_shape[1], rows, cols,
            nt.ptr(_camera_table(grid, device)), float(near_plane), _layout(key_defines), num_keys, nt.ptr(keys),
            nt.ptr(tri), live.data_ptr(), ws_ptr, ws_bytes, nt.stream(device))
    return PairedKeys(keys, tri, live)


def _keys(positions, depths, faces, shell_face_boundaries, grid, near_plane, num_faces, key_defines,
          key_capacity) -> PairedKeys:
    """Keys of a render call: one fused kernel when the call has a key
    capacity, else the reference's bound_triangles -> generate_keys chain."""
    if key_capacity is not None:
        return bound_and_generate_keys(positions, depths, faces, shell_face_boundaries, grid, near_plane,
                                       key_defines, key_capacity, num_faces)
    bounds = bound_triangles(positions, depths, faces, grid, near_plane, num_faces)
    return generate_keys(depths, faces, shell_face_boundaries, bounds.tile_minima, bounds.tile_maxima,
                         bounds.num_tiles_overlapped, grid, key_defines)


@record_function("sort_keys")
def sort_keys(paired_keys: PairedKeys, grid: TileGrid | None = None) -> PairedKeys:
    """Stable sort by signed int64 key (the CUB SortPairs of the reference);
    stream-ordered, so no device synchronisation is needed afterwards."""
    keys = paired_keys.keys.contiguous()
    tri = _i32(paired_keys.triangle_indices)
    n = keys.numel()
    out_keys = torch.empty_like(keys)
    out_tri = torch.empty_like(tri)
    live = paired_keys.count
    if n == 0:
        return PairedKeys(out_keys, out_tri, live)
    device = nt.require_cuda(keys, tri)
    ws_ptr, ws_bytes = nt.workspace(device).get(nt.library().mt_sort_pairs_workspace_bytes(n))
    nt.call("mt_sort_pairs_i64_i32", keys.data_ptr(), tri.data_ptr(), out_keys.data_ptr(), out_tri.data_ptr(), n,
            nt.ptr(live), 0, 64, ws_ptr, ws_bytes, nt.stream(device))
    return PairedKeys(out_keys, out_tri, live)


@record_function("delineate_tiles")
def delineate_tiles(sorted_paired_keys: PairedKeys, grid: TileGrid, key_defines, separate_shells: bool,
                    epsilon: float = 1e-8) -> Tensor:
    keys = sorted_paired_keys.keys.contiguous()
    device = keys.device
    shape = [grid.num_cameras, grid.num_shells if separate_shells else 1, grid.num_tiles_per_image, 2]
    out = torch.empty(shape, dtype=torch.int64, device=device)
    if out.numel() == 0:
        return out
    nt.require_cuda(keys, out)
    nt.call("mt_delineate_tiles", nt.ptr(keys), keys.numel(), nt.ptr(sorted_paired_keys.count),
            _layout(key_defines), int(separate_shells), shape[0], shape[1], shape[2], out.data_ptr(),
            nt.stream(device))
    return out


def _sort_and_delineate(paired_keys: PairedKeys, grid: TileGrid, key_defines,
                        separate_shells: bool) -> tuple[PairedKeys, Tensor]:
    """``sort_keys`` followed by ``delineate_tiles`` (the render entry points'
    sequence) with identical outputs. Keys made by ``generate_keys`` are
    bucketed by tile and each tile is sorted on its own; layouts that do not
    allow it (a camera setting the key's sign bit, too many keys for the
    tie-breaking index) take the radix sort."""
    keys = paired_keys.keys.contiguous()
    tri = _i32(paired_keys.triangle_indices)
    n = keys.numel()
    layout = _layout(key_defines)
    b = grid.num_cameras
    sd = grid.num_shells if separate_shells else 1
    t = grid.num_tiles_per_image
    lib = nt.library()
    if n == 0 or not lib.mt_sort_keys_by_tile_supported(layout, int(separate_shells), b, n):
        paired = sort_keys(paired_keys, grid)
        bounds = delineate_tiles(paired, grid, key_defines, separate_shells)
        note(sorted_keys=paired.keys, sorted_triangles=paired.triangle_indices, tile_boundaries=bounds,
             key_count=paired.count)
        return paired, bounds
    device = nt.require_cuda(keys, tri)
    out_keys = torch.empty_like(keys)
    out_tri = torch.empty_like(tri)
    bounds = torch.empty((b, sd, t, 2), dtype=torch.int64, device=device)
    ws_ptr, ws_bytes = nt.workspace(device).get(lib.mt_sort_keys_by_tile_workspace_bytes(n, b * sd * t))
    nt.call("mt_sort_keys_by_tile", keys.data_ptr(), tri.data_ptr(), n, nt.ptr(paired_keys.count), layout,
            int(separate_shells), b, sd, t, out_keys.data_ptr(), out_tri.data_ptr(), bounds.data_ptr(), ws_ptr,
            ws_bytes, nt.stream(device))
    note(sorted_keys=out_keys, sorted_triangles=out_tri, tile_boundaries=bounds, key_count=paired_keys.count)
    return PairedKeys(out_keys, out_tri, paired_keys.count), bounds


# ---------------------------------------------------------------------------
# Spherical harmonics (evaluate_spherical_harmonics.py:23-111)
# ---------------------------------------------------------------------------
def _camera_positions(extrinsics: Tensor) -> Tensor:
    extrinsics = _f32(extrinsics)
    device = nt.require_cuda(extrinsics)
    b = extrinsics.shape[0]
    out = torch.empty((b, 3), dtype=torch.float32, device=device)
    nt.call("mt_camera_positions", nt.ptr(extrinsics), b, nt.ptr(out), nt.stream(device))
    return out


class EvaluateSphericalHarmonics(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vertices, spherical_harmonics, extrinsics, sh_degree):
        with record_function("evaluate_spherical_harmonics_forward"):
            vertices, sh = _f32(vertices), _f32(spherical_harmonics)
            device = nt.require_cuda(vertices, sh, extrinsics)
            campos = _camera_positions(extrinsics)
            b = campos.shape[0]
            v = vertices.shape[0]
            c = sh.shape[0]
            colors = torch.empty((b, v, 3), dtype=torch.float32, device=device)
            nt.call("mt_evaluate_spherical_harmonics", nt.ptr(vertices), v, nt.ptr(sh), c, int(sh_degree),
                    nt.ptr(campos), b, nt.ptr(colors), nt.stream(device))
            ctx.save_for_backward(vertices, campos, colors)
            ctx.sh_shape = sh.shape
            ctx.sh_degree = int(sh_degree)
            return colors

    @staticmethod
    def backward(ctx, grad_colors):
        with record_function("evaluate_spherical_harmonics_backward"):
            vertices, campos, colors = ctx.saved_tensors
            grad_colors = grad_colors.contiguous()
            device = vertices.device
            grad_sh = torch.empty(ctx.sh_shape, dtype=torch.float32, device=device)  # fully written
            nt.call("mt_evaluate_spherical_harmonics_backward", nt.ptr(vertices), vertices.shape[0],
                    ctx.sh_shape[0], ctx.sh_degree, nt.ptr(campos), campos.shape[0], nt.ptr(colors),
                    nt.ptr(grad_colors), nt.ptr(grad_sh), nt.stream(device))
            return None, grad_sh, None, None


def evaluate_spherical_harmonics(vertices: Tensor, spherical_harmonics: Tensor, extrinsics: Tensor,
                                 sh_degree: int) -> Tensor:
    """``spherical_harmonics``: the [C, V, 3] rows, or (not in the reference)
    a deferred-SH object of the tessellation (``triangle_extraction.DeferredSH``)
    whose ``evaluate`` gives the same colours from the grid coefficients."""
    if not isinstance(spherical_harmonics, Tensor) and hasattr(spherical_harmonics, "evaluate"):
        return spherical_harmonics.evaluate(vertices, extrinsics, sh_degree)
    return EvaluateSphericalHarmonics.apply(vertices, spherical_harmonics, extrinsics, sh_degree)


# ---------------------------------------------------------------------------
# Fused compositing (intersect_and_composite.py:24-175)
# ---------------------------------------------------------------------------
# Byte budget of the compositing hit-bit store, per pixel of the render (not
# in the reference). The forward stores, per warp and batch of 32 triangles,
# the bits of the triangles each pixel hits, so that the backward need not
# test them again; batches beyond the budget are tested again by the
# backward (same gradients). 16 B per pixel is a sixth of the explicit
# mode's 12 * num_shells B per pixel at 8 shells; 0 turns the store off.
HIT_BITS_BYTES_PER_PIXEL = 16

# Compositing backward with its triangles' vertex records staged into shared
# memory by bulk copies (cp.async.bulk on an mbarrier), the next batch's while
# the current one composites (not in the reference; same gradients).
STAGED_BACKWARD = False


def _staging(b: int, v: int, device) -> Tensor | None:
    if not STAGED_BACKWARD:
        return None
    nbytes = int(nt.library().mt_composite_staging_bytes(b, v))
    return torch.zeros((nbytes,), dtype=torch.uint8, device=device) if nbytes else None


# Longest-first tile order of the compositing kernels (not in the reference):
# the tiles with the most keys are composited first, so the few expensive
# ones do not start last and hold up the launch (same results).
TILE_ORDER = True


def _tile_order(grid: TileGrid, device) -> Tensor | None:
    if not TILE_ORDER:
        return None
    nbytes = int(nt.library().mt_composite_tile_order_bytes(grid.camera_tiles))
    return torch.empty((nbytes // 4,), dtype=torch.int32, device=device)


def _hit_bits(ctx, grid: TileGrid, num_keys: int, device) -> Tensor | None:
    """The hit-bit store for the forward and its backward (only when a
    gradient will be asked for): the batches num_keys keys can form at most,
    capped by HIT_BITS_BYTES_PER_PIXEL."""
    if not any(ctx.needs_input_grad) or HIT_BITS_BYTES_PER_PIXEL <= 0:
        return None
    th, tw = grid.tile_shape
    warps = (th * tw + 31) // 32
    items = grid.camera_tiles * warps
    most = int(num_keys) * warps // 32 + items
    budget = HIT_BITS_BYTES_PER_PIXEL * grid.camera_tiles * th * tw // 128
    batches = min(most, budget)
    if batches <= 0:
        return None
    nbytes = int(nt.library().mt_composite_hit_bits_bytes(grid.camera_tiles, th, tw, batches))
    return torch.empty((nbytes,), dtype=torch.uint8, device=device)


class IntersectAndComposite(torch.autograd.Function):
    @staticmethod
    def forward(ctx, vertices, colors, signed_distances, faces, sharpness, sorted_keys, sorted_triangle_indices,
                tile_boundaries, num_shells, grid, key_defines, gradient_mode=None, num_keys=None):
        with record_function("intersect_and_composite_forward"):
            xy, colors, sdf, faces = _f32(vertices), _f32(colors), _f32(signed_distances), _i32(faces)
            device = nt.require_cuda(xy, colors, sdf, faces)
            sharp = _sharpness(sharpness, device)
            keys, tri = sorted_keys.contiguous(), _i32(sorted_triangle_indices)
            bounds = tile_boundaries.contiguous()
            b, v, _ = xy.shape
            k = keys.numel()
            h, w = grid.image_shape
            rows, cols = grid.grid_shape
            masks = torch.empty((k,), dtype=torch.int32, device=device)
            counter = torch.empty((1,), dtype=torch.int64, device=device)
            table = _camera_table(grid, device)
            # Uniform cameras: [B, 4, H, W]; ragged: every camera's [4, h, w] back to back.
            out = torch.empty((grid.output_numel,) if grid.ragged else (b, 4, h, w), dtype=torch.float32,
                              device=device)
            hits = _hit_bits(ctx, grid, k, device)
            order = _tile_order(grid, device)
            nt.call("mt_intersect_and_composite_forward", nt.ptr(xy), nt.ptr(colors), nt.ptr(sdf), v,
                    nt.ptr(faces), nt.ptr(sharp), nt.ptr(keys), nt.ptr(tri), k, nt.ptr(num_keys), nt.ptr(bounds), b,
                    int(num_shells), rows, cols, grid.tile_shape[0], grid.tile_shape[1], h, w, _layout(key_defines),
                    nt.ptr(table), grid.camera_tiles, nt.ptr(masks), nt.ptr(counter), nt.ptr(out), None, None,
                    0.0, None, nt.ptr(hits), _numel(hits), nt.ptr(order), _numel(order), grid.cta_threads,
                    nt.stream(device))
            note(composite=out)
            ctx.hits = hits
            ctx.order = order
            ctx.save_for_backward(xy, colors, sdf, faces, sharp, keys, tri, bounds, masks, out)
            ctx.meta = (int(num_shells), grid, key_defines, gradient_mode or _GRADIENT_MODE,
                        torch.is_tensor(sharpness))
            return out

    @staticmethod
    def backward(ctx, grad_out):
        with record_function("intersect_and_composite_backward"):
            xy, colors, sdf, faces, sharp, keys, tri, bounds, masks, out = ctx.saved_tensors
            num_shells, grid, key_defines, mode, sharp_is_tensor = ctx.meta
            device = xy.device
            grad_out = grad_out.contiguous()
            grad_colors = torch.zeros_like(colors)
            grad_sdf = torch.zeros_like(sdf)
            grad_sharp = torch.zeros_like(sharp)
            b, v, _ = xy.shape
            h, w = grid.image_shape
            rows, cols = grid.grid_shape
            counter = torch.empty((1,), dtype=torch.int64, device=device)
            staging = _staging(b, v, device)
            nt.call("mt_intersect_and_composite_backward", nt.ptr(xy), nt.ptr(colors), nt.ptr(sdf), v,
                    nt.ptr(faces), nt.ptr(sharp), nt.ptr(keys), nt.ptr(tri), keys.numel(), nt.ptr(bounds), b,
                    num_shells, rows, cols, grid.tile_shape[0], grid.tile_shape[1], h, w, _layout(key_defines),
                    nt.ptr(_camera_table(grid, device)), grid.camera_tiles, nt.ptr(masks), nt.ptr(counter),
                    nt.ptr(out), nt.ptr(grad_out), None, None, 0.0, None, 1, nt.ptr(grad_colors), nt.ptr(grad_sdf),
                    nt.ptr(grad_sharp), int(mode == "exact"), nt.ptr(ctx.hits), _numel(ctx.hits),
                    nt.ptr(staging), _numel(staging), nt.ptr(ctx.order), _numel(ctx.order), grid.cta_threads,
                    nt.stream(device))
            return (None, grad_colors, grad_sdf, None, grad_sharp if sharp_is_tensor else None, None, None, None,
                    None, None, None, None, None)


class IntersectCompositeLoss(torch.autograd.Function):
    """Fused compositing with the MSE epilogue (not in the reference): returns
    mean((clip(rgb + T * background, 0, 1) - target)^2) over every pixel and
    channel; the backward forms d loss / d (rgb, T) inside the compositing
    adjoint. Without SSAA the epilogue runs inside the compositing kernel and
    the image is never materialised; with ``ssaa`` > 1 the compositing output
    is at the supersampled size and one kernel averages each ssaa x ssaa block
    (after the background blend, before the clip, as the render entry points
    do) and takes the loss, keeping a per-pixel factor for the backward."""

    @staticmethod
    def forward(ctx, vertices, colors, signed_distances, faces, sharpness, sorted_keys, sorted_triangle_indices,
                tile_boundaries, num_shells, grid, key_defines, target, background, gradient_mode=None,
                num_keys=None, ssaa=1):
        with record_function("intersect_composite_loss_forward"):
            xy, colors, sdf, faces = _f32(vertices), _f32(colors), _f32(signed_distances), _i32(faces)
            target, background = _f32(target), _f32(background)
            device = nt.require_cuda(xy, colors, sdf, faces, target, background)
            sharp = _sharpness(sharpness, device)
            keys, tri = sorted_keys.contiguous(), _i32(sorted_triangle_indices)
            bounds = tile_boundaries.contiguous()
            b, v, _ = xy.shape
            k = keys.numel()
            h, w = grid.image_shape
            rows, cols = grid.grid_shape
            ssaa = int(ssaa)
            if ssaa > 1 and (grid.ragged or h % ssaa or w % ssaa):
                raise ValueError("SSAA needs cameras of one image size, a multiple of ssaa")
            if target.numel() * 4 * ssaa * ssaa != grid.output_numel * 3:
                raise ValueError("target must hold 3 channels of every camera's image")
            masks = torch.empty((k,), dtype=torch.int32, device=device)
            counter = torch.empty((1,), dtype=torch.int64, device=device)
            table = _camera_table(grid, device)
            out = torch.empty((grid.output_numel,) if grid.ragged else (b, 4, h, w), dtype=torch.float32,
                              device=device)
            loss = torch.empty((), dtype=torch.float32, device=device)
            scale = 1.0 / target.numel()
            hits = _hit_bits(ctx, grid, k, device)
            order = _tile_order(grid, device)
            in_kernel = ssaa == 1
            nt.call("mt_intersect_and_composite_forward", nt.ptr(xy), nt.ptr(colors), nt.ptr(sdf), v,
                    nt.ptr(faces), nt.ptr(sharp), nt.ptr(keys), nt.ptr(tri), k, nt.ptr(num_keys), nt.ptr(bounds), b,
                    int(num_shells), rows, cols, grid.tile_shape[0], grid.tile_shape[1], h, w, _layout(key_defines),
                    nt.ptr(table), grid.camera_tiles, nt.ptr(masks), nt.ptr(counter), nt.ptr(out),
                    nt.ptr(target) if in_kernel else None, nt.ptr(background) if in_kernel else None, scale,
                    loss.data_ptr() if in_kernel else None, nt.ptr(hits), _numel(hits), nt.ptr(order),
                    _numel(order), grid.cta_threads, nt.stream(device))
            factor = target
            if not in_kernel:
                factor = torch.empty_like(target)
                nt.call("mt_ssaa_loss", out.data_ptr(), b, h, w, ssaa, nt.ptr(background), nt.ptr(target), scale,
                        loss.data_ptr(), factor.data_ptr(), nt.stream(device))
            note(composite=out, loss=loss)
            ctx.hits = hits
            ctx.order = order
            ctx.save_for_backward(xy, colors, sdf, faces, sharp, keys, tri, bounds, masks, out, factor, background)
            ctx.meta = (int(num_shells), grid, key_defines, gradient_mode or _GRADIENT_MODE,
                        torch.is_tensor(sharpness), scale, ssaa)
            return loss

    @staticmethod
    def backward(ctx, grad_loss):
        with record_function("intersect_composite_loss_backward"):
            xy, colors, sdf, faces, sharp, keys, tri, bounds, masks, out, target, background = ctx.saved_tensors
            num_shells, grid, key_defines, mode, sharp_is_tensor, scale, ssaa = ctx.meta
            device = xy.device
            grad_loss = grad_loss.to(torch.float32).contiguous()
            grad_colors = torch.zeros_like(colors)
            grad_sdf = torch.zeros_like(sdf)
            grad_sharp = torch.zeros_like(sharp)
            b, v, _ = xy.shape
            h, w = grid.image_shape
            rows, cols = grid.grid_shape
            counter = torch.empty((1,), dtype=torch.int64, device=device)
            staging = _staging(b, v, device)
            nt.call("mt_intersect_and_composite_backward", nt.ptr(xy), nt.ptr(colors), nt.ptr(sdf), v,
                    nt.ptr(faces), nt.ptr(sharp), nt.ptr(keys), nt.ptr(tri), keys.numel(), nt.ptr(bounds), b,
                    num_shells, rows, cols, grid.tile_shape[0], grid.tile_shape[1], h, w, _layout(key_defines),
                    nt.ptr(_camera_table(grid, device)), grid.camera_tiles, nt.ptr(masks), nt.ptr(counter),
                    nt.ptr(out), None, nt.ptr(target), nt.ptr(background), scale, grad_loss.data_ptr(), ssaa,
                    nt.ptr(grad_colors), nt.ptr(grad_sdf), nt.ptr(grad_sharp), int(mode == "exact"),
                    nt.ptr(ctx.hits), _numel(ctx.hits), nt.ptr(staging), _numel(staging), nt.ptr(ctx.order),
                    _numel(ctx.order), grid.cta_threads, nt.stream(device))
            return (None, grad_colors, grad_sdf, None, grad_sharp if sharp_is_tensor else None, None, None, None,
                    None, None, None, None, None, None, None, None)


def intersect_and_composite(vertices, colors, signed_distances, faces, sharpness, sorted_keys,
                            sorted_triangle_indices, tile_boundaries, num_shells, grid, key_defines,
                            gradient_mode: str | None = None, num_keys: Tensor | None = None) -> Tensor:
    """``num_keys`` (optional): device int64 count of live keys when the key
    buffers are capacity-sized."""
    return IntersectAndComposite.apply(vertices, colors, signed_distances, faces, sharpness, sorted_keys,
                                       sorted_triangle_indices, tile_boundaries, num_shells, grid, key_defines,
                                       gradient_mode, num_keys)


# ---------------------------------------------------------------------------
# Explicit mode (intersect.py, interpolate.py, composite.py)
# ---------------------------------------------------------------------------
class RenderedImages(NamedTuple):
    uv: Tensor  # [B, S, H, W, 2]
    index: Tensor  # [B, S, H, W] (-1 = miss)


@record_function("intersect")
def intersect(vertices: Tensor, faces: Tensor, sorted_triangle_indices: Tensor, tile_boundaries: Tensor,
              grid: TileGrid, key_defines) -> RenderedImages:
    xy, faces, tri = _f32(vertices), _i32(faces), _i32(sorted_triangle_indices)
    device = nt.require_cuda(xy, faces)
    h, w = grid.image_shape
    out_shape = (grid.num_cameras * grid.num_shells, h, w)
    uv = torch.empty((*out_shape, 2), dtype=torch.float32, device=device)
    index = torch.empty(out_shape, dtype=torch.int32, device=device)
    rows, cols = grid.grid_shape
    tile_boundaries = tile_boundaries.contiguous()
    nt.call("mt_intersect", nt.ptr(xy), xy.shape[1], nt.ptr(faces), nt.ptr(tri), nt.ptr(tile_boundaries),
            grid.num_cameras, grid.num_shells, rows, cols, grid.tile_shape[0], grid.tile_shape[1], h, w,
            nt.ptr(uv), nt.ptr(index), nt.stream(device))
    shape = (grid.num_cameras, grid.num_shells, h, w)
    return RenderedImages(uv.view(*shape, 2), index.view(shape))


class Interpolate(torch.autograd.Function):
    @staticmethod
    def forward(ctx, uv, index, faces, signed_distances, colors):
        with record_function("interpolate_forward"):
            uv, index, faces = _f32(uv), _i32(index), _i32(faces)
            sdf, colors = _f32(signed_distances), _f32(colors)
            device = nt.require_cuda(uv, index, faces, sdf, colors)
            b, s, h, w, _ = uv.shape
            out_sdf = torch.empty((b, s, h, w), dtype=torch.float32, device=device)
            out_colors = torch.empty((b, s, h, w, 3), dtype=torch.float32, device=device)
            nt.call("mt_interpolate", nt.ptr(uv), nt.ptr(index), b, s, h, w, nt.ptr(faces), nt.ptr(sdf),
                    nt.ptr(colors), sdf.shape[0], nt.ptr(out_sdf), nt.ptr(out_colors), nt.stream(device))
            ctx.save_for_backward(uv, index, faces)
            ctx.shapes = (sdf.shape, colors.shape)
            ctx.set_materialize_grads(False)
            return out_sdf, out_colors

    @staticmethod
    def backward(ctx, grad_sdf, grad_colors):
        with record_function("interpolate_backward"):
            uv, index, faces = ctx.saved_tensors
            sdf_shape, colors_shape = ctx.shapes
            device = uv.device
            b, s, h, w, _ = uv.shape
            gsdf = torch.zeros(sdf_shape, dtype=torch.float32, device=device)
            gcol = torch.zeros(colors_shape, dtype=torch.float32, device=device)
            gs = grad_sdf.contiguous() if grad_sdf is not None else None
            gc = grad_colors.contiguous() if grad_colors is not None else None
            nt.call("mt_interpolate_backward", nt.ptr(uv), nt.ptr(index), b, s, h, w, nt.ptr(faces), sdf_shape[0],
                    nt.ptr(gs), nt.ptr(gc), nt.ptr(gsdf), nt.ptr(gcol), nt.stream(device))
            return None, None, None, gsdf, gcol


def interpolate(uv, index, faces, signed_distances, colors):
    return Interpolate.apply(uv, index, faces, signed_distances, colors)


class Composite(torch.autograd.Function):
    @staticmethod
    def forward(ctx, signed_distances, colors, mask, sharpness, gradient_mode=None):
        with record_function("composite_forward"):
            sdf, colors = _f32(signed_distances), _f32(colors)
            device = nt.require_cuda(sdf, colors, mask)
            mask_u8 = mask.contiguous().view(torch.uint8) if mask.dtype == torch.bool else mask.to(torch.uint8)
            sharp = _sharpness(sharpness, device)
            p, s = sdf.shape
            out_colors = torch.empty((p, 3), dtype=torch.float32, device=device)
            out_t = torch.empty((p,), dtype=torch.float32, device=device)
            nt.call("mt_composite", nt.ptr(sdf), nt.ptr(colors), nt.ptr(mask_u8), p, s, nt.ptr(sharp),
                    nt.ptr(out_colors), nt.ptr(out_t), nt.stream(device))
            ctx.save_for_backward(sdf, colors, mask_u8, sharp, out_colors, out_t)
            ctx.meta = (gradient_mode or _GRADIENT_MODE, torch.is_tensor(sharpness))
            ctx.set_materialize_grads(False)
            return out_colors, out_t

    @staticmethod
    def backward(ctx, grad_colors, grad_t):
        with record_function("composite_backward"):
            sdf, colors, mask, sharp, out_colors, out_t = ctx.saved_tensors
            mode, sharp_is_tensor = ctx.meta
            device = sdf.device
            p, s = sdf.shape
            gsdf = torch.zeros_like(sdf)
            gcol = torch.zeros_like(colors)
            gsharp = torch.zeros_like(sharp)
            gc = grad_colors.contiguous() if grad_colors is not None else None
            gt = grad_t.contiguous() if grad_t is not None else None
            nt.call("mt_composite_backward", nt.ptr(sdf), nt.ptr(colors), nt.ptr(mask), p, s, nt.ptr(sharp),
                    nt.ptr(out_colors), nt.ptr(out_t), nt.ptr(gc), nt.ptr(gt), nt.ptr(gsdf), nt.ptr(gcol),
                    nt.ptr(gsharp), int(mode == "exact"), nt.stream(device))
            return gsdf, gcol, None, (gsharp if sharp_is_tensor else None), None


def composite(signed_distances, colors, mask, background, sharpness, gradient_mode: str | None = None) -> Tensor:
    out_colors, out_t = Composite.apply(signed_distances, colors, mask, sharpness, gradient_mode)
    return out_colors + background * out_t[:, None]


# ---------------------------------------------------------------------------
# Render entry points (triangle_rasterization/__init__.py:22-329)
# ---------------------------------------------------------------------------
@record_function("rasterize")
def rasterize(vertices, faces, shell_face_boundaries, extrinsics, intrinsics, image_shape, tile_shape=(16, 16),
              near_plane=0.2, num_camera_bits=6, num_shell_bits=6, num_tile_bits=20) -> RenderedImages:
    h, w = image_shape
    device = vertices.device
    c = extrinsics.shape[0]
    (s,) = shell_face_boundaries.shape
    if vertices.numel() == 0 or faces.numel() == 0:
        # The reference's branch here has a dtype typo (torch.fsoat32,
        # __init__.py:48); the intended empty result is returned.
        uv = torch.zeros((c, s, h, w, 2), device=device, dtype=torch.float32)
        index = torch.full((c, s, h, w), -1, device=device, dtype=torch.int32)
        return RenderedImages(uv, index)
    grid = TileGrid(tuple(tile_shape), tuple(image_shape), c, s)
    key_defines = create_key_defines(("camera", num_camera_bits), ("shell", num_shell_bits),
                                     ("tile", num_tile_bits), ("depth", 32))
    positions, depths = project_vertices(vertices, extrinsics, intrinsics)
    bounds = bound_triangles(positions, depths, faces, grid, near_plane)
    paired = generate_keys(depths, faces, shell_face_boundaries, bounds.tile_minima, bounds.tile_maxima,
                           bounds.num_tiles_overlapped, grid, key_defines)
    del bounds, depths
    paired, tile_boundaries = _sort_and_delineate(paired, grid, key_defines, True)
    return intersect(positions, faces, paired.triangle_indices, tile_boundaries, grid, key_defines)


def _ssaa(intrinsics: Tensor, image_shape, ssaa: int):
    h, w = image_shape
    multiplier = torch.tensor((ssaa, ssaa, 1), device=intrinsics.device)
    return (h * ssaa, w * ssaa), intrinsics * multiplier[:, None]


def _mean_pool(images: Tensor, ssaa: int) -> Tensor:
    b, c, h, w = images.shape
    return images.reshape(b, c, h // ssaa, ssaa, w // ssaa, ssaa).mean(dim=(3, 5))


@record_function("render_explicit")
def render_explicit(extrinsics, intrinsics, image_shape, vertices, faces, shell_face_boundaries, signed_distances,
                    spherical_harmonics, sh_degree, sharpness, background, tile_shape=(16, 16), near_plane=0.2,
                    num_camera_bits=6, num_shell_bits=6, num_tile_bits=20, ssaa=1, gradient_mode=None) -> Tensor:
    if ssaa > 1:
        image_shape, intrinsics = _ssaa(intrinsics, image_shape, ssaa)
    uv, index = rasterize(vertices, faces, shell_face_boundaries, extrinsics, intrinsics, image_shape,
                          tile_shape=tile_shape, near_plane=near_plane, num_camera_bits=num_camera_bits,
                          num_shell_bits=num_shell_bits, num_tile_bits=num_tile_bits)
    colors = evaluate_spherical_harmonics(vertices, spherical_harmonics, extrinsics, sh_degree)
    sdf, colors = interpolate(uv, index, faces, signed_distances, colors)
    mask = index != -1
    b, s, h, w = sdf.shape
    sdf = sdf.permute(0, 2, 3, 1).reshape(b * h * w, s).contiguous()
    colors = colors.permute(0, 2, 3, 1, 4).reshape(b * h * w, s, 3).contiguous()
    mask = mask.permute(0, 2, 3, 1).reshape(b * h * w, s).contiguous()
    image = composite(sdf, colors, mask, background, sharpness, gradient_mode)
    image = image.reshape(b, h, w, 3).permute(0, 3, 1, 2)
    if ssaa > 1:
        image = _mean_pool(image, ssaa)
    return image


@record_function("render_fused")
def render_fused(extrinsics, intrinsics, image_shape, vertices, faces, shell_face_boundaries, signed_distances,
                 spherical_harmonics, sh_degree, sharpness, background, tile_shape=(16, 16), near_plane=0.2, ssaa=1,
                 num_camera_bits=6, num_shell_bits=6, num_tile_bits=20, gradient_mode=None,
                 num_faces: Tensor | None = None, key_capacity: int | None = None) -> Tensor:
    """Fused render (triangle_rasterization/__init__.py:167-287).

    Capacity mode (not in the reference): with ``num_faces`` (device int32
    count of live face rows) and ``key_capacity`` the call reads nothing back
    from the device, so it can be captured in a CUDA graph; keys past the
    capacity are dropped and ``LAST_RENDER_STATS["key_count"]`` holds the live
    key count as a device scalar for the caller to check."""
    b = extrinsics.shape[0]
    h, w = image_shape
    if vertices.numel() == 0 or faces.numel() == 0:
        return background.reshape(1, 3, 1, 1).expand(b, 3, h, w)
    if ssaa > 1:
        image_shape, intrinsics = _ssaa(intrinsics, image_shape, ssaa)
    (s,) = shell_face_boundaries.shape
    grid = TileGrid(tuple(tile_shape), tuple(image_shape), b, s)
    key_defines = create_key_defines(("camera", num_camera_bits), ("tile", num_tile_bits), ("depth", 32),
                                     ("shell", num_shell_bits))
    positions, depths = project_vertices(vertices, extrinsics, intrinsics)
    paired = _keys(positions, depths, faces, shell_face_boundaries, grid, near_plane, num_faces, key_defines,
                   key_capacity)
    del depths
    LAST_RENDER_STATS.update(num_keys=paired.num_keys, num_tiles=grid.num_tiles_per_image, key_count=paired.count)
    paired, tile_boundaries = _sort_and_delineate(paired, grid, key_defines, False)
    colors = evaluate_spherical_harmonics(vertices, spherical_harmonics, extrinsics, sh_degree)
    t = tile_boundaries.shape[2]
    images = intersect_and_composite(positions, colors, signed_distances, faces, sharpness, paired.keys,
                                     paired.triangle_indices, tile_boundaries.view(b, t, 2), s, grid, key_defines,
                                     gradient_mode, paired.count)
    images = images[:, :3] + images[:, 3:4] * background[:, None, None]
    if ssaa > 1:
        images = _mean_pool(images, ssaa)
    return images.clip(min=0, max=1)


def split_cameras(raw: Tensor, grid: TileGrid) -> list[Tensor]:
    """Per-camera [4, h, w] views of a ragged compositing output."""
    views, start = [], 0
    for h, w in grid.camera_shapes:
        views.append(raw[start:start + 4 * h * w].view(4, h, w))
        start += 4 * h * w
    return views


@record_function("render_cameras")
def render_cameras(extrinsics, intrinsics, image_shapes, vertices, faces, shell_face_boundaries, signed_distances,
                   spherical_harmonics, sh_degree, sharpness, background, tile_shape=(16, 16), near_plane=0.2,
                   num_camera_bits=6, num_shell_bits=6, num_tile_bits=20, gradient_mode=None,
                   num_faces: Tensor | None = None, key_capacity: int | None = None) -> list[Tensor]:
    """Fused render of cameras with different image sizes in one pass (not in
    the reference, which renders one image size per call).

    ``image_shapes``: one (height, width) per camera. Every stage runs once
    for all cameras; the compositing kernel's persistent warps take (camera,
    tile) work items of every camera from one queue. Returns one [3, h, w]
    image per camera, equal to rendering each camera on its own with
    ``render_fused``. ``num_faces`` / ``key_capacity`` as in ``render_fused``.
    """
    b = extrinsics.shape[0]
    (s,) = shell_face_boundaries.shape
    grid = TileGrid.for_cameras(tile_shape, image_shapes, s)
    if len(grid.camera_shapes) != b:
        raise ValueError("one image shape per camera is required")
    if vertices.numel() == 0 or faces.numel() == 0:
        return [background.reshape(3, 1, 1).expand(3, h, w) for h, w in grid.camera_shapes]
    key_defines = create_key_defines(("camera", num_camera_bits), ("tile", num_tile_bits), ("depth", 32),
                                     ("shell", num_shell_bits))
    positions, depths = project_vertices(vertices, extrinsics, intrinsics)
    paired = _keys(positions, depths, faces, shell_face_boundaries, grid, near_plane, num_faces, key_defines,
                   key_capacity)
    del depths
    LAST_RENDER_STATS.update(num_keys=paired.num_keys, num_tiles=grid.camera_tiles, key_count=paired.count)
    paired, tile_boundaries = _sort_and_delineate(paired, grid, key_defines, False)
    colors = evaluate_spherical_harmonics(vertices, spherical_harmonics, extrinsics, sh_degree)
    t = tile_boundaries.shape[2]
    raw = intersect_and_composite(positions, colors, signed_distances, faces, sharpness, paired.keys,
                                  paired.triangle_indices, tile_boundaries.view(b, t, 2), s, grid, key_defines,
                                  gradient_mode, paired.count)
    bg = background[:, None, None]
    return [(r[:3] + r[3:4] * bg).clip(min=0, max=1) for r in split_cameras(raw, grid)]


@record_function("render_fused_loss")
def render_fused_loss(extrinsics, intrinsics, image_shape, vertices, faces, shell_face_boundaries, signed_distances,
                      spherical_harmonics, sh_degree, sharpness, background, target, tile_shape=(16, 16),
                      near_plane=0.2, num_camera_bits=6, num_shell_bits=6, num_tile_bits=20, gradient_mode=None,
                      num_faces: Tensor | None = None, key_capacity: int | None = None,
                      camera_shapes=None, ssaa: int = 1) -> Tensor:
    """mean((render_fused(...) - target)^2) with the background blend, clip and
    MSE inside the compositing kernels (not in the reference, where the
    trainer applies them as separate tensor ops). Same loss and gradients as
    the unfused composition. target: [B, 3, H, W]; with ``camera_shapes``
    (one (h, w) per camera, as ``render_cameras``) every camera's [3, h, w]
    back to back. ``ssaa`` > 1 (cameras of one size): rendered at ssaa times
    the size and averaged per pixel after the background blend and before the
    clip, as ``render_fused`` does."""
    b = extrinsics.shape[0]
    (s,) = shell_face_boundaries.shape
    if ssaa > 1:
        if camera_shapes is not None:
            raise ValueError("SSAA needs cameras of one image size")
        if vertices.numel() == 0 or faces.numel() == 0:
            image = background.reshape(1, 3, 1, 1).expand(b, 3, *image_shape)
            return ((image - target) ** 2).mean()
        image_shape, intrinsics = _ssaa(intrinsics, image_shape, ssaa)
    grid = (TileGrid.for_cameras(tile_shape, camera_shapes, s) if camera_shapes is not None
            else TileGrid(tuple(tile_shape), tuple(image_shape), b, s))
    if vertices.numel() == 0 or faces.numel() == 0:
        if camera_shapes is None:
            image = background.reshape(1, 3, 1, 1).expand(b, 3, *image_shape)
            return ((image - target) ** 2).mean()
        images = torch.cat([background.reshape(3, 1).expand(3, h * w).reshape(-1) for h, w in grid.camera_shapes])
        return ((images - target) ** 2).mean()
    key_defines = create_key_defines(("camera", num_camera_bits), ("tile", num_tile_bits), ("depth", 32),
                                     ("shell", num_shell_bits))
    positions, depths = project_vertices(vertices, extrinsics, intrinsics)
    paired = _keys(positions, depths, faces, shell_face_boundaries, grid, near_plane, num_faces, key_defines,
                   key_capacity)
    del depths
    LAST_RENDER_STATS.update(num_keys=paired.num_keys, num_tiles=grid.camera_tiles, key_count=paired.count)
    paired, tile_boundaries = _sort_and_delineate(paired, grid, key_defines, False)
    colors = evaluate_spherical_harmonics(vertices, spherical_harmonics, extrinsics, sh_degree)
    t = tile_boundaries.shape[2]
    return IntersectCompositeLoss.apply(positions, colors, signed_distances, faces, sharpness, paired.keys,
                                        paired.triangle_indices, tile_boundaries.view(b, t, 2), s, grid, key_defines,
                                        target, background, gradient_mode, paired.count, ssaa)


def render(extrinsics, intrinsics, image_shape, vertices, faces, shell_face_boundaries, signed_distances,
           spherical_harmonics, sh_degree, sharpness, background, tile_shape=(16, 16), near_plane=0.2,
           num_camera_bits=6, num_shell_bits=6, num_tile_bits=20, ssaa=1,
           mode: Literal["explicit", "fused"] = "fused", gradient_mode: str | None = None) -> Tensor:
    _render = render_fused if mode == "fused" else render_explicit
    return _render(extrinsics, intrinsics, image_shape, vertices, faces, shell_face_boundaries, signed_distances,
                   spherical_harmonics, sh_degree, sharpness, background, tile_shape=tile_shape,
                   near_plane=near_plane, num_camera_bits=num_camera_bits, num_shell_bits=num_shell_bits,
                   num_tile_bits=num_tile_bits, ssaa=ssaa, gradient_mode=gradient_mode)
