"""numpy front end of the CPU oracle (``liboracle.so``). Test infrastructure only.

Each function mirrors the reference function of the same name (shapes and
dtypes as in dcharatan/meshtryoshka) and runs the C++ restatement in
``mt_oracle.cpp``. Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline leg of ``bench.py`` use this module.
"""

from __future__ import annotations

import ctypes
from ctypes import c_float, c_int32, c_int64, c_uint64, c_void_p
from typing import NamedTuple

import numpy as np

from . import build_oracle

_lib = None

P = c_void_p
I32 = c_int32
I64 = c_int64
F32 = c_float

_SIGNATURES = {
    "or_mc_first_checksum": (c_uint64, []),
    "or_mc_ids_checksum": (c_uint64, []),
    "or_exclusive_scan_i32": (None, [P, I64]),
    "or_exclusive_scan_i64": (None, [P, I64]),
    "or_inclusive_scan_i32_to_i64": (None, [P, P, I64]),
    "or_compute_vertex_occupancy": (None, [P, I32, I32, I32, P, P]),
    "or_count_occupancy": (None, [P, I32, I32, I32, P]),
    "or_create_voxels": (None, [P, P, P, P, I32, I32, I32, I64, I64, P, P, P, P, P]),
    "or_dilate_occupancy": (None, [P, I32, I32, I32, I32, P]),
    "or_write_occupancy": (None, [P, I64, P, I64]),
    "or_upscale_occupancy": (None, [P, P, I32, I32, I32, I32, I32, I32, P]),
    "or_upscale_parameters": (None, [P, P, P, P, I32, I64, I32, I32, I32, P, P, I32, I32, I32, I64, P, P]),
    "or_count_occupancy_mesh_triangles": (None, [P, I32, I32, I32, P]),
    "or_create_occupancy_mesh_triangles": (None, [P, I32, I32, I32, P, P, P, P]),
    "or_count_triangle_vertices": (None, [P, P, I64, P, I32, P]),
    "or_create_triangle_vertices": (None, [P, P, P, I32, P, I64, P, I32, P, I64, P, P, P, P]),
    "or_create_triangle_vertices_backward": (None, [P, I32, P, I64, P, I32, P, P, P, P, I64, P, P, P]),
    "or_triangle_vertex_sources": (None, [P, P, I64, P, I32, P, P, P, P]),
    "or_compute_sdf_regularizers": (None, [P, P, P, I64, P, I64, I32, I32, I32, P, P, P]),
    "or_compute_sdf_regularizers_backward": (None, [P, P, P, I64, P, I64, I32, I32, I32, P, P, P, P]),
    "or_count_triangle_faces": (None, [P, P, I64, P, I64, P, I32, P, P]),
    "or_create_triangle_faces": (None, [P, P, I64, I64, P, P, P, I32, P, P, P]),
}


def lib():
    global _lib
    if _lib is None:
        path = build_oracle.build()
        _lib = ctypes.CDLL(str(path))
        for name, (restype, argtypes) in _SIGNATURES.items():
            fn = getattr(_lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
    return _lib


def _p(a: np.ndarray | None):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "oracle arrays must be C-contiguous"
    return a.ctypes.data if a.size > 0 else None


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def mc_checksums() -> tuple[int, int]:
    return int(lib().or_mc_first_checksum()), int(lib().or_mc_ids_checksum())


def exclusive_cumsum(x: np.ndarray) -> np.ndarray:
    x = np.array(x, copy=True)
    if x.dtype == np.int32:
        lib().or_exclusive_scan_i32(_p(x), x.size)
    elif x.dtype == np.int64:
        lib().or_exclusive_scan_i64(_p(x), x.size)
    else:
        raise TypeError(x.dtype)
    return x


def inclusive_cumsum_i64(x: np.ndarray) -> np.ndarray:
    x = _c(x, np.int32)
    out = np.empty(x.shape, np.int64)
    lib().or_inclusive_scan_i32_to_i64(_p(x), _p(out), x.size)
    return out


# ---------------------------------------------------------------------------
# Voxel extraction
# ---------------------------------------------------------------------------
class Voxels(NamedTuple):
    vertices: np.ndarray
    neighbors: np.ndarray
    lower_corners: np.ndarray
    upper_corners: np.ndarray
    indices: np.ndarray
    grid_shape: tuple[int, int, int]


def compute_vertex_occupancy(occ: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    occ = _c(occ, np.int32)
    i, j, kp = occ.shape
    vocc = np.empty((i + 1, j + 1, kp + 1), np.int32)
    counts = np.empty(((i + 1) * (j + 1) * (kp + 1) + 1,), np.int32)
    lib().or_compute_vertex_occupancy(_p(occ), i, j, kp, _p(vocc), _p(counts))
    return vocc, counts


def count_occupancy(occ: np.ndarray) -> np.ndarray:
    occ = _c(occ, np.int32)
    i, j, kp = occ.shape
    counts = np.empty(((i + 1) * (j + 1) * (kp + 1) + 1,), np.int32)
    lib().or_count_occupancy(_p(occ), i, j, kp, _p(counts))
    return counts


def extract_voxels(occ: np.ndarray) -> Voxels:
    """triangle_extraction/__init__.py:31-62 on the host."""
    occ = _c(occ, np.int32)
    i, j, kp = occ.shape
    vocc, vcounts = compute_vertex_occupancy(occ)
    voff = exclusive_cumsum(vcounts)
    num_vertices = int(voff[-1])
    xoff = exclusive_cumsum(count_occupancy(occ))
    num_voxels = int(xoff[-1])
    vertices = np.zeros((num_vertices, 3), np.float32)
    neighbors = np.zeros((7, num_voxels), np.int32)
    lower = np.zeros((4, num_vertices), np.int32)
    upper = np.zeros((4, num_voxels), np.int32)
    indices = np.zeros((num_voxels,), np.int32)
    lib().or_create_voxels(
        _p(occ), _p(xoff), _p(vocc), _p(voff), i, j, kp, num_voxels, num_vertices,
        _p(vertices), _p(neighbors), _p(lower), _p(upper), _p(indices),
    )
    return Voxels(vertices, neighbors, lower, upper, indices, (i, j, kp * 32))


def dilate_occupancy(occ: np.ndarray, dilation: int) -> np.ndarray:
    occ = _c(occ, np.int32)
    if dilation == 0:
        return occ.copy()
    i, j, kp = occ.shape
    out = np.empty_like(occ)
    lib().or_dilate_occupancy(_p(occ), i, j, kp, dilation, _p(out))
    return out


# ---------------------------------------------------------------------------
# Coarse-to-fine subdivision, occupancy mesh, vertex de-duplication
# ---------------------------------------------------------------------------
def write_occupancy(voxel_indices, packed_shape) -> np.ndarray:
    idx = _c(voxel_indices, np.int32)
    occ = np.zeros(packed_shape, np.int32)
    lib().or_write_occupancy(_p(idx), idx.size, _p(occ), occ.size)
    return occ


def upscale_occupancy(occ, target_shape, mask=None) -> np.ndarray:
    """upscale_occupancy.py:24-54; ``mask`` is AND-ed into the old words."""
    occ = _c(occ, np.int32)
    i, j, kp = occ.shape
    it, jt, kt = target_shape
    assert kt % 32 == 0 and it >= i and jt >= j and kt // 32 >= kp
    out = np.empty((it, jt, kt // 32), np.int32)
    mask = None if mask is None else _c(mask, np.int32)
    lib().or_upscale_occupancy(_p(occ), _p(mask), i, j, kp, it, jt, kt // 32, _p(out))
    return out


def upscale_parameters(old_sdf, old_sh, old_occ, occ_to_upscale, new_resolution):
    """upscale_parameters.py:35-99 on the host -> (sdf, sh, occupancy)."""
    old_sdf = _c(old_sdf, np.float32)
    old_sh = _c(old_sh, np.float32)
    old_occ = _c(old_occ, np.int32)
    new_occ = upscale_occupancy(old_occ, new_resolution, mask=occ_to_upscale)
    ovocc, ovcounts = compute_vertex_occupancy(old_occ)
    ovoff = exclusive_cumsum(ovcounts)
    nvocc, nvcounts = compute_vertex_occupancy(new_occ)
    nvoff = exclusive_cumsum(nvcounts)
    n = int(nvoff[-1])
    c = old_sh.shape[0]
    sdf = np.zeros((n,), np.float32)
    sh = np.zeros((c, n, 3), np.float32)
    if n > 0:
        lib().or_upscale_parameters(_p(ovocc), _p(ovoff), _p(old_sdf), _p(old_sh), c, old_sdf.shape[0],
                                    *ovocc.shape, _p(nvocc), _p(nvoff), *nvocc.shape, n, _p(sdf), _p(sh))
    return sdf, sh, new_occ


def get_occupancy_mesh(occ, colors):
    """get_occupancy_mesh.py:32-80 on the host -> (vertices [T,3,3], colors [T,3])."""
    occ = _c(occ, np.int32)
    colors = _c(colors, np.float32)
    i, j, kp = occ.shape
    counts = np.empty(((i + 1) * (j + 1) * (kp + 1) + 1,), np.int32)
    lib().or_count_occupancy_mesh_triangles(_p(occ), i, j, kp, _p(counts))
    offsets = exclusive_cumsum(counts)
    t = int(offsets[-1])
    verts = np.zeros((t, 3, 3), np.float32)
    tcol = np.zeros((t, 3), np.float32)
    if t > 0:
        lib().or_create_occupancy_mesh_triangles(_p(occ), i, j, kp, _p(offsets), _p(colors), _p(verts), _p(tcol))
    return verts, tcol


def subdivide(vertices, sdf, sh, occ, triangle_voxel_indices, new_resolution, dilation=4, tol=1e-6):
    """tesseract.py:432-475 for one component on the host -> (sdf, sh, occupancy)."""
    canonical = index_vertices(vertices, tol).astype(np.int64)
    sdf = np.asarray(sdf, np.float32)[canonical]
    sh = np.asarray(sh, np.float32)[:, canonical, :]
    mask = write_occupancy(triangle_voxel_indices, np.asarray(occ).shape)
    mask = dilate_occupancy(mask, dilation)
    return upscale_parameters(sdf, sh, occ, mask, new_resolution)


def index_keys(keys) -> np.ndarray:
    """index_vertices.py:30-51: every key mapped to the index of the first
    equal key (a stable sort puts it at the start of its run)."""
    keys = np.asarray(keys, np.int64)
    n = keys.size
    order = np.argsort(keys, kind="stable")
    sk = keys[order]
    head = np.ones(n, bool)
    head[1:] = sk[1:] != sk[:-1]
    start = np.maximum.accumulate(np.where(head, np.arange(n), 0))
    out = np.empty(n, np.int32)
    out[order] = order[start]
    return out


def index_vertices(points, tol=1e-5) -> np.ndarray:
    """index_vertices.py:6-27 with the reference device's quantization:
    round-half-even of points * float32(1 / float32(tol))."""
    points = np.asarray(points, np.float32)
    inv = np.float32(1.0) / np.float32(tol)
    q = np.rint(points * inv).astype(np.int64)
    bits = int(np.abs(q).max()).bit_length() + 1
    if bits * 3 > 63:
        raise RuntimeError(f"need {bits*3} bits, exceed 63 bits total")
    x, y, z = q[:, 0], q[:, 1], q[:, 2]
    keys = (x << (2 * bits)) | (y << bits) | z
    return index_keys(keys)


# ---------------------------------------------------------------------------
# Per-step marching cubes
# ---------------------------------------------------------------------------
class Triangles(NamedTuple):
    vertices: np.ndarray
    signed_distances: np.ndarray
    spherical_harmonics: np.ndarray
    faces: np.ndarray
    voxel_indices: np.ndarray
    vertex_boundaries: np.ndarray
    face_boundaries: np.ndarray
    # Internals exposed for stage-by-stage parity checks.
    vertex_offsets: np.ndarray
    face_offsets: np.ndarray
    cell_codes: np.ndarray
    vertex_types: np.ndarray


def count_triangle_vertices(sdf, lower, level_sets) -> np.ndarray:
    sdf, lower, level_sets = _c(sdf, np.float32), _c(lower, np.int32), _c(level_sets, np.float32)
    g = lower.shape[1]
    s = level_sets.shape[0]
    counts = np.empty((s * g + 1,), np.int32)
    lib().or_count_triangle_vertices(_p(sdf), _p(lower), g, _p(level_sets), s, _p(counts))
    return counts


def count_triangle_faces(sdf, lower, upper, level_sets) -> tuple[np.ndarray, np.ndarray]:
    sdf, lower, upper = _c(sdf, np.float32), _c(lower, np.int32), _c(upper, np.int32)
    level_sets = _c(level_sets, np.float32)
    g, nv, s = lower.shape[1], upper.shape[1], level_sets.shape[0]
    counts = np.empty((s * nv + 1,), np.int32)
    codes = np.empty((s, nv), np.uint8)
    lib().or_count_triangle_faces(_p(sdf), _p(lower), g, _p(upper), nv, _p(level_sets), s, _p(counts), _p(codes))
    return counts, codes


def tessellate_voxels(sdf, vertices, sh, neighbors, lower, upper, indices, level_sets) -> Triangles:
    """triangle_extraction/__init__.py:75-157 on the host."""
    sdf, vertices, sh = _c(sdf, np.float32), _c(vertices, np.float32), _c(sh, np.float32)
    neighbors, lower, upper = _c(neighbors, np.int32), _c(lower, np.int32), _c(upper, np.int32)
    indices, level_sets = _c(indices, np.int32), _c(level_sets, np.float32)
    s = level_sets.shape[0]
    g, nv, c = lower.shape[1], upper.shape[1], sh.shape[0]
    voff = exclusive_cumsum(count_triangle_vertices(sdf, lower, level_sets))
    v = int(voff[-1])
    out_v = np.zeros((v, 3), np.float32)
    out_sdf = np.zeros((v,), np.float32)
    out_sh = np.zeros((c, v, 3), np.float32)
    types = np.zeros((v,), np.uint8)
    lib().or_create_triangle_vertices(
        _p(vertices), _p(sdf), _p(sh), c, _p(lower), g, _p(level_sets), s, _p(voff), v,
        _p(out_v), _p(out_sdf), _p(out_sh), _p(types),
    )
    fcounts, codes = count_triangle_faces(sdf, lower, upper, level_sets)
    foff = exclusive_cumsum(fcounts)
    f = int(foff[-1]) // 3
    faces = np.zeros((f, 3), np.int32)
    vidx = np.zeros((f,), np.int32)
    lib().or_create_triangle_faces(
        _p(neighbors), _p(indices), nv, g, _p(voff), _p(types), _p(codes), s, _p(foff), _p(faces), _p(vidx),
    )
    vb = voff[1:].reshape(s, -1)[:, -1].copy() if g > 0 else np.zeros((s,), np.int32)
    fb = foff[1:].reshape(s, -1)[:, -1].copy() // 3 if nv > 0 else np.zeros((s,), np.int32)
    return Triangles(out_v, out_sdf, out_sh, faces, vidx, vb, fb, voff, foff, codes, types)


def compute_sdf_regularizers(sdf, neighbors, lower, upper, grid_size):
    """(eikonal_pos, eikonal_neg, curvature) per voxel; grid_size = (i, j, k)."""
    sdf, neighbors = _c(sdf, np.float32), _c(neighbors, np.int32)
    lower, upper = _c(lower, np.int32), _c(upper, np.int32)
    g, nv = lower.shape[1], upper.shape[1]
    i, j, k = (int(x) for x in grid_size)
    out = [np.zeros((nv,), np.float32) for _ in range(3)]
    lib().or_compute_sdf_regularizers(_p(sdf), _p(neighbors), _p(lower), g, _p(upper), nv, k, j, i,
                                      *(_p(o) for o in out))
    return tuple(out)


def compute_sdf_regularizers_backward(sdf, neighbors, lower, upper, grid_size, g_pos, g_neg, g_curv):
    sdf, neighbors = _c(sdf, np.float32), _c(neighbors, np.int32)
    lower, upper = _c(lower, np.int32), _c(upper, np.int32)
    g_pos, g_neg, g_curv = _c(g_pos, np.float32), _c(g_neg, np.float32), _c(g_curv, np.float32)
    g, nv = lower.shape[1], upper.shape[1]
    i, j, k = (int(x) for x in grid_size)
    grad = np.zeros_like(sdf)
    lib().or_compute_sdf_regularizers_backward(_p(sdf), _p(neighbors), _p(lower), g, _p(upper), nv, k, j, i,
                                               _p(g_pos), _p(g_neg), _p(g_curv), _p(grad))
    return grad


def triangle_vertex_sources(sdf, lower, level_sets, vertex_offsets, num_vertices):
    """(origin corner, axis corner, weight t) of every triangle vertex."""
    sdf, lower = _c(sdf, np.float32), _c(lower, np.int32)
    level_sets, voff = _c(level_sets, np.float32), _c(vertex_offsets, np.int32)
    g, s = lower.shape[1], level_sets.shape[0]
    i0 = np.zeros((num_vertices,), np.int32)
    i1 = np.zeros((num_vertices,), np.int32)
    t = np.zeros((num_vertices,), np.float32)
    lib().or_triangle_vertex_sources(_p(sdf), _p(lower), g, _p(level_sets), s, _p(voff), _p(i0), _p(i1), _p(t))
    return i0, i1, t


def create_triangle_vertices_backward(sdf, sh_shape, lower, level_sets, vertex_offsets, grad_vertices,
                                      grad_sdf, grad_sh):
    """create_triangle_vertices.py:104-170: returns (d grid_vertices, d grid_sdf, d grid_sh)."""
    sdf, lower, level_sets = _c(sdf, np.float32), _c(lower, np.int32), _c(level_sets, np.float32)
    voff = _c(vertex_offsets, np.int32)
    g = lower.shape[1]
    s = level_sets.shape[0]
    c = sh_shape[0]
    v = int(voff[-1])
    gv = None if grad_vertices is None else _c(grad_vertices, np.float32)
    gd = None if grad_sdf is None else _c(grad_sdf, np.float32)
    gs = None if grad_sh is None else _c(grad_sh, np.float32)
    out_v = np.zeros((sdf.shape[0], 3), np.float32)
    out_d = np.zeros_like(sdf)
    out_sh = np.zeros(sh_shape, np.float32)
    lib().or_create_triangle_vertices_backward(
        _p(sdf), c, _p(lower), g, _p(level_sets), s, _p(voff), _p(gv), _p(gd), _p(gs), v,
        _p(out_v), _p(out_d), _p(out_sh),
    )
    return out_v, out_d, out_sh


# ---------------------------------------------------------------------------
# Rasterization
# ---------------------------------------------------------------------------
_SIGNATURES.update({
    "or_camera_positions": (None, [P, I32, P]),
    "or_project_vertices": (None, [P, I64, P, P, I32, P, P]),
    "or_evaluate_sh": (None, [P, I64, P, I32, P, I32, P]),
    "or_evaluate_sh_backward": (None, [P, I64, I32, P, I32, P, P, P]),
    "or_bound_triangles": (None, [P, P, I64, P, I64, I32, I32, I32, I32, I32, F32, P, P, P]),
    "or_generate_keys": (None, [P, I64, P, I64, P, I32, P, P, P, I32, I32, P, P, P]),
    "or_sort_pairs": (None, [P, P, I64, P, P]),
    "or_delineate_tiles": (None, [P, I64, P, I32, I32, I32, I64, P]),
    "or_intersect_and_composite_forward": (
        None, [P, P, P, I64, P, F32, P, P, P, I32, I32, I32, I32, I32, I32, I32, I32, I32, I32, P]),
    "or_intersect_and_composite_backward": (
        None, [P, P, P, I64, P, F32, P, P, P, I32, I32, I32, I32, I32, I32, I32, I32, I32, I32, P, P, P, P, P,
               I32]),
    "or_fused_hits": (None, [P, I64, P, P, P, P, I32, I32, I32, I32, I32, I32, I32, I32, I32, I32, P, P]),
    "or_intersect": (None, [P, I64, P, P, P, I32, I32, I32, I32, I32, I32, I32, I32, P, P]),
    "or_interpolate": (None, [P, P, I32, I32, I32, I32, P, P, P, I64, P, P]),
    "or_interpolate_backward": (None, [P, P, I32, I32, I32, I32, P, I64, P, P, P, P]),
    "or_composite": (None, [P, P, P, I64, I32, F32, P, P]),
    "or_composite_backward": (None, [P, P, P, I64, I32, F32, P, P, P, P, P, P, P, I32]),
})


def key_layout(key_defines) -> np.ndarray:
    d = dict(key_defines)
    return np.array([d["CAMERA_BIT_OFFSET"], d["CAMERA_BIT_LENGTH"], d["SHELL_BIT_OFFSET"], d["SHELL_BIT_LENGTH"],
                     d["TILE_BIT_OFFSET"], d["TILE_BIT_LENGTH"], d["DEPTH_BIT_OFFSET"]], np.int32)


def fused_key_defines(camera=6, shell=6, tile=20):
    """Fused layout, MSB first: camera | tile | depth | shell (__init__.py:207-212)."""
    return (("SHELL_BIT_OFFSET", 0), ("SHELL_BIT_LENGTH", shell), ("DEPTH_BIT_OFFSET", shell),
            ("DEPTH_BIT_LENGTH", 32), ("TILE_BIT_OFFSET", shell + 32), ("TILE_BIT_LENGTH", tile),
            ("CAMERA_BIT_OFFSET", shell + 32 + tile), ("CAMERA_BIT_LENGTH", camera))


def explicit_key_defines(camera=6, shell=6, tile=20):
    """Explicit layout, MSB first: camera | shell | tile | depth (__init__.py:53-58)."""
    return (("DEPTH_BIT_OFFSET", 0), ("DEPTH_BIT_LENGTH", 32), ("TILE_BIT_OFFSET", 32), ("TILE_BIT_LENGTH", tile),
            ("SHELL_BIT_OFFSET", 32 + tile), ("SHELL_BIT_LENGTH", shell), ("CAMERA_BIT_OFFSET", 32 + tile + shell),
            ("CAMERA_BIT_LENGTH", camera))


def camera_positions(extrinsics) -> np.ndarray:
    e = _c(extrinsics, np.float32)
    out = np.empty((e.shape[0], 3), np.float32)
    lib().or_camera_positions(_p(e), e.shape[0], _p(out))
    return out


def project_vertices(vertices, extrinsics, intrinsics):
    v, e, k = _c(vertices, np.float32), _c(extrinsics, np.float32), _c(intrinsics, np.float32)
    b = e.shape[0]
    xy = np.empty((b, v.shape[0], 2), np.float32)
    depth = np.empty((b, v.shape[0]), np.float32)
    lib().or_project_vertices(_p(v), v.shape[0], _p(e), _p(k), b, _p(xy), _p(depth))
    return xy, depth


def evaluate_spherical_harmonics(vertices, sh, extrinsics, sh_degree):
    v, sh = _c(vertices, np.float32), _c(sh, np.float32)
    campos = camera_positions(extrinsics)
    b = campos.shape[0]
    out = np.empty((b, v.shape[0], 3), np.float32)
    lib().or_evaluate_sh(_p(v), v.shape[0], _p(sh), sh_degree, _p(campos), b, _p(out))
    return out


def evaluate_spherical_harmonics_backward(vertices, sh_shape, extrinsics, sh_degree, colors, grad_colors):
    v = _c(vertices, np.float32)
    campos = camera_positions(extrinsics)
    out = np.zeros(sh_shape, np.float32)
    colors, grad_colors = _c(colors, np.float32), _c(grad_colors, np.float32)
    lib().or_evaluate_sh_backward(_p(v), v.shape[0], sh_degree, _p(campos), campos.shape[0],
                                  _p(colors), _p(grad_colors), _p(out))
    return out


def bound_triangles(xy, depth, faces, tile_shape, grid_shape, near_plane):
    xy, depth, faces = _c(xy, np.float32), _c(depth, np.float32), _c(faces, np.int32)
    b, v, _ = xy.shape
    f = faces.shape[0]
    tmin = np.empty((b, f, 2), np.int32)
    tmax = np.empty((b, f, 2), np.int32)
    count = np.empty((b, f), np.int32)
    lib().or_bound_triangles(_p(xy), _p(depth), v, _p(faces), f, b, tile_shape[0], tile_shape[1], grid_shape[0],
                             grid_shape[1], near_plane, _p(tmin), _p(tmax), _p(count))
    return tmin, tmax, count


def generate_keys(depth, faces, shell_face_boundaries, tmin, tmax, count, grid_width, key_defines):
    depth, faces = _c(depth, np.float32), _c(faces, np.int32)
    sfb = _c(shell_face_boundaries, np.int32)
    offsets = inclusive_cumsum_i64(count.reshape(-1))
    k = int(offsets[-1]) if offsets.size else 0
    keys = np.zeros((k,), np.int64)
    tri = np.zeros((k,), np.int32)
    b, v = depth.shape
    tmin, tmax, layout = _c(tmin, np.int32), _c(tmax, np.int32), key_layout(key_defines)
    lib().or_generate_keys(_p(depth), v, _p(faces), faces.shape[0], _p(sfb), sfb.shape[0], _p(tmin), _p(tmax),
                           _p(offsets), b, grid_width, _p(layout), _p(keys), _p(tri))
    return keys, tri


def sort_pairs(keys, tri):
    keys, tri = _c(keys, np.int64), _c(tri, np.int32)
    ok, ot = np.empty_like(keys), np.empty_like(tri)
    lib().or_sort_pairs(_p(keys), _p(tri), keys.size, _p(ok), _p(ot))
    return ok, ot


def delineate_tiles(sorted_keys, key_defines, separate_shells, num_cameras, num_shells, num_tiles):
    keys = _c(sorted_keys, np.int64)
    sd = num_shells if separate_shells else 1
    out = np.empty((num_cameras, sd, num_tiles, 2), np.int64)
    layout = key_layout(key_defines)
    lib().or_delineate_tiles(_p(keys), keys.size, _p(layout), int(separate_shells), num_cameras, sd, num_tiles,
                             _p(out))
    return out


class FusedRender(NamedTuple):
    xy: np.ndarray
    depth: np.ndarray
    tile_min: np.ndarray
    tile_max: np.ndarray
    counts: np.ndarray
    keys: np.ndarray
    tri: np.ndarray
    sorted_keys: np.ndarray
    sorted_tri: np.ndarray
    tile_boundaries: np.ndarray
    colors: np.ndarray
    raw: np.ndarray  # [B, 4, H, W] compositor output before the epilogue
    image: np.ndarray  # [B, 3, H, W] after background / clip


def intersect_and_composite(xy, colors, sdf, faces, sharpness, sorted_keys, sorted_tri, tile_boundaries, num_shells,
                            tile_shape, image_shape, key_defines):
    xy, colors, sdf, faces = _c(xy, np.float32), _c(colors, np.float32), _c(sdf, np.float32), _c(faces, np.int32)
    b, v, _ = xy.shape
    h, w = image_shape
    rows, cols = -(-h // tile_shape[0]), -(-w // tile_shape[1])
    d = dict(key_defines)
    out = np.zeros((b, 4, h, w), np.float32)
    sk, st, tb = _c(sorted_keys, np.int64), _c(sorted_tri, np.int32), _c(tile_boundaries, np.int64)
    lib().or_intersect_and_composite_forward(
        _p(xy), _p(colors), _p(sdf), v, _p(faces), float(sharpness), _p(sk), _p(st), _p(tb), b, num_shells, rows,
        cols, tile_shape[0], tile_shape[1], h, w, d["SHELL_BIT_OFFSET"], d["SHELL_BIT_LENGTH"], _p(out))
    return out


def intersect_and_composite_backward(xy, colors, sdf, faces, sharpness, sorted_keys, sorted_tri, tile_boundaries,
                                     num_shells, tile_shape, image_shape, key_defines, out, grad_out, exact=False):
    xy, colors, sdf, faces = _c(xy, np.float32), _c(colors, np.float32), _c(sdf, np.float32), _c(faces, np.int32)
    b, v, _ = xy.shape
    h, w = image_shape
    rows, cols = -(-h // tile_shape[0]), -(-w // tile_shape[1])
    d = dict(key_defines)
    gcol = np.zeros_like(colors)
    gsdf = np.zeros_like(sdf)
    gsharp = np.zeros((1,), np.float32)
    sk, st, tb = _c(sorted_keys, np.int64), _c(sorted_tri, np.int32), _c(tile_boundaries, np.int64)
    out, grad_out = _c(out, np.float32), _c(grad_out, np.float32)
    lib().or_intersect_and_composite_backward(
        _p(xy), _p(colors), _p(sdf), v, _p(faces), float(sharpness), _p(sk), _p(st), _p(tb), b, num_shells, rows,
        cols, tile_shape[0], tile_shape[1], h, w, d["SHELL_BIT_OFFSET"], d["SHELL_BIT_LENGTH"], _p(out),
        _p(grad_out), _p(gcol), _p(gsdf), _p(gsharp), int(exact))
    return gcol, gsdf, float(gsharp[0])


def fused_hits(xy, faces, sorted_keys, sorted_tri, tile_boundaries, num_shells, tile_shape, image_shape, key_defines):
    """Per pixel, the hits the fused walk accepts in compositing order:
    faces [B, H, W, S] (-1 = none) and barycentrics [B, H, W, S, 3]."""
    xy, faces = _c(xy, np.float32), _c(faces, np.int32)
    b, v, _ = xy.shape
    h, w = image_shape
    rows, cols = -(-h // tile_shape[0]), -(-w // tile_shape[1])
    d = dict(key_defines)
    out_face = np.full((b, h, w, num_shells), -1, np.int32)
    out_uvw = np.zeros((b, h, w, num_shells, 3), np.float32)
    sk, st, tb = _c(sorted_keys, np.int64), _c(sorted_tri, np.int32), _c(tile_boundaries, np.int64)
    lib().or_fused_hits(_p(xy), v, _p(faces), _p(sk), _p(st), _p(tb), b, num_shells, rows, cols, tile_shape[0],
                        tile_shape[1], h, w, d["SHELL_BIT_OFFSET"], d["SHELL_BIT_LENGTH"], _p(out_face), _p(out_uvw))
    return out_face, out_uvw


def render_fused(extrinsics, intrinsics, image_shape, vertices, faces, shell_face_boundaries, sdf, sh, sh_degree,
                 sharpness, background, tile_shape=(16, 16), near_plane=0.2, num_camera_bits=6, num_shell_bits=6,
                 num_tile_bits=20) -> FusedRender:
    """triangle_rasterization/__init__.py:167-287 on the host (ssaa = 1)."""
    h, w = image_shape
    b = extrinsics.shape[0]
    s = shell_face_boundaries.shape[0]
    rows, cols = -(-h // tile_shape[0]), -(-w // tile_shape[1])
    kd = fused_key_defines(num_camera_bits, num_shell_bits, num_tile_bits)
    xy, depth = project_vertices(vertices, extrinsics, intrinsics)
    tmin, tmax, count = bound_triangles(xy, depth, faces, tile_shape, (rows, cols), near_plane)
    keys, tri = generate_keys(depth, faces, shell_face_boundaries, tmin, tmax, count, cols, kd)
    sk, st = sort_pairs(keys, tri)
    tb = delineate_tiles(sk, kd, False, b, s, rows * cols)
    colors = evaluate_spherical_harmonics(vertices, sh, extrinsics, sh_degree)
    raw = intersect_and_composite(xy, colors, sdf, faces, sharpness, sk, st, tb.reshape(b, rows * cols, 2), s,
                                  tile_shape, image_shape, kd)
    bg = np.asarray(background, np.float32)
    image = np.clip(raw[:, :3] + raw[:, 3:4] * bg[None, :, None, None], 0.0, 1.0)
    return FusedRender(xy, depth, tmin, tmax, count, keys, tri, sk, st, tb, colors, raw, image)


def render_explicit(extrinsics, intrinsics, image_shape, vertices, faces, shell_face_boundaries, sdf, sh, sh_degree,
                    sharpness, background, tile_shape=(16, 16), near_plane=0.2, num_camera_bits=6, num_shell_bits=6,
                    num_tile_bits=20) -> np.ndarray:
    """triangle_rasterization/__init__.py:97-164 on the host (ssaa = 1):
    per-shell rasterization, interpolation, then compositing with the
    background blended in (composite.py:117). Returns [B, 3, H, W]."""
    h, w = image_shape
    b = extrinsics.shape[0]
    s = shell_face_boundaries.shape[0]
    rows, cols = -(-h // tile_shape[0]), -(-w // tile_shape[1])
    kd = explicit_key_defines(num_camera_bits, num_shell_bits, num_tile_bits)
    xy, depth = project_vertices(vertices, extrinsics, intrinsics)
    tmin, tmax, count = bound_triangles(xy, depth, faces, tile_shape, (rows, cols), near_plane)
    keys, tri = generate_keys(depth, faces, shell_face_boundaries, tmin, tmax, count, cols, kd)
    sk, st = sort_pairs(keys, tri)
    tb = delineate_tiles(sk, kd, True, b, s, rows * cols)
    uv, index = intersect(xy, faces, st, tb, s, tile_shape, image_shape)
    colors = evaluate_spherical_harmonics(vertices, sh, extrinsics, sh_degree)
    isdf, icol = interpolate(uv, index, faces, sdf, colors)
    per_pixel_sdf = isdf.transpose(0, 2, 3, 1).reshape(-1, s)
    per_pixel_col = icol.transpose(0, 2, 3, 1, 4).reshape(-1, s, 3)
    mask = (index != -1).transpose(0, 2, 3, 1).reshape(-1, s)
    out_c, out_t = composite(per_pixel_sdf, per_pixel_col, mask, sharpness)
    image = out_c + np.asarray(background, np.float32)[None, :] * out_t[:, None]
    return image.reshape(b, h, w, 3).transpose(0, 3, 1, 2)


def intersect(xy, faces, sorted_tri, tile_boundaries, num_shells, tile_shape, image_shape):
    xy, faces = _c(xy, np.float32), _c(faces, np.int32)
    b, v, _ = xy.shape
    h, w = image_shape
    rows, cols = -(-h // tile_shape[0]), -(-w // tile_shape[1])
    uv = np.zeros((b * num_shells, h, w, 2), np.float32)
    index = np.zeros((b * num_shells, h, w), np.int32)
    st, tb = _c(sorted_tri, np.int32), _c(tile_boundaries, np.int64)
    lib().or_intersect(_p(xy), v, _p(faces), _p(st), _p(tb), b,
                       num_shells, rows, cols, tile_shape[0], tile_shape[1], h, w, _p(uv), _p(index))
    return uv.reshape(b, num_shells, h, w, 2), index.reshape(b, num_shells, h, w)


def interpolate(uv, index, faces, sdf, colors):
    uv, index, faces = _c(uv, np.float32), _c(index, np.int32), _c(faces, np.int32)
    sdf, colors = _c(sdf, np.float32), _c(colors, np.float32)
    b, s, h, w, _ = uv.shape
    out_sdf = np.empty((b, s, h, w), np.float32)
    out_col = np.empty((b, s, h, w, 3), np.float32)
    lib().or_interpolate(_p(uv), _p(index), b, s, h, w, _p(faces), _p(sdf), _p(colors), sdf.shape[0], _p(out_sdf),
                         _p(out_col))
    return out_sdf, out_col


def interpolate_backward(uv, index, faces, v, num_cameras, grad_sdf, grad_colors):
    uv, index, faces = _c(uv, np.float32), _c(index, np.int32), _c(faces, np.int32)
    b, s, h, w, _ = uv.shape
    gsdf = np.zeros((v,), np.float32)
    gcol = np.zeros((num_cameras, v, 3), np.float32)
    grad_sdf, grad_colors = _c(grad_sdf, np.float32), _c(grad_colors, np.float32)
    lib().or_interpolate_backward(_p(uv), _p(index), b, s, h, w, _p(faces), v, _p(grad_sdf), _p(grad_colors),
                                  _p(gsdf), _p(gcol))
    return gsdf, gcol


def composite(sdf, colors, mask, sharpness):
    sdf, colors = _c(sdf, np.float32), _c(colors, np.float32)
    mask = _c(mask, np.uint8)
    p, s = sdf.shape
    out_c = np.empty((p, 3), np.float32)
    out_t = np.empty((p,), np.float32)
    lib().or_composite(_p(sdf), _p(colors), _p(mask), p, s, float(sharpness), _p(out_c), _p(out_t))
    return out_c, out_t


def composite_backward(sdf, colors, mask, sharpness, out_c, out_t, grad_c, grad_t, exact=False):
    sdf, colors = _c(sdf, np.float32), _c(colors, np.float32)
    mask = _c(mask, np.uint8)
    p, s = sdf.shape
    gsdf = np.zeros_like(sdf)
    gcol = np.zeros_like(colors)
    gsharp = np.zeros((1,), np.float32)
    out_c, out_t = _c(out_c, np.float32), _c(out_t, np.float32)
    grad_c, grad_t = _c(grad_c, np.float32), _c(grad_t, np.float32)
    lib().or_composite_backward(_p(sdf), _p(colors), _p(mask), p, s, float(sharpness), _p(out_c), _p(out_t),
                                _p(grad_c), _p(grad_t), _p(gsdf), _p(gcol), _p(gsharp), int(exact))
    return gsdf, gcol, float(gsharp[0])
