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
    "or_count_triangle_vertices": (None, [P, P, I64, P, I32, P]),
    "or_create_triangle_vertices": (None, [P, P, P, I32, P, I64, P, I32, P, I64, P, P, P, P]),
    "or_create_triangle_vertices_backward": (None, [P, I32, P, I64, P, I32, P, P, P, P, I64, P, P, P]),
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
