"""numpy front end of the reference's own kernels compiled on the host
(``oracle/_ref/libref.so``, built by ``oracle/build_ref.py`` from the mounted
reference tree). Test infrastructure only: used to pin the oracle.

``available()`` is False when the reference tree is not mounted; callers
then rely on the committed golden fixtures instead.
"""

from __future__ import annotations

import ctypes
from ctypes import c_float, c_int, c_int64, c_void_p

import numpy as np

from . import build_ref

P, I, I64, F32 = c_void_p, c_int, c_int64, c_float

_SIGNATURES = {
    "ref_compute_vertex_occupancy": [P, I, I, I, P, P],
    "ref_count_occupancy": [P, I, I, I, P],
    "ref_create_voxels": [P, P, P, P, I, I, I, I64, I64, P, P, P, P, P],
    "ref_dilate_occupancy": [P, I, I, I, I, P],
    "ref_write_occupancy": [P, I64, P, I64],
    "ref_upscale_occupancy": [P, I, I, I, I, I, I, P],
    "ref_upscale_parameters": [I, P, P, P, P, I64, I, I, I, P, P, I, I, I, I64, P, P],
    "ref_count_occupancy_mesh_triangles": [P, I, I, I, P],
    "ref_create_occupancy_mesh_triangles": [P, I, I, I, P, I64, P, P, P],
    "ref_count_triangle_vertices": [P, P, I64, P, I, P],
    "ref_create_triangle_vertices": [P, P, P, I, P, I64, P, I, P, I64, P, P, P, P],
    "ref_count_triangle_faces": [P, P, I64, P, I64, P, I, P, P],
    "ref_compute_sdf_regularizers": [P, I64, P, P, P, I64, I, I, I, P, P, P],
    "ref_create_triangle_faces": [P, I64, P, P, I64, P, P, I64, P, P, I, P, P, P, I64],
    "ref_project_vertices": [P, P, I, P, I64, P, P],
    "ref_bound_triangles": [P, P, I, I64, P, I64, I, I, I, I, F32, P, P, P],
    "ref_generate_keys": [I, P, I, I64, P, I64, P, I, P, P, P, I, I64, P, P],
    "ref_delineate_tiles": [I, P, I64, I, I, I64, I, P],
    "ref_evaluate_sh": [I, P, I64, P, I, P, I, P],
    "ref_intersect_and_composite_forward": [P, P, P, I, I64, P, I64, F32, P, P, I64, P, I, I, I, I, I, P],
    "ref_intersect": [P, I, I64, P, I64, P, I64, P, I, I, I, I, I, P, P],
    "ref_interpolate": [P, P, I, I, I, I, P, I64, P, P, I64, P, P],
    "ref_composite_forward": [P, P, P, I64, I, F32, P, P],
    "ref_intersect_and_composite_backward": [P, P, P, I, I64, P, I64, F32, P, P, I64, P, I, I, I, I, I, P, P, P, P,
                                             P],
    "ref_composite_backward": [P, P, P, I64, I, F32, P, P, P, P, P, P, P],
}

_lib = None


def available() -> bool:
    return lib() is not None


def lib():
    global _lib
    if _lib is None:
        path = build_ref.build()
        if path is None:
            return None
        _lib = ctypes.CDLL(str(path))
        for name, argtypes in _SIGNATURES.items():
            fn = getattr(_lib, name)
            fn.restype = None
            fn.argtypes = argtypes
    return _lib


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return a.ctypes.data if a is not None and a.size > 0 else None


def extract_voxels(occ):
    occ = _c(occ, np.int32)
    i, j, kp = occ.shape
    vocc = np.zeros((i + 1, j + 1, kp + 1), np.int32)
    vcounts = np.zeros(((i + 1) * (j + 1) * (kp + 1) + 1,), np.int32)
    lib().ref_compute_vertex_occupancy(_p(occ), i, j, kp, _p(vocc), _p(vcounts))
    voff = np.concatenate(([0], np.cumsum(vcounts)[:-1])).astype(np.int32)
    xcounts = np.zeros_like(vcounts)
    lib().ref_count_occupancy(_p(occ), i, j, kp, _p(xcounts))
    xoff = np.concatenate(([0], np.cumsum(xcounts)[:-1])).astype(np.int32)
    nv, g = int(xoff[-1]), int(voff[-1])
    out = dict(vertices=np.zeros((g, 3), np.float32), neighbors=np.zeros((7, nv), np.int32),
               lower_corners=np.zeros((4, g), np.int32), upper_corners=np.zeros((4, nv), np.int32),
               indices=np.zeros((nv,), np.int32))
    lib().ref_create_voxels(_p(occ), _p(xoff), _p(vocc), _p(voff), i, j, kp, nv, g, _p(out["vertices"]),
                            _p(out["neighbors"]), _p(out["lower_corners"]), _p(out["upper_corners"]),
                            _p(out["indices"]))
    out.update(vertex_occupancy=vocc, vertex_counts=vcounts, voxel_counts=xcounts)
    return out


def dilate_occupancy(occ, d):
    occ = _c(occ, np.int32)
    out = np.zeros_like(occ)
    lib().ref_dilate_occupancy(_p(occ), *occ.shape, d, _p(out))
    return out


def python_module(relative_path: str):
    """Imports one of the reference's pure-Python modules (e.g.
    ``triangle_extraction/index_vertices.py``) from the mounted tree. Its
    ``jaxtyping`` annotations are satisfied by a stand-in module when the
    package is not installed (annotations only; no behaviour)."""
    import importlib.util
    import sys
    import types

    if "jaxtyping" not in sys.modules:
        try:
            import jaxtyping  # noqa: F401
        except ImportError:
            stub = types.ModuleType("jaxtyping")

            class _Annotation:
                def __class_getitem__(cls, item):
                    return object

            for name in ("Float", "Float32", "Int", "Int32", "Int64", "Bool", "Shaped"):
                setattr(stub, name, _Annotation)
            sys.modules["jaxtyping"] = stub
    path = build_ref.reference_root() / relative_path
    spec = importlib.util.spec_from_file_location("reference_" + path.stem, path)
    module = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(module)
    return module


def write_occupancy(voxel_indices, packed_shape):
    idx = _c(voxel_indices, np.int32)
    occ = np.zeros(packed_shape, np.int32)
    lib().ref_write_occupancy(_p(idx), idx.size, _p(occ), occ.size)
    return occ


def upscale_occupancy(occ, target_shape):
    occ = _c(occ, np.int32)
    it, jt, kt = target_shape
    out = np.zeros((it, jt, kt // 32), np.int32)
    lib().ref_upscale_occupancy(_p(occ), *occ.shape, it, jt, kt // 32, _p(out))
    return out


def _vertex_offsets(occ):
    i, j, kp = occ.shape
    vocc = np.zeros((i + 1, j + 1, kp + 1), np.int32)
    vcounts = np.zeros(((i + 1) * (j + 1) * (kp + 1) + 1,), np.int32)
    lib().ref_compute_vertex_occupancy(_p(occ), i, j, kp, _p(vocc), _p(vcounts))
    voff = np.concatenate(([0], np.cumsum(vcounts)[:-1])).astype(np.int32)
    return vocc, voff


def upscale_parameters(old_sdf, old_sh, old_occ, occ_to_upscale, new_resolution):
    """upscale_parameters.py:35-99 with the reference's kernels (numpy scans)."""
    old_sdf, old_sh = _c(old_sdf, np.float32), _c(old_sh, np.float32)
    old_occ = _c(old_occ, np.int32)
    new_occ = upscale_occupancy(old_occ & _c(occ_to_upscale, np.int32), new_resolution)
    ovocc, ovoff = _vertex_offsets(old_occ)
    nvocc, nvoff = _vertex_offsets(new_occ)
    n, c = int(nvoff[-1]), old_sh.shape[0]
    sdf, sh = np.zeros((n,), np.float32), np.zeros((c, n, 3), np.float32)
    if n > 0:
        lib().ref_upscale_parameters(c, _p(ovocc), _p(ovoff), _p(old_sdf), _p(old_sh), old_sdf.shape[0],
                                     *ovocc.shape, _p(nvocc), _p(nvoff), *nvocc.shape, n, _p(sdf), _p(sh))
    return sdf, sh, new_occ


def get_occupancy_mesh(occ, colors):
    """get_occupancy_mesh.py:32-80 with the reference's kernels (numpy scan)."""
    occ, colors = _c(occ, np.int32), _c(colors, np.float32)
    i, j, kp = occ.shape
    counts = np.zeros(((i + 1) * (j + 1) * (kp + 1) + 1,), np.int32)
    lib().ref_count_occupancy_mesh_triangles(_p(occ), i, j, kp, _p(counts))
    offsets = np.concatenate(([0], np.cumsum(counts)[:-1])).astype(np.int32)
    t = int(offsets[-1])
    verts, tcol = np.zeros((t, 3, 3), np.float32), np.zeros((t, 3), np.float32)
    if t > 0:
        lib().ref_create_occupancy_mesh_triangles(_p(occ), i, j, kp, _p(offsets), t, _p(verts), _p(tcol),
                                                  _p(colors))
    return verts, tcol


def tessellate(sdf, vertices, sh, neighbors, lower, upper, indices, level_sets):
    """triangle_extraction/__init__.py:75-157 with the reference's kernels
    (the exclusive scans are numpy cumsums)."""
    sdf, vertices, sh = _c(sdf, np.float32), _c(vertices, np.float32), _c(sh, np.float32)
    neighbors, lower, upper, indices = (_c(x, np.int32) for x in (neighbors, lower, upper, indices))
    ls = _c(level_sets, np.float32)
    s, g, nv, c = ls.shape[0], lower.shape[1], upper.shape[1], sh.shape[0]
    counts = np.zeros((s * g + 1,), np.int32)
    lib().ref_count_triangle_vertices(_p(sdf), _p(lower), g, _p(ls), s, _p(counts))
    voff = np.concatenate(([0], np.cumsum(counts)[:-1])).astype(np.int32)
    v = int(voff[-1])
    out_v, out_d = np.zeros((v, 3), np.float32), np.zeros((v,), np.float32)
    out_sh, types = np.zeros((c, v, 3), np.float32), np.zeros((v,), np.uint8)
    lib().ref_create_triangle_vertices(_p(vertices), _p(sdf), _p(sh), c, _p(lower), g, _p(ls), s, _p(voff), v,
                                       _p(out_v), _p(out_d), _p(out_sh), _p(types))
    fcounts = np.zeros((s * nv + 1,), np.int32)
    codes = np.zeros((s, nv), np.uint8)
    lib().ref_count_triangle_faces(_p(sdf), _p(lower), g, _p(upper), nv, _p(ls), s, _p(fcounts), _p(codes))
    foff = np.concatenate(([0], np.cumsum(fcounts)[:-1])).astype(np.int32)
    f = int(foff[-1]) // 3
    faces, vidx = np.zeros((f, 3), np.int32), np.zeros((f,), np.int32)
    lib().ref_create_triangle_faces(_p(sdf), g, _p(neighbors), _p(indices), nv, _p(voff), _p(types), v, _p(codes),
                                    _p(ls), s, _p(foff), _p(faces), _p(vidx), f)
    return dict(vertices=out_v, signed_distances=out_d, spherical_harmonics=out_sh, faces=faces, voxel_indices=vidx,
                vertex_offsets=voff, face_offsets=foff, cell_codes=codes, vertex_types=types, vertex_counts=counts,
                face_counts=fcounts)


def project_vertices(vertices, extrinsics, intrinsics):
    v, e, k = _c(vertices, np.float32), _c(extrinsics, np.float32), _c(intrinsics, np.float32)
    b = e.shape[0]
    xy, depth = np.zeros((b, v.shape[0], 2), np.float32), np.zeros((b, v.shape[0]), np.float32)
    lib().ref_project_vertices(_p(e), _p(k), b, _p(v), v.shape[0], _p(xy), _p(depth))
    return xy, depth


def bound_triangles(xy, depth, faces, tile_shape, grid_shape, near):
    xy, depth, faces = _c(xy, np.float32), _c(depth, np.float32), _c(faces, np.int32)
    b, v, _ = xy.shape
    f = faces.shape[0]
    mn, mx, ct = np.zeros((b, f, 2), np.int32), np.zeros((b, f, 2), np.int32), np.zeros((b, f), np.int32)
    lib().ref_bound_triangles(_p(xy), _p(depth), b, v, _p(faces), f, tile_shape[0], tile_shape[1], grid_shape[0],
                              grid_shape[1], near, _p(mn), _p(mx), _p(ct))
    return mn, mx, ct


def generate_keys(explicit, depth, faces, sfb, tmin, tmax, count, grid_width):
    depth, faces, sfb = _c(depth, np.float32), _c(faces, np.int32), _c(sfb, np.int32)
    tmin, tmax = _c(tmin, np.int32), _c(tmax, np.int32)
    offsets = np.cumsum(count.reshape(-1).astype(np.int64))
    k = int(offsets[-1]) if offsets.size else 0
    keys, tri = np.zeros((k,), np.int64), np.zeros((k,), np.int32)
    b, v = depth.shape
    lib().ref_generate_keys(int(explicit), _p(depth), b, v, _p(faces), faces.shape[0], _p(sfb), sfb.shape[0],
                            _p(tmin), _p(tmax), _p(offsets), grid_width, k, _p(keys), _p(tri))
    return keys, tri


def delineate_tiles(explicit, keys, b, sd, t, separate):
    keys = _c(keys, np.int64)
    out = np.zeros((b, sd, t, 2), np.int64)
    lib().ref_delineate_tiles(int(explicit), _p(keys), keys.size, b, sd, t, int(separate), _p(out))
    return out


def evaluate_sh(degree, vertices, sh, campos):
    v, sh, cp = _c(vertices, np.float32), _c(sh, np.float32), _c(campos, np.float32)
    out = np.zeros((cp.shape[0], v.shape[0], 3), np.float32)
    lib().ref_evaluate_sh(degree, _p(v), v.shape[0], _p(sh), sh.shape[0], _p(cp), cp.shape[0], _p(out))
    return out


def intersect_and_composite(xy, colors, sdf, faces, sharpness, keys, tri, bounds, num_shells, image_shape):
    xy, colors, sdf, faces = _c(xy, np.float32), _c(colors, np.float32), _c(sdf, np.float32), _c(faces, np.int32)
    keys, tri, bounds = _c(keys, np.int64), _c(tri, np.int32), _c(bounds, np.int64)
    b, v, _ = xy.shape
    h, w = image_shape
    rows, cols = -(-h // 16), -(-w // 16)
    out = np.zeros((b, 4, h, w), np.float32)
    lib().ref_intersect_and_composite_forward(_p(xy), _p(colors), _p(sdf), b, v, _p(faces), faces.shape[0],
                                              float(sharpness), _p(keys), _p(tri), keys.size, _p(bounds), num_shells,
                                              rows, cols, h, w, _p(out))
    return out


def intersect(xy, faces, tri, bounds, num_shells, image_shape):
    xy, faces, tri, bounds = _c(xy, np.float32), _c(faces, np.int32), _c(tri, np.int32), _c(bounds, np.int64)
    b, v, _ = xy.shape
    h, w = image_shape
    rows, cols = -(-h // 16), -(-w // 16)
    uv = np.zeros((b * num_shells, h, w, 2), np.float32)
    index = np.zeros((b * num_shells, h, w), np.int32)
    lib().ref_intersect(_p(xy), b, v, _p(faces), faces.shape[0], _p(tri), tri.size, _p(bounds), num_shells, rows,
                        cols, h, w, _p(uv), _p(index))
    return uv.reshape(b, num_shells, h, w, 2), index.reshape(b, num_shells, h, w)


def interpolate(uv, index, faces, sdf, colors):
    uv, index, faces = _c(uv, np.float32), _c(index, np.int32), _c(faces, np.int32)
    sdf, colors = _c(sdf, np.float32), _c(colors, np.float32)
    b, s, h, w, _ = uv.shape
    out_sdf, out_col = np.zeros((b, s, h, w), np.float32), np.zeros((b, s, h, w, 3), np.float32)
    lib().ref_interpolate(_p(uv), _p(index), b, s, h, w, _p(faces), faces.shape[0], _p(sdf), _p(colors),
                          sdf.shape[0], _p(out_sdf), _p(out_col))
    return out_sdf, out_col


def composite(sdf, colors, mask, sharpness):
    sdf, colors, mask = _c(sdf, np.float32), _c(colors, np.float32), _c(mask, np.uint8)
    p, s = sdf.shape
    oc, ot = np.zeros((p, 3), np.float32), np.zeros((p,), np.float32)
    lib().ref_composite_forward(_p(sdf), _p(colors), _p(mask), p, s, float(sharpness), _p(oc), _p(ot))
    return oc, ot


def intersect_and_composite_backward(xy, colors, sdf, faces, sharpness, keys, tri, bounds, num_shells, image_shape,
                                     out, grad_out):
    """The reference's fused backward (hand-written kernel, shim adjoints for
    its bwd_diff helpers): gradients of colours, signed distances, sharpness."""
    xy, colors, sdf, faces = _c(xy, np.float32), _c(colors, np.float32), _c(sdf, np.float32), _c(faces, np.int32)
    keys, tri, bounds = _c(keys, np.int64), _c(tri, np.int32), _c(bounds, np.int64)
    out, grad_out = _c(out, np.float32), _c(grad_out, np.float32)
    b, v, _ = xy.shape
    h, w = image_shape
    rows, cols = -(-h // 16), -(-w // 16)
    gc, gs, gsh = np.zeros_like(colors), np.zeros_like(sdf), np.zeros((1,), np.float32)
    lib().ref_intersect_and_composite_backward(_p(xy), _p(colors), _p(sdf), b, v, _p(faces), faces.shape[0],
                                               float(sharpness), _p(keys), _p(tri), keys.size, _p(bounds),
                                               num_shells, rows, cols, h, w, _p(out), _p(grad_out), _p(gc), _p(gs),
                                               _p(gsh))
    return gc, gs, float(gsh[0])


def composite_backward(sdf, colors, mask, sharpness, out_colors, out_t, grad_colors, grad_t):
    sdf, colors, mask = _c(sdf, np.float32), _c(colors, np.float32), _c(mask, np.uint8)
    out_colors, out_t = _c(out_colors, np.float32), _c(out_t, np.float32)
    grad_colors, grad_t = _c(grad_colors, np.float32), _c(grad_t, np.float32)
    p, s = sdf.shape
    gsdf, gcol, gsh = np.zeros_like(sdf), np.zeros_like(colors), np.zeros((1,), np.float32)
    lib().ref_composite_backward(_p(sdf), _p(colors), _p(mask), p, s, float(sharpness), _p(out_colors), _p(out_t),
                                 _p(grad_colors), _p(grad_t), _p(gsdf), _p(gcol), _p(gsh))
    return gsdf, gcol, float(gsh[0])


def compute_sdf_regularizers(sdf, neighbors, lower, upper, grid_size):
    sdf, neighbors = _c(sdf, np.float32), _c(neighbors, np.int32)
    lower, upper = _c(lower, np.int32), _c(upper, np.int32)
    g, nv = lower.shape[1], upper.shape[1]
    i, j, k = (int(x) for x in grid_size)
    out = [np.zeros((nv,), np.float32) for _ in range(3)]
    lib().ref_compute_sdf_regularizers(_p(sdf), g, _p(neighbors), _p(lower), _p(upper), nv, k, j, i,
                                       *(_p(o) for o in out))
    return tuple(out)
