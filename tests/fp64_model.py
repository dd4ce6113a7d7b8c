"""FP64 model of the differentiable part of the render path, for finite
differences.

Geometry is held fixed, as in the reference's adjoint: triangle vertex
positions are not differentiated (intersect_and_composite.slang:6,35-36) and
the marching-cubes weight t is detached (create_triangle_vertices.slang:92-96).
With the hits, barycentrics and t fixed, the image is a smooth function of
the grid signed distances, the grid SH coefficients, the per-vertex colours /
signed distances and the sharpness, which this module evaluates in float64:

* vertex values: x = x0 + t (x1 - x0) over the two corners of the crossing
  edge (create_triangle_vertices.slang:105-127),
* colours: real SH up to degree 3, rgb = max(sum_k basis_k(dir) sh_k + 0.5, 0)
  with dir = normalize(vertex - camera centre)
  (evaluate_spherical_harmonics.slang:124-270),
* compositing over the hits of each pixel, front to back:
  cdf = 1 / (1 + exp(-sdf s)), alpha = clamp(((cdf_o - cdf_i) + 1e-5) /
  (cdf_o + 1e-5), 0, 1), rgb += c T alpha, T *= 1 - alpha, starting from an
  outer sample at sdf = 1e10 (intersect_and_composite.slang:153-172,319;
  composite.slang:60-120).
"""

from __future__ import annotations

import numpy as np

SH_C0 = 0.28209479177387814
SH_C1 = 0.4886025119029199
SH_C2 = (1.0925484305920792, -1.0925484305920792, 0.31539156525252005, -1.0925484305920792, 0.5462742152960396)
SH_C3 = (-0.5900435899266435, 2.890611442640554, -0.4570457994644658, 0.3731763325901154, -0.4570457994644658,
         1.445305721320277, -0.5900435899266435)


def lerp_vertices(grid_values: np.ndarray, i0: np.ndarray, i1: np.ndarray, t: np.ndarray) -> np.ndarray:
    """x0 + t (x1 - x0) along the first axis of ``grid_values`` ([G, ...])."""
    x0, x1 = grid_values[i0], grid_values[i1]
    tt = t.astype(np.float64).reshape((-1,) + (1,) * (grid_values.ndim - 1))
    return x0 + tt * (x1 - x0)


def sh_basis(d: np.ndarray, n: int) -> np.ndarray:
    """[N, n] real SH basis at unit directions d [N, 3]."""
    x, y, z = d[:, 0], d[:, 1], d[:, 2]
    out = [np.full_like(x, SH_C0)]
    if n > 1:
        out += [-SH_C1 * y, SH_C1 * z, -SH_C1 * x]
    if n > 4:
        xx, yy, zz, xy, yz, xz = x * x, y * y, z * z, x * y, y * z, x * z
        out += [SH_C2[0] * xy, SH_C2[1] * yz, SH_C2[2] * (2 * zz - xx - yy), SH_C2[3] * xz, SH_C2[4] * (xx - yy)]
    if n > 9:
        out += [SH_C3[0] * y * (3 * xx - yy), SH_C3[1] * xy * z, SH_C3[2] * y * (4 * zz - xx - yy),
                SH_C3[3] * z * (2 * zz - 3 * xx - 3 * yy), SH_C3[4] * x * (4 * zz - xx - yy),
                SH_C3[5] * z * (xx - yy), SH_C3[6] * x * (xx - 3 * yy)]
    return np.stack(out, axis=1)


def camera_centres(extrinsics: np.ndarray) -> np.ndarray:
    return np.linalg.inv(extrinsics.astype(np.float64))[:, :3, 3]


def sh_colors(vertices: np.ndarray, sh: np.ndarray, extrinsics: np.ndarray, sh_degree: int) -> np.ndarray:
    """[B, V, 3] colours from sh [C, V, 3] (only the first (deg+1)^2 used)."""
    n = (sh_degree + 1) ** 2
    v = vertices.astype(np.float64)
    out = []
    for c in camera_centres(extrinsics):
        d = v - c
        d = d / np.sqrt((d * d).sum(axis=1, keepdims=True))
        basis = sh_basis(d, n)  # [V, n]
        rgb = np.einsum("vk,kvc->vc", basis, sh[:n])
        out.append(np.maximum(rgb + 0.5, 0.0))
    return np.stack(out)


def composite_hits(faces: np.ndarray, hit_faces: np.ndarray, hit_uvw: np.ndarray, colors: np.ndarray,
                   sdf: np.ndarray, sharpness: float) -> tuple[np.ndarray, np.ndarray]:
    """Front-to-back compositing of per-pixel hit lists.

    hit_faces [B, P, S] (-1 = no hit in that slot), hit_uvw [B, P, S, 3],
    colors [B, V, 3], sdf [V] -> (rgb [B, P, 3], T [B, P]).
    """
    b, p, s = hit_faces.shape
    rgb_out = np.zeros((b, p, 3))
    t_out = np.ones((b, p))
    for cam in range(b):
        acc = np.zeros((p, 3))
        trans = np.ones(p)
        outer = np.ones(p)  # 1 / (1 + exp(-1e10 s)) == 1 in float64
        for slot in range(s):
            f = hit_faces[cam, :, slot]
            valid = f >= 0
            tri = faces[np.where(valid, f, 0)]  # [P, 3]
            w = hit_uvw[cam, :, slot].astype(np.float64)  # [P, 3]
            rgb = (w[:, :, None] * colors[cam][tri]).sum(axis=1)
            d = (w * sdf[tri]).sum(axis=1)
            inner = 1.0 / (1.0 + np.exp(-d * sharpness))
            alpha = np.clip(((outer - inner) + 1e-5) / (outer + 1e-5), 0.0, 1.0)
            acc = np.where(valid[:, None], acc + rgb * (trans * alpha)[:, None], acc)
            trans = np.where(valid, trans * (1.0 - alpha), trans)
            outer = np.where(valid, inner, outer)
        rgb_out[cam], t_out[cam] = acc, trans
    return rgb_out, t_out


def central_difference(f, x: np.ndarray, index: tuple, h: float) -> float:
    """(f(x + h e_i) - f(x - h e_i)) / 2h, restoring x afterwards."""
    old = x[index]
    x[index] = old + h
    fp = f()
    x[index] = old - h
    fm = f()
    x[index] = old
    return (fp - fm) / (2 * h)


def sdf_regularizers(sdf: np.ndarray, neighbors: np.ndarray, lower: np.ndarray, upper: np.ndarray,
                     grid_size) -> tuple[np.ndarray, np.ndarray, np.ndarray]:
    """compute_sdf_regularizers.slang:18-128 in float64 (same case split)."""
    i, j, k = (float(x) for x in grid_size)
    nv = upper.shape[1]
    d000, d001, d010, d100 = (sdf[lower[r][:nv]] for r in range(4))  # voxel entries come first
    d111, d110, d101, d011 = (sdf[upper[r]] for r in range(4))
    dx = 0.25 * ((d001 - d000) + (d011 - d010) + (d101 - d100) + (d111 - d110))
    dy = 0.25 * ((d010 - d000) + (d011 - d001) + (d110 - d100) + (d111 - d101))
    dz = 0.25 * ((d100 - d000) + (d101 - d001) + (d110 - d010) + (d111 - d011))
    norm = np.sqrt((k * dx) ** 2 + (j * dy) ** 2 + (i * dz) ** 2)
    scale = np.maximum(np.maximum(np.abs(k * dx), np.abs(j * dy)), np.abs(i * dz))
    delta = np.where(scale < 1e-10, 0.0, norm) - 1.0
    pos = np.where(delta > 0, delta * delta, 0.0)
    neg = np.where(delta < 0, delta * delta, 0.0)
    sub = neighbors[6]
    cs = d110 + d101 + d011
    counted = np.full(sdf[upper[0]].shape, 3.0)
    for r in range(1, 4):
        corner = lower[r][sub]
        present = corner >= 0
        cs = cs + np.where(present, sdf[np.where(present, corner, 0)], 0.0)
        counted = counted + present
    cs = cs - counted * d111
    return pos, neg, cs * cs
