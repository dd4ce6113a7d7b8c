"""First-principles definitions used to pin the oracle.

The reference ships no tests, golden files or fixtures, and its kernels need
slangtorch, which is absent, so its outputs cannot be produced here. These
numpy definitions state what each reference output *means* (derived from the
reference kernels' comments and data flow) without following their loops; the
oracle, which does follow the loops, must agree with them bit for bit.
"""

from __future__ import annotations

import numpy as np


def unpack(occ_packed: np.ndarray) -> np.ndarray:
    i, j, kp = occ_packed.shape
    bits = (occ_packed.astype(np.int64)[..., None] >> np.arange(32)) & 1
    return bits.reshape(i, j, kp * 32).astype(bool)


def pack(occ: np.ndarray) -> np.ndarray:
    i, j, k = occ.shape
    bits = occ.reshape(i, j, k // 32, 32).astype(np.int64) << np.arange(32)
    return bits.sum(-1).astype(np.uint32).view(np.int32)


def voxels(occ_packed: np.ndarray):
    """Sparse topology of a packed grid, as extract_voxels defines it:

    * grid vertices: lattice points that are a corner of an occupied voxel,
      numbered in row-major (i, j, k) order over a (I+1, J+1, 32*(KP+1))
      lattice; position (k / K, j / J, i / I) in float32;
    * entries (voxels then subvoxels): occupied voxels in row-major order,
      then grid vertices that are not occupied voxels, in row-major order;
    * lower_corners[c, entry]: vertex ids of the entry's point and its +x, +y,
      +z neighbours, -64 where that neighbour is not a grid vertex;
    * upper_corners[c, voxel]: vertex ids of +xyz, +yz, +xz, +xy;
    * neighbors[n, voxel]: entry ids of +x, +y, +z, +xy, +yz, +xz, +xyz;
    * indices[voxel]: K * (J * i + j) + k.
    """
    occ = unpack(occ_packed)
    I, J, K = occ.shape
    KL = K + 32
    lat = np.zeros((I + 1, J + 1, KL), bool)
    for di in (0, 1):
        for dj in (0, 1):
            for dk in (0, 1):
                lat[di:di + I, dj:dj + J, dk:dk + K] |= occ
    occ_l = np.zeros_like(lat)
    occ_l[:I, :J, :K] = occ
    vid = np.full(lat.shape, -64, np.int64)
    vid[lat] = np.arange(lat.sum())
    nv = int(occ.sum())
    sub = lat & ~occ_l
    gid = np.full(lat.shape, -1, np.int64)
    gid[occ_l] = np.arange(nv)
    gid[sub] = nv + np.arange(sub.sum())
    G = int(lat.sum())

    pts = np.argwhere(lat)  # row-major
    inv = (np.float32(1) / np.float32(I), np.float32(1) / np.float32(J), np.float32(1) / np.float32(K))
    vertices = np.stack(
        (pts[:, 2].astype(np.float32) * inv[2], pts[:, 1].astype(np.float32) * inv[1],
         pts[:, 0].astype(np.float32) * inv[0]), axis=1).astype(np.float32)

    def at(arr, p, d, fill):
        q = p + np.array(d)
        ok = (q[:, 0] <= I) & (q[:, 1] <= J) & (q[:, 2] < KL)
        out = np.full(len(p), fill, np.int64)
        out[ok] = arr[q[ok, 0], q[ok, 1], q[ok, 2]]
        return out

    entries = np.concatenate((np.argwhere(occ_l), np.argwhere(sub)))
    lower = np.empty((4, G), np.int64)
    lower[0] = vid[entries[:, 0], entries[:, 1], entries[:, 2]]
    for c, d in enumerate(((0, 0, 1), (0, 1, 0), (1, 0, 0)), start=1):
        lower[c] = at(vid, entries, d, -64)

    vox = np.argwhere(occ_l)
    upper = np.empty((4, nv), np.int64)
    for c, d in enumerate(((1, 1, 1), (1, 1, 0), (1, 0, 1), (0, 1, 1))):
        upper[c] = at(vid, vox, d, -64)
    neighbors = np.empty((7, nv), np.int64)
    for n, d in enumerate(((0, 0, 1), (0, 1, 0), (1, 0, 0), (0, 1, 1), (1, 1, 0), (1, 0, 1), (1, 1, 1))):
        neighbors[n] = at(gid, vox, d, -1)
    indices = K * (J * vox[:, 0] + vox[:, 1]) + vox[:, 2]
    return (vertices, neighbors.astype(np.int32), lower.astype(np.int32), upper.astype(np.int32),
            indices.astype(np.int32))


def dilate(occ_packed: np.ndarray, d: int) -> np.ndarray:
    """Cube (Chebyshev) dilation by d voxels, clipped to the grid."""
    occ = unpack(occ_packed)
    I, J, K = occ.shape
    out = np.zeros_like(occ)
    for di in range(-d, d + 1):
        for dj in range(-d, d + 1):
            for dk in range(-d, d + 1):
                src = occ[max(0, -di):I - max(0, di), max(0, -dj):J - max(0, dj), max(0, -dk):K - max(0, dk)]
                out[max(0, di):I - max(0, -di), max(0, dj):J - max(0, -dj), max(0, dk):K - max(0, -dk)] |= src
    return pack(out)
