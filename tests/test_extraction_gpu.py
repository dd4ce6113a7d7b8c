"""GPU parity of the extraction path against the CPU oracle.

Topology, offsets, faces and vertex indices must be bit-exact; interpolated
vertex attributes are bit-exact too (the reference source's operations in
its order, no contraction);
gradients of the marching-cubes vertices agree within 1e-5 relative.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from meshtryoshka_gb300 import triangle_extraction as te
from oracle import oracle
from tests import semantics

pytestmark = pytest.mark.gpu


def _random_grid(rng, shape, density):
    return semantics.pack(rng.random(shape) < density)


GRIDS = {
    "single_voxel": lambda rng: semantics.pack(np.pad(np.ones((1, 1, 1), bool), ((1, 2), (2, 1), (3, 28)))),
    "random_sparse": lambda rng: _random_grid(rng, (5, 6, 64), 0.1),
    "random_dense": lambda rng: _random_grid(rng, (4, 3, 96), 0.6),
    "full": lambda rng: semantics.pack(np.ones((3, 4, 64), bool)),
    "empty": lambda rng: semantics.pack(np.zeros((3, 3, 32), bool)),
    "bit31_edges": lambda rng: semantics.pack(
        (np.arange(96)[None, None, :] % 32 >= 30) & (rng.random((4, 4, 96)) < 0.7)),
    "non_cubic": lambda rng: _random_grid(rng, (7, 3, 160), 0.3),
    "medium": lambda rng: _random_grid(rng, (40, 33, 128), 0.05),
}


def _t(a, device):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _n(t):
    return t.detach().cpu().numpy()


@pytest.mark.parametrize("name", list(GRIDS))
def test_extract_voxels_bit_exact(cuda_device, name):
    occ = GRIDS[name](np.random.default_rng(11))
    want = oracle.extract_voxels(occ)
    got = te.extract_voxels(_t(occ, cuda_device))
    assert got.grid_shape == want.grid_shape
    for field in ("vertices", "neighbors", "lower_corners", "upper_corners", "indices"):
        np.testing.assert_array_equal(_n(getattr(got, field)), getattr(want, field), err_msg=field)


def test_extract_voxels_intermediates(cuda_device):
    occ = GRIDS["random_dense"](np.random.default_rng(3))
    vocc, vcounts = te.compute_vertex_occupancy(_t(occ, cuda_device))
    want_vocc, want_vcounts = oracle.compute_vertex_occupancy(occ)
    np.testing.assert_array_equal(_n(vocc), want_vocc)
    np.testing.assert_array_equal(_n(vcounts), want_vcounts)
    np.testing.assert_array_equal(_n(te.count_occupancy(_t(occ, cuda_device))), oracle.count_occupancy(occ))


@pytest.mark.parametrize("d", [1, 2, 4, 31])
def test_dilate_bit_exact(cuda_device, d):
    occ = _random_grid(np.random.default_rng(d), (12, 10, 128), 0.005)
    got = te.dilate_occupancy(_t(occ, cuda_device), d)
    np.testing.assert_array_equal(_n(got), oracle.dilate_occupancy(occ, d))


@pytest.mark.parametrize("n", [0, 1, 5, 4095, 4096, 4097, 123457, 3_000_001])
def test_exclusive_cumsum_i32(cuda_device, n):
    rng = np.random.default_rng(n)
    x = rng.integers(0, 16, n).astype(np.int32)
    t = _t(x, cuda_device)
    te.compute_exclusive_cumsum(t)
    np.testing.assert_array_equal(_n(t), oracle.exclusive_cumsum(x))


def test_exclusive_cumsum_unaligned_view(cuda_device):
    x = np.random.default_rng(1).integers(0, 9, 100_003).astype(np.int32)
    base = _t(np.concatenate((np.array([7], np.int32), x)), cuda_device)
    view = base[1:]  # 4-byte aligned only: exercises the scalar path
    te.compute_exclusive_cumsum(view)
    np.testing.assert_array_equal(_n(view), oracle.exclusive_cumsum(x))
    assert int(base[0]) == 7


@pytest.mark.parametrize("n", [1, 511, 4097, 1_000_003])
@pytest.mark.parametrize("offset", [0, 1])
def test_scan_i64_and_widening(cuda_device, n, offset):
    """The int64 exclusive scan and the int32 -> int64 inclusive scan (keys'
    offsets), with sums past 2^31, on 16-byte aligned and unaligned views."""
    from meshtryoshka_gb300 import _native as nt

    rng = np.random.default_rng(n + 3 * offset)
    lib = nt.library()
    ws_ptr, ws_bytes = nt.workspace(cuda_device).get(lib.mt_scan_workspace_bytes(n))
    stream = nt.stream(cuda_device)
    x64 = rng.integers(0, 1 << 40, n).astype(np.int64)
    base64 = _t(np.concatenate((np.zeros(offset, np.int64), x64)), cuda_device)
    view64 = base64[offset:]
    nt.call("mt_exclusive_scan_i64", view64.data_ptr(), n, ws_ptr, ws_bytes, stream)
    np.testing.assert_array_equal(_n(view64), np.concatenate(([0], np.cumsum(x64)[:-1])))
    x32 = rng.integers(0, 1 << 30, n).astype(np.int32)
    base32 = _t(np.concatenate((np.zeros(offset, np.int32), x32)), cuda_device)
    out = torch.empty(n + offset, dtype=torch.int64, device=cuda_device)[offset:]
    nt.call("mt_inclusive_scan_i32_to_i64", base32[offset:].data_ptr(), out.data_ptr(), n, ws_ptr, ws_bytes, stream)
    np.testing.assert_array_equal(_n(out), np.cumsum(x32.astype(np.int64)))


def _sphere_scene(n, levels, sh_coeffs=4, seed=0):
    coords = -1 + (np.arange(n) + 0.5) * 2 / n
    z, y, x = np.meshgrid(coords, coords, coords, indexing="ij")
    d = np.sqrt(x * x + y * y + z * z) - 0.5
    occ = semantics.pack(np.abs(d) < 2.5 * 2 / n)
    vox = oracle.extract_voxels(occ)
    p = 2 * vox.vertices.astype(np.float64) - 1
    rng = np.random.default_rng(seed)
    sdf = (np.linalg.norm(p, axis=1) - 0.5 + rng.normal(0, 0.002, len(p))).astype(np.float32)
    sh = rng.uniform(0, 1, (sh_coeffs, len(p), 3)).astype(np.float32)
    return occ, vox, sdf, sh, np.array(levels, np.float32)


def _tessellate_both(cuda_device, vox, sdf, sh, ls):
    want = oracle.tessellate_voxels(sdf, vox.vertices, sh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                    vox.indices, ls)
    d = cuda_device
    got = te.tessellate_voxels(_t(sdf, d), _t(vox.vertices, d), _t(sh, d), _t(vox.neighbors, d),
                               _t(vox.lower_corners, d), _t(vox.upper_corners, d), _t(vox.indices, d), _t(ls, d))
    return got, want


@pytest.mark.parametrize("n,levels,c", [
    (32, (0.04, 0.0, -0.04), 1),
    (64, (0.02, 0.0, -0.02), 16),
    (64, tuple(np.linspace(0.03, -0.03, 8)), 4),
    (32, (0.0,), 9),
])
def test_tessellate_bit_exact(cuda_device, n, levels, c):
    occ, vox, sdf, sh, ls = _sphere_scene(n, levels, c)
    got, want = _tessellate_both(cuda_device, vox, sdf, sh, ls)
    for field in ("faces", "voxel_indices", "vertex_boundaries", "face_boundaries"):
        np.testing.assert_array_equal(_n(getattr(got, field)), getattr(want, field), err_msg=field)
    for field in ("vertices", "signed_distances", "spherical_harmonics"):
        np.testing.assert_array_equal(_n(getattr(got, field)), getattr(want, field), err_msg=field)


def test_tessellate_stages_bit_exact(cuda_device):
    occ, vox, sdf, sh, ls = _sphere_scene(64, (0.03, 0.01, -0.01, -0.03), 4)
    d = cuda_device
    counts = te.count_triangle_vertices(_t(sdf, d), _t(vox.lower_corners, d), _t(ls, d))
    np.testing.assert_array_equal(_n(counts), oracle.count_triangle_vertices(sdf, vox.lower_corners, ls))
    fcounts, codes = te.count_triangle_faces(_t(sdf, d), _t(vox.lower_corners, d), _t(vox.upper_corners, d),
                                             _t(ls, d))
    wc, wcodes = oracle.count_triangle_faces(sdf, vox.lower_corners, vox.upper_corners, ls)
    np.testing.assert_array_equal(_n(fcounts), wc)
    np.testing.assert_array_equal(_n(codes), wcodes)


def test_tessellate_all_256_cube_codes(cuda_device):
    """A 2x2x2-voxel block per case with random corner SDFs reproduces every
    cube code; faces must match the oracle exactly."""
    occ = np.zeros((4, 4, 32), bool)
    occ[1:3, 1:3, 1:3] = True
    vox = oracle.extract_voxels(semantics.pack(occ))
    rng = np.random.default_rng(5)
    seen = set()
    for trial in range(64):
        sdf = rng.normal(0, 1, vox.vertices.shape[0]).astype(np.float32)
        sh = rng.uniform(0, 1, (1, len(sdf), 3)).astype(np.float32)
        ls = np.array([0.3, 0.0, -0.3], np.float32)
        got, want = _tessellate_both(cuda_device, vox, sdf, sh, ls)
        np.testing.assert_array_equal(_n(got.faces), want.faces)
        np.testing.assert_array_equal(_n(got.vertices), want.vertices)
        seen.update(np.unique(want.cell_codes).tolist())
    assert len(seen) > 200


def test_tessellate_empty_level_set_and_empty_voxels(cuda_device):
    occ, vox, sdf, sh, ls = _sphere_scene(32, (5.0, 0.0, -5.0), 1)
    got, want = _tessellate_both(cuda_device, vox, sdf, sh, ls)
    np.testing.assert_array_equal(_n(got.face_boundaries), want.face_boundaries)
    assert int(got.face_boundaries[0]) == 0


@pytest.mark.parametrize("c", [1, 16])
def test_create_triangle_vertices_backward(cuda_device, c):
    occ, vox, sdf, sh, ls = _sphere_scene(64, (0.02, 0.0, -0.02), c, seed=3)
    d = cuda_device
    sdf_t = _t(sdf, d).requires_grad_(True)
    sh_t = _t(sh, d).requires_grad_(True)
    v_t = _t(vox.vertices, d).requires_grad_(True)
    tri = te.tessellate_voxels(sdf_t, v_t, sh_t, _t(vox.neighbors, d), _t(vox.lower_corners, d),
                               _t(vox.upper_corners, d), _t(vox.indices, d), _t(ls, d))
    rng = np.random.default_rng(9)
    gv = rng.normal(0, 1, tri.vertices.shape).astype(np.float32)
    gd = rng.normal(0, 1, tri.signed_distances.shape).astype(np.float32)
    gs = rng.normal(0, 1, tri.spherical_harmonics.shape).astype(np.float32)
    torch.autograd.backward([tri.vertices, tri.signed_distances, tri.spherical_harmonics],
                            [_t(gv, d), _t(gd, d), _t(gs, d)])
    want = oracle.tessellate_voxels(sdf, vox.vertices, sh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                    vox.indices, ls)
    wv, wd, ws = oracle.create_triangle_vertices_backward(sdf, sh.shape, vox.lower_corners, ls,
                                                          want.vertex_offsets, gv, gd, gs)
    for got, ref in ((v_t.grad, wv), (sdf_t.grad, wd), (sh_t.grad, ws)):
        np.testing.assert_allclose(_n(got), ref, rtol=1e-5, atol=1e-5 * max(1.0, np.abs(ref).max()))
