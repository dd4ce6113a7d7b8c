"""Subdivision ops on the GPU: write / upscale occupancy, parameter
upscaling, the occupancy mesh and vertex de-duplication.

* Golden parity: every op reproduces the reference's kernel outputs
  (tests/golden/subdivision.npz) bit for bit, and index_vertices /
  index_keys the reference's Python with the stable sort torch uses on CUDA.
* Oracle parity on seeded grids larger than the fixtures, with masks,
  non-power-of-two extents and every SH size.
* Edge cases the reference meets: empty inputs, indices outside the grid,
  an all-zero mask (no vertices), full grids, a single run of equal keys.
* Size-independent properties at 512^3: a factor-2 upscale is the
  nearest-parent copy, a linear field survives parameter upscaling on a
  full grid, and de-duplication maps every key to the first equal key.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from meshtryoshka_gb300 import triangle_extraction as te
from oracle import oracle
from tests import goldens, semantics

pytestmark = pytest.mark.gpu


def _t(a, device):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _case(g, case):
    return {k.split("/", 1)[1]: v for k, v in g.items() if k.startswith(case + "/")}


@pytest.fixture(scope="module")
def golden():
    return goldens.load("subdivision")


@pytest.mark.parametrize("case", goldens.SUBDIVISION_CASES)
def test_subdivision_matches_reference(golden, case, cuda_device):
    g = _case(golden, case)
    d = cuda_device
    resolution = tuple(int(x) for x in g["resolution"])
    occ = _t(g["occupancy"], d)
    np.testing.assert_array_equal(te.upscale_occupancy(occ, resolution).cpu().numpy(), g["upscaled_occupancy"])
    up = te.upscale_parameters(_t(g["signed_distances"], d), _t(g["spherical_harmonics"], d), occ, _t(g["mask"], d),
                               resolution)
    assert isinstance(up, te.UpscaledParameters)
    np.testing.assert_array_equal(up.occupancy.cpu().numpy(), g["new_occupancy"])
    np.testing.assert_array_equal(up.signed_distances.cpu().numpy(), g["new_signed_distances"])
    np.testing.assert_array_equal(up.spherical_harmonics.cpu().numpy(), g["new_spherical_harmonics"])
    mesh = te.get_occupancy_mesh(occ, _t(g["mesh_colors_in"], d))
    assert isinstance(mesh, te.Mesh)
    np.testing.assert_array_equal(mesh.vertices.cpu().numpy(), g["mesh_vertices"])
    np.testing.assert_array_equal(mesh.colors.cpu().numpy(), g["mesh_colors"])
    written = te.write_occupancy(_t(g["voxel_indices"], d), tuple(g["occupancy"].shape), 0, 1)
    np.testing.assert_array_equal(written.cpu().numpy(), g["written"])


@pytest.mark.parametrize("tol", goldens.INDEX_TOLERANCES)
def test_index_vertices_matches_reference(golden, tol, cuda_device):
    key = f"index_{tol:g}"
    got = te.index_vertices(_t(golden[f"{key}/points"], cuda_device), tol)
    assert got.dtype == torch.int32
    np.testing.assert_array_equal(got.cpu().numpy(), golden[f"{key}/index"])


def test_index_keys_matches_reference(golden, cuda_device):
    got = te.index_keys(_t(golden["index_keys/keys"], cuda_device))
    np.testing.assert_array_equal(got.cpu().numpy(), golden["index_keys/index"])


# ---------------------------------------------------------------------------
# Oracle parity at larger sizes
# ---------------------------------------------------------------------------
UPSCALES = [
    ((16, 24, 64), (32, 48, 128)),
    ((20, 12, 96), (33, 29, 160)),
    ((8, 8, 32), (8, 8, 32)),
    ((7, 9, 64), (50, 41, 352)),
]


@pytest.mark.parametrize("shape,target", UPSCALES)
def test_upscale_occupancy_matches_oracle(shape, target, cuda_device):
    rng = np.random.default_rng(sum(shape))
    occ = semantics.pack(rng.random(shape) < 0.2)
    mask = semantics.pack(rng.random(shape) < 0.5)
    want = oracle.upscale_occupancy(occ, target)
    got = te.upscale_occupancy(_t(occ, cuda_device), target).cpu().numpy()
    np.testing.assert_array_equal(got, want)
    # The masked form used by upscale_parameters.
    want_masked = oracle.upscale_occupancy(occ, target, mask=mask)
    np.testing.assert_array_equal(want_masked, oracle.upscale_occupancy(occ & mask, target))
    got_masked = te._upscale_occupancy(_t(occ, cuda_device), _t(mask, cuda_device), target).cpu().numpy()
    np.testing.assert_array_equal(got_masked, want_masked)


def _sphere_band(n, radius=0.6, width=3.0):
    c = -1 + (np.arange(n) + 0.5) * 2 / n
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    d = np.sqrt(x * x + y * y + z * z) - radius
    return semantics.pack(np.abs(d) < width * 2 / n)


@pytest.mark.parametrize("c", [1, 4, 9, 16])
def test_upscale_parameters_matches_oracle(c, cuda_device):
    d = cuda_device
    rng = np.random.default_rng(c)
    occ = _sphere_band(64)
    mask = semantics.pack(rng.random((64, 64, 64)) < 0.8)
    vox = te.extract_voxels(_t(occ, d))
    v = vox.num_vertices
    sdf = rng.normal(0, 0.1, v).astype(np.float32)
    sh = rng.normal(0, 1, (c, v, 3)).astype(np.float32)
    target = (128, 96, 160)
    want = oracle.upscale_parameters(sdf, sh, occ, mask, target)
    got = te.upscale_parameters(_t(sdf, d), _t(sh, d), _t(occ, d), _t(mask, d), target)
    np.testing.assert_array_equal(got.occupancy.cpu().numpy(), want[2])
    np.testing.assert_array_equal(got.signed_distances.cpu().numpy(), want[0])
    np.testing.assert_array_equal(got.spherical_harmonics.cpu().numpy(), want[1])


@pytest.mark.parametrize("n", [32, 96])
def test_occupancy_mesh_matches_oracle(n, cuda_device):
    occ = _sphere_band(n)
    colors = np.random.default_rng(n).uniform(0, 1, (3, 2, 3)).astype(np.float32)
    want = oracle.get_occupancy_mesh(occ, colors)
    got = te.get_occupancy_mesh(_t(occ, cuda_device), _t(colors, cuda_device))
    np.testing.assert_array_equal(got.vertices.cpu().numpy(), want[0])
    np.testing.assert_array_equal(got.colors.cpu().numpy(), want[1])


def test_index_vertices_of_voxel_vertices(cuda_device):
    """The tesseract's use: voxel vertices (with duplicates from two copies of
    the grid) de-duplicated at 1e-6."""
    d = cuda_device
    vox = te.extract_voxels(_t(_sphere_band(64), d))
    pts = vox.vertices.cpu().numpy()
    perm = np.random.default_rng(0).permutation(2 * len(pts))
    both = np.concatenate([pts, pts])[perm]
    want = oracle.index_vertices(both, 1e-6)
    got = te.index_vertices(_t(both, d), 1e-6).cpu().numpy()
    np.testing.assert_array_equal(got, want)
    assert len(np.unique(got)) == len(pts)


# ---------------------------------------------------------------------------
# Edge cases
# ---------------------------------------------------------------------------
def test_write_occupancy_edges(cuda_device):
    d = cuda_device
    shape = (3, 4, 2)
    empty = te.write_occupancy(torch.empty(0, dtype=torch.int32, device=d), shape, 0, 1)
    assert empty.shape == shape and int(empty.abs().sum()) == 0
    words = 3 * 4 * 2
    idx = np.array([-5, 0, 31, 32, 32 * words - 1, 32 * words, 10**9, 77, 77], np.int32)
    got = te.write_occupancy(_t(idx, d), shape, 0, 1).cpu().numpy()
    np.testing.assert_array_equal(got, oracle.write_occupancy(idx, shape))
    assert got.reshape(-1)[0] == np.int32(-2147483647)  # bits 0 and 31 of word 0


def test_upscale_parameters_with_empty_mask(cuda_device):
    d = cuda_device
    occ = _sphere_band(32)
    vox = te.extract_voxels(_t(occ, d))
    sdf = torch.zeros(vox.num_vertices, device=d)
    sh = torch.zeros((4, vox.num_vertices, 3), device=d)
    up = te.upscale_parameters(sdf, sh, _t(occ, d), torch.zeros_like(_t(occ, d)), (64, 64, 64))
    assert up.signed_distances.shape == (0,) and up.spherical_harmonics.shape == (4, 0, 3)
    assert int(up.occupancy.abs().sum()) == 0


def test_occupancy_mesh_edges(cuda_device):
    d = cuda_device
    colors = torch.rand((3, 2, 3), device=d)
    zero = te.get_occupancy_mesh(torch.zeros((4, 5, 2), dtype=torch.int32, device=d), colors)
    assert zero.vertices.shape == (0, 3, 3) and zero.colors.shape == (0, 3)
    full = np.full((4, 5, 2), -1, np.int32)
    want = oracle.get_occupancy_mesh(full, colors.cpu().numpy())
    got = te.get_occupancy_mesh(_t(full, d), colors)
    assert got.vertices.shape[0] == 2 * 2 * (4 * 5 + 5 * 64 + 4 * 64)  # the six outer faces
    np.testing.assert_array_equal(got.vertices.cpu().numpy(), want[0])
    np.testing.assert_array_equal(got.colors.cpu().numpy(), want[1])


def test_index_vertices_edges(cuda_device):
    d = cuda_device
    same = torch.full((100_000, 3), 0.25, device=d)
    out = te.index_vertices(same, 1e-6)
    assert int(out.max()) == 0 and int(out.min()) == 0
    with pytest.raises(RuntimeError, match="bits"):
        te.index_vertices(torch.tensor([[1e4, 0.0, 0.0]], device=d), 1e-6)
    with pytest.raises(RuntimeError):
        te.index_vertices(torch.empty((0, 3), device=d))
    assert te.index_keys(torch.empty(0, dtype=torch.int64, device=d)).shape == (0,)


def test_index_vertices_reciprocal_rounding(cuda_device):
    """round(points / tol) as torch computes it on CUDA: the product with the
    float32 reciprocal of tol. A point where that product and the exact
    quotient round to different integers follows the product."""
    tol = 1e-5
    inv = np.float32(1.0) / np.float32(tol)
    rng = np.random.default_rng(5)
    pts = rng.random((200_000, 3)).astype(np.float32)
    differs = np.rint(pts / np.float32(tol)) != np.rint(pts * inv)
    assert differs.any()
    got = te.index_vertices(_t(pts, cuda_device), tol).cpu().numpy()
    np.testing.assert_array_equal(got, oracle.index_vertices(pts, tol))


# ---------------------------------------------------------------------------
# Properties at full size
# ---------------------------------------------------------------------------
def test_factor_two_upscale_is_parent_copy_512(cuda_device):
    d = cuda_device
    g = torch.Generator(device=d)
    g.manual_seed(0)
    bits = torch.rand((256, 256, 256), generator=g, device=d) < 0.1
    occ = te.pack_occupancy(bits)
    up = te.upscale_occupancy(occ, (512, 512, 512))
    want = bits.repeat_interleave(2, 0).repeat_interleave(2, 1).repeat_interleave(2, 2)
    assert torch.equal(te.unpack_occupancy(up), want)


def test_linear_field_survives_upscaling(cuda_device):
    """On a full grid every trilinear sample has all of its weight on
    existing corners, so a linear field is reproduced up to float rounding."""
    d = cuda_device
    occ = torch.full((64, 64, 2), -1, dtype=torch.int32, device=d)
    vox = te.extract_voxels(occ)
    coef = torch.tensor([0.3, -0.7, 0.45], device=d)
    sdf = (vox.vertices * coef).sum(dim=1)
    sh = torch.stack([vox.vertices, 1 - vox.vertices])  # [2, V, 3], linear per channel
    up = te.upscale_parameters(sdf, sh, occ, torch.full_like(occ, -1), (128, 128, 128))
    new_vox = te.extract_voxels(up.occupancy)
    assert up.signed_distances.shape[0] == new_vox.num_vertices == 129**3
    want = (new_vox.vertices * coef).sum(dim=1)
    assert float((up.signed_distances - want).abs().max()) < 5e-6
    assert float((up.spherical_harmonics[0] - new_vox.vertices).abs().max()) < 5e-6
    assert float((up.spherical_harmonics[1] - (1 - new_vox.vertices)).abs().max()) < 5e-6


def test_index_keys_first_seen_at_scale(cuda_device):
    d = cuda_device
    g = torch.Generator(device=d)
    g.manual_seed(1)
    n = 8_000_000
    keys = torch.randint(-(2**40), 2**40, (n // 4,), generator=g, device=d)
    keys = keys[torch.randint(0, n // 4, (n,), generator=g, device=d)]
    out = te.index_keys(keys).long()
    assert torch.equal(keys[out], keys)
    _, inverse = torch.unique(keys, return_inverse=True)
    first = torch.full((int(inverse.max()) + 1,), n, dtype=torch.int64, device=d)
    first.scatter_reduce_(0, inverse, torch.arange(n, device=d), reduce="amin")
    assert torch.equal(out, first[inverse])


def test_subdivide_matches_oracle(cuda_device):
    """The whole subdivision step (canonical copy, triangle mask, dilation,
    upscaling) of a tessellated scene, against the oracle's sequence."""
    from meshtryoshka_gb300 import subdivision, synthetic

    d = cuda_device
    cfg = synthetic.CONFIGS["small"]
    occ = synthetic.make_occupancy(cfg, d)
    vox = te.extract_voxels(occ)
    sdf = synthetic.corner_sdf(cfg, vox.vertices)
    sh = torch.randn((16, vox.num_vertices, 3), device=d)
    with torch.no_grad():
        tri = te.tessellate_voxels(sdf, vox.vertices, sh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                   vox.indices, synthetic.level_sets(cfg, d))
    got = subdivision.subdivide(vox, sdf, sh, occ, tri.voxel_indices, (128, 96, 160))
    want = oracle.subdivide(vox.vertices.cpu().numpy(), sdf.cpu().numpy(), sh.cpu().numpy(), occ.cpu().numpy(),
                            tri.voxel_indices.cpu().numpy(), (128, 96, 160))
    assert got.signed_distances.numel() > 0
    np.testing.assert_array_equal(got.occupancy.cpu().numpy(), want[2])
    np.testing.assert_array_equal(got.signed_distances.cpu().numpy(), want[0])
    np.testing.assert_array_equal(got.spherical_harmonics.cpu().numpy(), want[1])
