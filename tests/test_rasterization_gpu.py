"""GPU parity of the rasterization path against the CPU oracle.

Bit-exact: projected positions and depths, tile bounds, keys, sorted keys,
tile ranges, explicit-mode hits (uv, face index). Within 1e-5 max-abs:
colours and images. Within 1e-4 (relative to the largest magnitude):
gradients, in both gradient-routing modes.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from meshtryoshka_gb300 import _native as nt
from meshtryoshka_gb300 import triangle_rasterization as tr
from oracle import oracle
from tests.scenes import SCENES, make_scene

pytestmark = pytest.mark.gpu

IMAGE_ATOL = 1e-5
GRAD_RTOL = 1e-4


def _t(a, device):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _n(t):
    return t.detach().cpu().numpy()


def _close_grad(got, want, rtol=GRAD_RTOL):
    scale = max(float(np.abs(want).max()), 1e-12)
    err = float(np.abs(got - want).max())
    assert err <= rtol * scale, f"max abs err {err:.3e} > {rtol:g} x {scale:.3e}"


# ---------------------------------------------------------------------------
# Sort
# ---------------------------------------------------------------------------
def _sort_both(keys, vals, device):
    want_k, want_v = oracle.sort_pairs(keys, vals)
    got = tr.sort_keys(tr.PairedKeys(_t(keys, device), _t(vals, device)))
    return (_n(got.keys), _n(got.triangle_indices)), (want_k, want_v)


@pytest.mark.parametrize("n", [0, 1, 2, 3071, 3072, 3073, 100_000, 1_000_003])
def test_sort_random_full_width(cuda_device, n):
    rng = np.random.default_rng(n)
    keys = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, n, dtype=np.int64)
    vals = np.arange(n, dtype=np.int32)
    got, want = _sort_both(keys, vals, cuda_device)
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[1], want[1])


def test_sort_stability_and_skipped_passes(cuda_device):
    # Few distinct keys (heavy ties, most digit passes constant), negative keys
    # from camera indices >= 32 in the top bits.
    rng = np.random.default_rng(0)
    n = 250_000
    cams = rng.integers(0, 64, n).astype(np.int64)
    tiles = rng.integers(0, 50, n).astype(np.int64)
    keys = (cams << 58) | (tiles << 38) | (np.int64(0x3F800000) << 6)
    vals = np.arange(n, dtype=np.int32)
    got, want = _sort_both(keys, vals, cuda_device)
    np.testing.assert_array_equal(got[0], want[0])
    np.testing.assert_array_equal(got[1], want[1])
    ts = torch.sort(_t(keys, cuda_device), stable=True)
    np.testing.assert_array_equal(_n(ts.indices).astype(np.int32), want[1])


def test_sort_all_equal(cuda_device):
    keys = np.full(10_000, -5, np.int64)
    vals = np.arange(10_000, dtype=np.int32)[::-1].copy()
    got, want = _sort_both(keys, vals, cuda_device)
    np.testing.assert_array_equal(got[1], want[1])


# ---------------------------------------------------------------------------
# Front end, stage by stage
# ---------------------------------------------------------------------------
def _front(scene, device, tile=(16, 16)):
    h, w = scene.image_shape
    b = scene.extrinsics.shape[0]
    s = scene.face_boundaries.shape[0]
    grid = tr.TileGrid(tile, (h, w), b, s)
    kd = tr.create_key_defines(("camera", 6), ("tile", 20), ("depth", 32), ("shell", 6))
    xy, depth = tr.project_vertices(_t(scene.vertices, device), _t(scene.extrinsics, device),
                                    _t(scene.intrinsics, device))
    bounds = tr.bound_triangles(xy, depth, _t(scene.faces, device), grid, 0.2)
    paired = tr.generate_keys(depth, _t(scene.faces, device), _t(scene.face_boundaries, device), bounds.tile_minima,
                              bounds.tile_maxima, bounds.num_tiles_overlapped, grid, kd)
    sorted_ = tr.sort_keys(paired, grid)
    tb = tr.delineate_tiles(sorted_, grid, kd, False)
    return grid, kd, xy, depth, bounds, paired, sorted_, tb


@pytest.mark.parametrize("name", list(SCENES))
def test_front_end_bit_exact(cuda_device, name):
    scene = make_scene(**SCENES[name])
    grid, kd, xy, depth, bounds, paired, sorted_, tb = _front(scene, cuda_device)
    want = oracle.render_fused(scene.extrinsics, scene.intrinsics, scene.image_shape, scene.vertices, scene.faces,
                               scene.face_boundaries, scene.sdf, scene.sh, scene.sh_degree, scene.sharpness,
                               scene.background)
    assert oracle.key_layout(kd).tolist() == oracle.key_layout(oracle.fused_key_defines()).tolist()
    np.testing.assert_array_equal(_n(xy), want.xy)
    np.testing.assert_array_equal(_n(depth), want.depth)
    np.testing.assert_array_equal(_n(bounds.tile_minima), want.tile_min)
    np.testing.assert_array_equal(_n(bounds.tile_maxima), want.tile_max)
    np.testing.assert_array_equal(_n(bounds.num_tiles_overlapped), want.counts)
    np.testing.assert_array_equal(_n(paired.keys), want.keys)
    np.testing.assert_array_equal(_n(paired.triangle_indices), want.tri)
    np.testing.assert_array_equal(_n(sorted_.keys), want.sorted_keys)
    np.testing.assert_array_equal(_n(sorted_.triangle_indices), want.sorted_tri)
    np.testing.assert_array_equal(_n(tb), want.tile_boundaries)
    assert want.keys.size > 0


@pytest.mark.parametrize("degree", [0, 1, 2, 3])
def test_spherical_harmonics(cuda_device, degree):
    scene = make_scene(**dict(SCENES["three_cams_odd"], sh_degree=3))
    d = cuda_device
    sh = _t(scene.sh, d).requires_grad_(True)
    colors = tr.evaluate_spherical_harmonics(_t(scene.vertices, d), sh, _t(scene.extrinsics, d), degree)
    want = oracle.evaluate_spherical_harmonics(scene.vertices, scene.sh, scene.extrinsics, degree)
    np.testing.assert_allclose(_n(colors), want, atol=2e-6, rtol=0)
    g = np.random.default_rng(degree).normal(0, 1, want.shape).astype(np.float32)
    colors.backward(_t(g, d))
    want_g = oracle.evaluate_spherical_harmonics_backward(scene.vertices, scene.sh.shape, scene.extrinsics, degree,
                                                          want, g)
    _close_grad(_n(sh.grad), want_g)


def test_camera_positions_match_torch_inverse(cuda_device):
    scene = make_scene(**SCENES["three_cams_odd"])
    got = tr._camera_positions(_t(scene.extrinsics, cuda_device))
    want = torch.inverse(_t(scene.extrinsics, cuda_device))[:, :3, 3]
    torch.testing.assert_close(got, want, atol=1e-6, rtol=1e-6)


# ---------------------------------------------------------------------------
# Fused compositing
# ---------------------------------------------------------------------------
def _fused_inputs(scene, device):
    d = device
    return dict(
        extrinsics=_t(scene.extrinsics, d), intrinsics=_t(scene.intrinsics, d), image_shape=scene.image_shape,
        vertices=_t(scene.vertices, d), faces=_t(scene.faces, d), shell_face_boundaries=_t(scene.face_boundaries, d),
        signed_distances=_t(scene.sdf, d).requires_grad_(True), spherical_harmonics=_t(scene.sh, d).requires_grad_(True),
        sh_degree=scene.sh_degree, sharpness=torch.tensor(scene.sharpness, device=d).requires_grad_(True),
        background=_t(scene.background, d),
    )


@pytest.mark.parametrize("name", list(SCENES))
def test_fused_forward(cuda_device, name):
    scene = make_scene(**SCENES[name])
    inputs = _fused_inputs(scene, cuda_device)
    image = tr.render(**inputs, mode="fused")
    want = oracle.render_fused(scene.extrinsics, scene.intrinsics, scene.image_shape, scene.vertices, scene.faces,
                               scene.face_boundaries, scene.sdf, scene.sh, scene.sh_degree, scene.sharpness,
                               scene.background)
    np.testing.assert_allclose(_n(image), want.image, atol=IMAGE_ATOL, rtol=0)
    # The image is not trivially the background: some pixels see the mesh.
    assert (want.raw[:, 3] < 0.5).mean() > 0.01


@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("mode", ["reference", "exact"])
def test_fused_backward(cuda_device, name, mode):
    _check_fused_backward(make_scene(**SCENES[name]), cuda_device, mode, (16, 16))


@pytest.mark.parametrize("tile", [(8, 8), (32, 32), (16, 8), (12, 20), (4, 8)])
def test_fused_backward_tile_shapes(cuda_device, tile):
    """8x4-block tiles use per-triangle coverage; other shapes per-pixel tests."""
    _check_fused_backward(make_scene(**SCENES["three_cams_odd"]), cuda_device, "reference", tile)


def _check_fused_backward(scene, d, mode, tile):
    grid, kd, xy, depth, bounds, paired, sorted_, tb = _front(scene, d, tile)
    colors_np = oracle.evaluate_spherical_harmonics(scene.vertices, scene.sh, scene.extrinsics, scene.sh_degree)
    colors = _t(colors_np, d).requires_grad_(True)
    sdf = _t(scene.sdf, d).requires_grad_(True)
    sharp = torch.tensor(scene.sharpness, device=d).requires_grad_(True)
    b, s = grid.num_cameras, grid.num_shells
    t = grid.num_tiles_per_image
    out = tr.intersect_and_composite(xy, colors, sdf, _t(scene.faces, d), sharp, sorted_.keys,
                                     sorted_.triangle_indices, tb.view(b, t, 2), s, grid, kd, gradient_mode=mode)
    want_out = oracle.intersect_and_composite(_n(xy), colors_np, scene.sdf, scene.faces, scene.sharpness,
                                              _n(sorted_.keys), _n(sorted_.triangle_indices), _n(tb).reshape(b, t, 2),
                                              s, grid.tile_shape, grid.image_shape, kd)
    np.testing.assert_allclose(_n(out), want_out, atol=IMAGE_ATOL, rtol=0)
    g = np.random.default_rng(1).normal(0, 1, want_out.shape).astype(np.float32)
    out.backward(_t(g, d))
    wc, ws, wsharp = oracle.intersect_and_composite_backward(
        _n(xy), colors_np, scene.sdf, scene.faces, scene.sharpness, _n(sorted_.keys), _n(sorted_.triangle_indices),
        _n(tb).reshape(b, t, 2), s, grid.tile_shape, grid.image_shape, kd, want_out, g, exact=(mode == "exact"))
    _close_grad(_n(colors.grad), wc)
    _close_grad(_n(sdf.grad), ws)
    assert abs(float(sharp.grad) - wsharp) <= GRAD_RTOL * max(abs(wsharp), 1e-6) + 1e-6


def test_reference_and_exact_routing_differ_only_with_multiple_hits(cuda_device):
    one_shell = make_scene(levels=(0.0,))
    d = cuda_device
    grads = {}
    for mode in ("reference", "exact"):
        inputs = _fused_inputs(one_shell, d)
        img = tr.render(**inputs, mode="fused", gradient_mode=mode)
        img.sum().backward()
        grads[mode] = _n(inputs["signed_distances"].grad)
    # Equal up to the order of floating-point atomic accumulation.
    _close_grad(grads["reference"], grads["exact"], rtol=1e-6)


@pytest.mark.parametrize("tile", [(8, 8), (16, 16), (32, 32), (16, 8), (12, 20), (4, 8)])
def test_fused_tile_shapes(cuda_device, tile):
    scene = make_scene(**SCENES["three_cams_odd"])
    inputs = _fused_inputs(scene, cuda_device)
    image = tr.render(**inputs, tile_shape=tile, mode="fused")
    want = oracle.render_fused(scene.extrinsics, scene.intrinsics, scene.image_shape, scene.vertices, scene.faces,
                               scene.face_boundaries, scene.sdf, scene.sh, scene.sh_degree, scene.sharpness,
                               scene.background, tile_shape=tile)
    np.testing.assert_allclose(_n(image), want.image, atol=IMAGE_ATOL, rtol=0)


def test_fused_empty_scene_returns_background(cuda_device):
    scene = make_scene()
    inputs = _fused_inputs(scene, cuda_device)
    inputs["faces"] = inputs["faces"][:0]
    image = tr.render(**inputs)
    expect = np.broadcast_to(scene.background[None, :, None, None], (1, 3, *scene.image_shape))
    np.testing.assert_array_equal(_n(image), expect)


def test_ssaa_matches_mean_of_supersampled(cuda_device):
    scene = make_scene(image_shape=(64, 64))
    inputs = _fused_inputs(scene, cuda_device)
    image = tr.render(**inputs, ssaa=2)
    assert image.shape == (1, 3, 64, 64)
    sup = dict(inputs)
    sup["image_shape"] = (128, 128)
    sup["intrinsics"] = inputs["intrinsics"] * torch.tensor((2, 2, 1), device=cuda_device)[:, None]
    raw = tr.render(**sup)
    # Clip happens after the mean in the reference; the raw image is clipped
    # per sample, so compare in the interior where nothing saturates.
    assert float((image - raw.reshape(1, 3, 64, 2, 64, 2).mean((3, 5))).abs().max()) < 0.05


# ---------------------------------------------------------------------------
# Explicit mode
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", list(SCENES))
def test_explicit_rasterize_bit_exact(cuda_device, name):
    scene = make_scene(**SCENES[name])
    d = cuda_device
    uv, index = tr.rasterize(_t(scene.vertices, d), _t(scene.faces, d), _t(scene.face_boundaries, d),
                             _t(scene.extrinsics, d), _t(scene.intrinsics, d), scene.image_shape)
    h, w = scene.image_shape
    b = scene.extrinsics.shape[0]
    s = scene.face_boundaries.shape[0]
    rows, cols = -(-h // 16), -(-w // 16)
    kd = oracle.explicit_key_defines()
    xy, depth = oracle.project_vertices(scene.vertices, scene.extrinsics, scene.intrinsics)
    tmin, tmax, count = oracle.bound_triangles(xy, depth, scene.faces, (16, 16), (rows, cols), 0.2)
    keys, tri = oracle.generate_keys(depth, scene.faces, scene.face_boundaries, tmin, tmax, count, cols, kd)
    sk, st = oracle.sort_pairs(keys, tri)
    tb = oracle.delineate_tiles(sk, kd, True, b, s, rows * cols)
    want_uv, want_index = oracle.intersect(xy, scene.faces, st, tb, s, (16, 16), scene.image_shape)
    np.testing.assert_array_equal(_n(index), want_index)
    np.testing.assert_array_equal(_n(uv), want_uv)
    assert (want_index >= 0).any()


@pytest.mark.parametrize("name", list(SCENES))
@pytest.mark.parametrize("mode", ["reference", "exact"])
def test_explicit_render_and_gradients(cuda_device, name, mode):
    scene = make_scene(**SCENES[name])
    d = cuda_device
    inputs = _fused_inputs(scene, d)
    image = tr.render(**inputs, mode="explicit", gradient_mode=mode)
    # Oracle chain: rasterize -> SH -> interpolate -> composite -> background.
    uv, index = tr.rasterize(inputs["vertices"], inputs["faces"], inputs["shell_face_boundaries"],
                             inputs["extrinsics"], inputs["intrinsics"], scene.image_shape)
    uv, index = _n(uv), _n(index)
    colors = oracle.evaluate_spherical_harmonics(scene.vertices, scene.sh, scene.extrinsics, scene.sh_degree)
    isdf, icol = oracle.interpolate(uv, index, scene.faces, scene.sdf, colors)
    b, s, h, w = isdf.shape
    psdf = isdf.transpose(0, 2, 3, 1).reshape(-1, s)
    pcol = icol.transpose(0, 2, 3, 1, 4).reshape(-1, s, 3)
    mask = (index != -1).transpose(0, 2, 3, 1).reshape(-1, s)
    oc, ot = oracle.composite(psdf, pcol, mask, scene.sharpness)
    want = (oc + scene.background[None] * ot[:, None]).reshape(b, h, w, 3).transpose(0, 3, 1, 2)
    np.testing.assert_allclose(_n(image), want, atol=IMAGE_ATOL, rtol=0)

    g = np.random.default_rng(2).normal(0, 1, want.shape).astype(np.float32)
    image.backward(_t(g, d))
    gc = g.transpose(0, 2, 3, 1).reshape(-1, 3)
    gt = (gc * scene.background[None]).sum(-1)
    gpsdf, gpcol, gsharp = oracle.composite_backward(psdf, pcol, mask, scene.sharpness, oc, ot, gc, gt,
                                                     exact=(mode == "exact"))
    gisdf = gpsdf.reshape(b, h, w, s).transpose(0, 3, 1, 2)
    gicol = gpcol.reshape(b, h, w, s, 3).transpose(0, 3, 1, 2, 4)
    gsdf, gcolors = oracle.interpolate_backward(uv, index, scene.faces, scene.vertices.shape[0], b, gisdf, gicol)
    gsh = oracle.evaluate_spherical_harmonics_backward(scene.vertices, scene.sh.shape, scene.extrinsics,
                                                       scene.sh_degree, colors, gcolors)
    _close_grad(_n(inputs["signed_distances"].grad), gsdf)
    _close_grad(_n(inputs["spherical_harmonics"].grad), gsh)
    assert abs(float(inputs["sharpness"].grad) - gsharp) <= GRAD_RTOL * max(abs(gsharp), 1e-6) + 1e-6


# ---------------------------------------------------------------------------
# Adversarial triangles: warp culling and the numerator fast reject must not
# change a single hit decision (the oracle evaluates the full test for every
# pixel/triangle pair).
# ---------------------------------------------------------------------------
def _adversarial_triangles(rng, n, h, w):
    kinds = rng.integers(0, 6, n)
    pts = []
    for k in kinds:
        c = rng.uniform([0, 0], [w, h])
        if k == 0:  # small, well shaped
            p = c + rng.normal(0, 3, (3, 2))
        elif k == 1:  # sliver: nearly collinear
            d = rng.normal(0, 1, 2)
            d /= np.linalg.norm(d)
            t = rng.uniform(-20, 20, 3)
            p = c + t[:, None] * d + rng.normal(0, 1e-3, (3, 2))
        elif k == 2:  # degenerate: repeated vertex
            a, b = c, c + rng.normal(0, 5, 2)
            p = np.stack((a, b, a))
        elif k == 3:  # sub-pixel
            p = c + rng.normal(0, 0.3, (3, 2))
        elif k == 4:  # huge, partly off screen
            p = c + rng.normal(0, 200, (3, 2))
        else:  # vertices exactly on pixel centres / edges
            p = np.floor(c) + 0.5 + rng.integers(-4, 5, (3, 2)).astype(float)
        pts.append(p)
    xy = np.concatenate(pts).astype(np.float32)
    faces = np.arange(3 * n, dtype=np.int32).reshape(n, 3)
    # Orient every face so it survives back-face culling.
    a, b, c = xy[faces[:, 0]], xy[faces[:, 1]], xy[faces[:, 2]]
    cross = (b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0])
    flip = cross < 0
    faces[flip, 1], faces[flip, 2] = faces[flip, 2].copy(), faces[flip, 1].copy()
    return xy, faces


@pytest.mark.parametrize("seed", [0, 1, 2])
def test_fused_adversarial_triangles_exact_hits(cuda_device, seed):
    rng = np.random.default_rng(seed)
    h, w, n, s = 96, 112, 3000, 4
    xy, faces = _adversarial_triangles(rng, n, h, w)
    v = xy.shape[0]
    depth = rng.uniform(1.0, 3.0, v).astype(np.float32)
    colors = rng.uniform(0, 1, (1, v, 3)).astype(np.float32)
    sdf = rng.uniform(-0.05, 0.05, v).astype(np.float32)
    sfb = np.array([n // 4, n // 2, 3 * n // 4, n], np.int32)
    d = cuda_device
    grid = tr.TileGrid((16, 16), (h, w), 1, s)
    kd = tr.create_key_defines(("camera", 6), ("tile", 20), ("depth", 32), ("shell", 6))
    xy_t, depth_t = _t(xy[None], d), _t(depth[None], d)
    bounds = tr.bound_triangles(xy_t, depth_t, _t(faces, d), grid, 0.2)
    paired = tr.sort_keys(tr.generate_keys(depth_t, _t(faces, d), _t(sfb, d), bounds.tile_minima, bounds.tile_maxima,
                                           bounds.num_tiles_overlapped, grid, kd))
    tb = tr.delineate_tiles(paired, grid, kd, False)
    t = grid.num_tiles_per_image
    out = tr.intersect_and_composite(xy_t, _t(colors, d), _t(sdf, d), _t(faces, d), torch.tensor(50.0, device=d),
                                     paired.keys, paired.triangle_indices, tb.view(1, t, 2), s, grid, kd)
    want = oracle.intersect_and_composite(xy[None], colors, sdf, faces, 50.0, _n(paired.keys),
                                          _n(paired.triangle_indices), _n(tb).reshape(1, t, 2), s, (16, 16), (h, w), kd)
    np.testing.assert_allclose(_n(out), want, atol=IMAGE_ATOL, rtol=0)
    assert (want[0, 3] < 1).mean() > 0.2


@pytest.mark.parametrize("name", list(SCENES))
def test_both_modes_match_oracle_renders(cuda_device, name):
    """The full render in each mode equals the oracle's render of the same
    mode (the two modes themselves differ where shells of several objects
    interleave in depth, as the reference's do)."""
    scene = make_scene(**SCENES[name])
    inputs = _fused_inputs(scene, cuda_device)
    args = (scene.extrinsics, scene.intrinsics, scene.image_shape, scene.vertices, scene.faces,
            scene.face_boundaries, scene.sdf, scene.sh, scene.sh_degree, scene.sharpness, scene.background)
    with torch.no_grad():
        fused = _n(tr.render(**inputs, mode="fused"))
        explicit = _n(tr.render(**inputs, mode="explicit"))
    np.testing.assert_allclose(fused, oracle.render_fused(*args).image, atol=IMAGE_ATOL, rtol=0)
    np.testing.assert_allclose(explicit, oracle.render_explicit(*args), atol=IMAGE_ATOL, rtol=0)


# ---------------------------------------------------------------------------
# Tile-bucketed sort: the same keys, triangles and tile ranges as the stable
# radix sort followed by delineate_tiles.
# ---------------------------------------------------------------------------
def _random_keys(rng, n, b, s, rows, cols, explicit, hot_tile=None):
    kd = tr.create_key_defines(*(EXPLICIT_KEYS if explicit else FUSED_KEYS))
    d = dict(kd)
    cam = rng.integers(0, b, n).astype(np.uint64)
    tile = rng.integers(0, rows * cols, n).astype(np.uint64)
    if hot_tile is not None:
        tile[:] = hot_tile
    shell = rng.integers(0, s, n).astype(np.uint64)
    depth = rng.choice(rng.uniform(0.5, 4.0, max(n // 7, 1)).astype(np.float32), n).view(np.uint32).astype(np.uint64)
    key = ((cam << np.uint64(d["CAMERA_BIT_OFFSET"])) | (tile << np.uint64(d["TILE_BIT_OFFSET"]))
           | (depth << np.uint64(d["DEPTH_BIT_OFFSET"])) | (shell << np.uint64(d["SHELL_BIT_OFFSET"])))
    tri = rng.integers(0, 1 << 30, n).astype(np.int32)
    return key.view(np.int64), tri, kd


FUSED_KEYS = (("camera", 6), ("tile", 20), ("depth", 32), ("shell", 6))
EXPLICIT_KEYS = (("camera", 6), ("shell", 6), ("tile", 20), ("depth", 32))


@pytest.mark.parametrize("explicit", [False, True])
@pytest.mark.parametrize("n,b,s,rows,cols,hot", [
    (1, 1, 1, 1, 1, None),
    (5000, 4, 3, 7, 9, None),
    (300_000, 32, 8, 40, 50, None),
    (200_000, 2, 1, 10, 20, None),  # ~500 keys per bin: the 64- and 128-thread tiers
    (150_000, 1, 2, 15, 20, None),
    (100_000, 2, 4, 3, 3, 4),  # one tile of 50k keys per camera: chunks and merge rounds
    (20_000, 3, 2, 60, 70, 0),
])
def test_tile_sort_matches_radix_and_delineate(cuda_device, explicit, n, b, s, rows, cols, hot):
    d = cuda_device
    rng = np.random.default_rng(n + b + s)
    keys, tri, kd = _random_keys(rng, n, b, s, rows, cols, explicit, hot)
    grid = tr.TileGrid((16, 16), (16 * rows, 16 * cols), b, s)
    paired = tr.PairedKeys(_t(keys, d), _t(tri, d), None)
    got, got_bounds = tr._sort_and_delineate(paired, grid, kd, explicit)
    want = tr.sort_keys(paired, grid)
    want_bounds = tr.delineate_tiles(want, grid, kd, explicit)
    np.testing.assert_array_equal(_n(got.keys), _n(want.keys))
    np.testing.assert_array_equal(_n(got.triangle_indices), _n(want.triangle_indices))
    np.testing.assert_array_equal(_n(got_bounds), _n(want_bounds))
    assert nt.library().mt_sort_keys_by_tile_supported(tr._layout(kd), int(explicit), b, n) == 1


def test_tile_sort_live_count(cuda_device):
    """Keys past a device live count are neither sorted nor delineated."""
    d = cuda_device
    rng = np.random.default_rng(7)
    keys, tri, kd = _random_keys(rng, 40_000, 4, 8, 20, 30, False)
    grid = tr.TileGrid((16, 16), (320, 480), 4, 8)
    live = torch.tensor(31_337, dtype=torch.int64, device=d)
    paired = tr.PairedKeys(_t(keys, d), _t(tri, d), live)
    got, got_bounds = tr._sort_and_delineate(paired, grid, kd, False)
    want = tr.sort_keys(paired, grid)
    want_bounds = tr.delineate_tiles(want, grid, kd, False)
    np.testing.assert_array_equal(_n(got.keys)[:31_337], _n(want.keys)[:31_337])
    np.testing.assert_array_equal(_n(got.triangle_indices)[:31_337], _n(want.triangle_indices)[:31_337])
    np.testing.assert_array_equal(_n(got_bounds), _n(want_bounds))


def test_tile_sort_falls_back_when_a_camera_sets_the_sign_bit(cuda_device):
    """With more than 32 cameras in a 6-bit field, cameras 32.. sort first as
    signed keys; the bucketed order would differ, so the radix sort runs."""
    d = cuda_device
    rng = np.random.default_rng(3)
    keys, tri, kd = _random_keys(rng, 20_000, 40, 2, 4, 5, False)
    assert nt.library().mt_sort_keys_by_tile_supported(tr._layout(kd), 0, 40, 20_000) == 0
    grid = tr.TileGrid((16, 16), (64, 80), 40, 2)
    paired = tr.PairedKeys(_t(keys, d), _t(tri, d), None)
    got, got_bounds = tr._sort_and_delineate(paired, grid, kd, False)
    want = tr.sort_keys(paired, grid)
    np.testing.assert_array_equal(_n(got.keys), _n(want.keys))
    np.testing.assert_array_equal(_n(got_bounds), _n(tr.delineate_tiles(want, grid, kd, False)))


# ---------------------------------------------------------------------------
# Fused bound + scan + keys (capacity mode)
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", list(SCENES))
def test_bound_and_generate_keys_matches_oracle(cuda_device, name):
    scene = make_scene(**SCENES[name])
    grid, kd, xy, depth, bounds, paired, sorted_, tb = _front(scene, cuda_device)
    want = oracle.render_fused(scene.extrinsics, scene.intrinsics, scene.image_shape, scene.vertices, scene.faces,
                               scene.face_boundaries, scene.sdf, scene.sh, scene.sh_degree, scene.sharpness,
                               scene.background)
    faces, sfb = _t(scene.faces, cuda_device), _t(scene.face_boundaries, cuda_device)
    n = want.keys.size
    for capacity in (n, n + 1000, n // 2, 0):
        got = tr.bound_and_generate_keys(xy, depth, faces, sfb, grid, 0.2, kd, capacity)
        assert int(got.count.item()) == n
        m = min(n, capacity)
        np.testing.assert_array_equal(_n(got.keys)[:m], want.keys[:m])
        np.testing.assert_array_equal(_n(got.triangle_indices)[:m], want.tri[:m])


def _random_front(rng, b, f, v, grid):
    h, w = grid.image_shape
    xy = np.stack([rng.uniform(-40, w + 40, (b, v)), rng.uniform(-40, h + 40, (b, v))], -1).astype(np.float32)
    # Small triangles mostly, a few that span many tiles.
    centre = rng.integers(0, v, f)
    spread = rng.integers(1, 40, f)
    spread[rng.random(f) < 0.01] = v
    faces = np.stack([centre, (centre + rng.integers(0, 1 + spread)) % v, (centre + rng.integers(0, 1 + spread)) % v],
                     -1).astype(np.int32)
    depth = rng.uniform(0.1, 5.0, (b, v)).astype(np.float32)  # some corners before the near plane
    return xy, depth, faces


@pytest.mark.parametrize("b,f,ragged,live", [
    (1, 1, False, None),
    (1, 1023, False, None),
    (2, 1025, False, 700),
    (4, 200_000, False, None),
    (3, 150_001, True, None),
    (8, 90_000, True, 61_234),
])
def test_bound_and_generate_keys_matches_three_stage_chain(cuda_device, b, f, ragged, live):
    d = cuda_device
    rng = np.random.default_rng(b * 7 + f)
    s = 5
    if ragged:
        shapes = [(int(rng.integers(40, 400)), int(rng.integers(40, 500))) for _ in range(b)]
        grid = tr.TileGrid.for_cameras((16, 16), shapes, s)
    else:
        grid = tr.TileGrid((16, 16), (300, 420), b, s)
    xy, depth, faces = _random_front(rng, b, f, max(f // 2, 3), grid)
    kd = tr.create_key_defines(*FUSED_KEYS)
    sfb = np.sort(rng.integers(0, f + 1, s)).astype(np.int32)
    sfb[-1] = f
    xy_t, depth_t, faces_t, sfb_t = _t(xy, d), _t(depth, d), _t(faces, d), _t(sfb, d)
    nf = torch.tensor(live, dtype=torch.int32, device=d) if live is not None else None
    bounds = tr.bound_triangles(xy_t, depth_t, faces_t, grid, 0.2, nf)
    want = tr.generate_keys(depth_t, faces_t, sfb_t, bounds.tile_minima, bounds.tile_maxima,
                            bounds.num_tiles_overlapped, grid, kd)
    n = want.num_keys
    assert n > 0 or f < 100
    for capacity in (n, n + 333, (2 * n) // 3):
        got = tr.bound_and_generate_keys(xy_t, depth_t, faces_t, sfb_t, grid, 0.2, kd, capacity, nf)
        assert int(got.count.item()) == n
        m = min(n, capacity)
        np.testing.assert_array_equal(_n(got.keys)[:m], _n(want.keys)[:m])
        np.testing.assert_array_equal(_n(got.triangle_indices)[:m], _n(want.triangle_indices)[:m])
    assert nt.workspace(torch.device(d)).status() == 0


# A whole 8-shell sphere in a few tiles: warps walk hundreds of batches, so
# a small hit-bit budget runs out inside a work item and the backward mixes
# stored and re-tested batches.
DENSE = dict(cameras=((0.0, 0.0, 8.0),), image_shape=(32, 32), fov=20.0,
             levels=tuple(float(x) for x in np.linspace(0.03, -0.03, 8)), sh_degree=1)


@pytest.mark.parametrize("budget", [16, 1])
def test_fused_backward_past_the_stored_batches(cuda_device, budget, monkeypatch):
    """Against the oracle with the default hit-bit budget and with 1 byte per
    pixel, which runs out part-way through the dense tiles' walks."""
    monkeypatch.setattr(tr, "HIT_BITS_BYTES_PER_PIXEL", budget)
    scene = make_scene(**DENSE)
    grid, kd, xy, depth, bounds, paired, sorted_, tb = _front(scene, cuda_device)
    counts = _n(tb)[..., 1] - _n(tb)[..., 0]
    assert counts.max() > 32 * 32 * 4  # tiles of hundreds of batches
    _check_fused_backward(scene, cuda_device, "reference", (16, 16))


def test_hit_bit_store_size_follows_the_work(cuda_device):
    """The store holds the batches the keys can form, not a fixed number of
    batches per warp: at most K * warps / 32 + work items batches, and never
    more than the byte budget."""
    lib = nt.library()
    header = lib.mt_composite_hit_bits_bytes(1000, 8, 8, 1) - 128
    assert header == (8 + 4 * 2000 + 127) // 128 * 128
    assert lib.mt_composite_hit_bits_bytes(1000, 8, 8, 10) == header + 10 * 128
    assert lib.mt_composite_hit_bits_bytes(0, 8, 8, 10) == 0

    class Ctx:
        needs_input_grad = (True,)

    grid = tr.TileGrid((8, 8), (800, 800), 4, 8)
    hits = tr._hit_bits(Ctx(), grid, 2_500_000, cuda_device)
    most = 2_500_000 * 2 // 32 + grid.camera_tiles * 2
    assert hits.numel() == lib.mt_composite_hit_bits_bytes(grid.camera_tiles, 8, 8, most)
    assert hits.numel() < 12 * 4 * 8 * 800 * 800 / 6  # far below the explicit mode's buffers
    dense = tr._hit_bits(Ctx(), grid, 100_000_000, cuda_device)  # capped by the budget
    budget = tr.HIT_BITS_BYTES_PER_PIXEL * grid.camera_tiles * 64 // 128
    assert dense.numel() == lib.mt_composite_hit_bits_bytes(grid.camera_tiles, 8, 8, budget)


@pytest.mark.parametrize("name", ["three_cams_odd", "multi_inside", "dense"])
def test_backward_with_and_without_stored_hit_bits(cuda_device, name, monkeypatch):
    """The backward reads the forward's hit bits for the batches the store
    holds; without them it tests every batch again. Both give the same
    gradients (up to the order of the compositing atomics)."""
    d = cuda_device
    scene = make_scene(**(DENSE if name == "dense" else SCENES[name]))
    grid, kd, xy, depth, bounds, paired, sorted_, tb = _front(scene, d)
    colors_np = oracle.evaluate_spherical_harmonics(scene.vertices, scene.sh, scene.extrinsics, scene.sh_degree)
    b, s, t = grid.num_cameras, grid.num_shells, grid.num_tiles_per_image
    g = None
    grads = []
    for stored in (True, False):
        if not stored:
            monkeypatch.setattr(tr, "HIT_BITS_BYTES_PER_PIXEL", 0)
        colors = _t(colors_np, d).requires_grad_(True)
        sdf = _t(scene.sdf, d).requires_grad_(True)
        sharp = torch.tensor(scene.sharpness, device=d).requires_grad_(True)
        out = tr.intersect_and_composite(xy, colors, sdf, _t(scene.faces, d), sharp, sorted_.keys,
                                         sorted_.triangle_indices, tb.view(b, t, 2), s, grid, kd)
        if g is None:
            g = _t(np.random.default_rng(2).normal(0, 1, tuple(out.shape)).astype(np.float32), d)
        out.backward(g)
        grads.append((_n(colors.grad), _n(sdf.grad), float(sharp.grad)))
    (c1, s1, h1), (c0, s0, h0) = grads
    _close_grad(c1, c0, 1e-5)
    _close_grad(s1, s0, 1e-5)
    assert abs(h1 - h0) <= 1e-5 * max(abs(h0), 1e-12)
    assert np.abs(c0).max() > 0


@pytest.mark.parametrize("name", ["three_cams_odd", "multi_inside", "dense"])
@pytest.mark.parametrize("budget", [16, 1, 0])
def test_staged_backward_matches_unstaged(cuda_device, name, budget, monkeypatch):
    """The backward whose vertex records arrive by bulk copies into shared
    memory gives the gradients of the plain backward (up to the order of the
    compositing atomics), with all, some or none of the hit bits stored."""
    d = cuda_device
    monkeypatch.setattr(tr, "HIT_BITS_BYTES_PER_PIXEL", budget)
    scene = make_scene(**(DENSE if name == "dense" else SCENES[name]))
    grid, kd, xy, depth, bounds, paired, sorted_, tb = _front(scene, d)
    colors_np = oracle.evaluate_spherical_harmonics(scene.vertices, scene.sh, scene.extrinsics, scene.sh_degree)
    b, s, t = grid.num_cameras, grid.num_shells, grid.num_tiles_per_image
    g = None
    grads = []
    for staged in (False, True):
        monkeypatch.setattr(tr, "STAGED_BACKWARD", staged)
        colors = _t(colors_np, d).requires_grad_(True)
        sdf = _t(scene.sdf, d).requires_grad_(True)
        sharp = torch.tensor(scene.sharpness, device=d).requires_grad_(True)
        out = tr.intersect_and_composite(xy, colors, sdf, _t(scene.faces, d), sharp, sorted_.keys,
                                         sorted_.triangle_indices, tb.view(b, t, 2), s, grid, kd)
        if g is None:
            g = _t(np.random.default_rng(4).normal(0, 1, tuple(out.shape)).astype(np.float32), d)
        out.backward(g)
        grads.append((_n(colors.grad), _n(sdf.grad), float(sharp.grad)))
    (c0, s0, h0), (c1, s1, h1) = grads
    _close_grad(c1, c0, 1e-5)
    _close_grad(s1, s0, 1e-5)
    assert abs(h1 - h0) <= 1e-5 * max(abs(h0), 1e-12)
    assert np.abs(c0).max() > 0


def test_staged_backward_in_the_fused_loss_matches_oracle(cuda_device, monkeypatch):
    monkeypatch.setattr(tr, "STAGED_BACKWARD", True)
    scene = make_scene(**SCENES["three_cams_odd"])
    _check_fused_backward(scene, cuda_device, "reference", (16, 16))


@pytest.mark.parametrize("name", ["three_cams_odd", "multi_inside"])
@pytest.mark.parametrize("tile", [(8, 8), (16, 16), (16, 8)])
def test_threads_per_cta_leave_results_unchanged(cuda_device, name, tile):
    """The compositing kernels' CTA size (128, 256 or 512 threads of
    persistent warps, the third element of tile_shape) only changes the
    launch: identical images, the same gradients up to atomic order."""
    scene = make_scene(**SCENES[name])
    results = []
    for threads in (256, 128, 512):
        inputs = _fused_inputs(scene, cuda_device)
        image = tr.render(**inputs, tile_shape=(*tile, threads), mode="fused")
        g = _t(np.random.default_rng(7).normal(0, 1, tuple(image.shape)).astype(np.float32), cuda_device)
        (image * g).sum().backward()
        results.append((_n(image), _n(inputs["signed_distances"].grad), _n(inputs["spherical_harmonics"].grad)))
    for img, gs, gh in results[1:]:
        np.testing.assert_array_equal(img, results[0][0])
        _close_grad(gs, results[0][1], 1e-5)
        _close_grad(gh, results[0][2], 1e-5)


def test_tile_grid_rejects_other_thread_counts():
    with pytest.raises(ValueError):
        tr.TileGrid((8, 8, 96), (64, 64), 1, 3)
    assert tr.TileGrid((8, 8, 512), (64, 64), 1, 3).tile_shape == (8, 8)


@pytest.mark.parametrize("name", ["three_cams_odd", "dense"])
def test_tile_order_leaves_fused_results_unchanged(cuda_device, name, monkeypatch):
    """Longest-first tile order on or off: identical images, the same
    gradients up to atomic order (uniform cameras, hit bits stored)."""
    scene = make_scene(**(DENSE if name == "dense" else SCENES[name]))
    results = []
    for ordered in (False, True):
        monkeypatch.setattr(tr, "TILE_ORDER", ordered)
        inputs = _fused_inputs(scene, cuda_device)
        image = tr.render(**inputs, tile_shape=(8, 8), mode="fused")
        g = _t(np.random.default_rng(8).normal(0, 1, tuple(image.shape)).astype(np.float32), cuda_device)
        (image * g).sum().backward()
        results.append((_n(image), _n(inputs["signed_distances"].grad), _n(inputs["spherical_harmonics"].grad)))
    np.testing.assert_array_equal(results[1][0], results[0][0])
    _close_grad(results[1][1], results[0][1], 1e-5)
    _close_grad(results[1][2], results[0][2], 1e-5)


def test_fused_loss_with_every_tile_keyless(cuda_device):
    """Triangles, but all of them far outside the image: every tile is
    keyless (the backward then takes no work item): the loss is the
    background's squared error and every gradient is zero."""
    scene = make_scene()
    inputs = _fused_inputs(scene, cuda_device)
    inputs["vertices"] = inputs["vertices"] + torch.tensor([50.0, 0.0, 0.0], device=cuda_device)
    h, w = scene.image_shape
    target = _t(np.random.default_rng(11).uniform(0, 1, (1, 3, h, w)).astype(np.float32), cuda_device)
    loss = tr.render_fused_loss(inputs["extrinsics"], inputs["intrinsics"], (h, w), inputs["vertices"],
                                inputs["faces"], inputs["shell_face_boundaries"], inputs["signed_distances"],
                                inputs["spherical_harmonics"], inputs["sh_degree"], inputs["sharpness"],
                                inputs["background"], target, tile_shape=(8, 8))
    loss.backward()
    bg = torch.clamp(inputs["background"], 0, 1)[None, :, None, None].expand(1, 3, h, w)
    want = float(((bg - target) ** 2).mean())
    assert abs(float(loss) - want) <= 1e-5 * want
    assert float(inputs["signed_distances"].grad.abs().max()) == 0.0
    assert float(inputs["spherical_harmonics"].grad.abs().max()) == 0.0
