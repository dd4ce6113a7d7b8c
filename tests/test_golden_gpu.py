"""GPU path against the reference's own kernel outputs (tests/golden/).

The product API is chained stage by stage on the fixtures' inputs, exactly
as the reference's Python call sites chain its kernels; every stage must
match the reference bit for bit: voxels, dilation, tessellation, projection,
tile bounds, keys in both layouts, sorted keys, tile ranges, camera centres,
SH colours, explicit hits (face index and barycentrics) and interpolation.
Outputs that pass through exp() (the fused image, the shell compositing and
the rendered images) agree within 1e-5 max-abs: CUDA's expf and the host
libm's exp may differ in the last bits. The full render entry points are
checked against the fixtures' images with the background blended in.

Gradients in the default ("reference") routing must reproduce the
reference's hand-written backward kernels within 1e-4 of the largest
gradient magnitude, and within 1e-4 relative on every entry whose magnitude
is at least 1e-3 of the largest.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from meshtryoshka_gb300 import triangle_extraction as te
from meshtryoshka_gb300 import triangle_rasterization as tr
from tests import goldens

pytestmark = pytest.mark.gpu

FUSED_KEYS = (("camera", 6), ("tile", 20), ("depth", 32), ("shell", 6))
EXPLICIT_KEYS = (("camera", 6), ("shell", 6), ("tile", 20), ("depth", 32))
BACKGROUND = np.array([0.2, 0.4, 0.6], np.float32)
IMAGE_ATOL = 1e-5
GRAD_RTOL = 1e-4
ENTRY_FLOOR = 1e-3


def _t(a, device):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _n(t):
    return t.detach().cpu().numpy()


def _eq(got, want, what):
    np.testing.assert_array_equal(_n(got), want, err_msg=what)


def _near(got, want, what):
    np.testing.assert_allclose(_n(got), want, atol=IMAGE_ATOL, rtol=0, err_msg=what)


def _close_grad(got, want, what):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    scale = max(float(np.abs(want).max()), 1e-30)
    err = float(np.abs(got - want).max())
    assert err <= GRAD_RTOL * scale, f"{what}: max abs err {err:.3e} > {GRAD_RTOL:g} x {scale:.3e}"
    # Per entry, relative, wherever the entry is not lost in the atomics'
    # rounding: magnitude at least 1e-3 of the largest.
    big = np.abs(want) >= ENTRY_FLOOR * scale
    if big.any():
        rel = float((np.abs(got - want)[big] / np.abs(want[big])).max())
        assert rel <= GRAD_RTOL, f"{what}: per-entry relative err {rel:.3e} > {GRAD_RTOL:g}"


@pytest.fixture(scope="module")
def extraction():
    return goldens.load("extraction")


@pytest.mark.parametrize("grid", goldens.EXTRACTION_GRIDS)
def test_voxels_match_reference(cuda_device, extraction, grid):
    g = {k.split("/", 1)[1]: v for k, v in extraction.items() if k.startswith(grid + "/")}
    occ = _t(g["occupancy"], cuda_device)
    vox = te.extract_voxels(occ)
    for field in ("vertices", "neighbors", "lower_corners", "upper_corners", "indices"):
        _eq(getattr(vox, field), g[field], field)
    vocc = te.compute_vertex_occupancy(occ)
    _eq(vocc.vertex_occupancy, g["vertex_occupancy"], "vertex_occupancy")
    _eq(vocc.vertex_counts, g["vertex_counts"], "vertex_counts")
    _eq(te.count_occupancy(occ), g["voxel_counts"], "voxel_counts")
    for d in (1, 3):
        _eq(te.dilate_occupancy(occ, d), g[f"dilated_{d}"], f"dilated_{d}")


def test_tessellation_matches_reference(cuda_device, extraction):
    e, d = extraction, cuda_device
    tri = te.tessellate_voxels(_t(e["tess/signed_distances"], d), _t(e["sphere/vertices"], d),
                               _t(e["tess/spherical_harmonics"], d), _t(e["sphere/neighbors"], d),
                               _t(e["sphere/lower_corners"], d), _t(e["sphere/upper_corners"], d),
                               _t(e["sphere/indices"], d), _t(e["tess/level_sets"], d))
    for field in ("vertices", "signed_distances", "spherical_harmonics", "faces", "voxel_indices"):
        _eq(getattr(tri, field), e[f"tess/out_{field}"], field)
    s = e["tess/level_sets"].shape[0]
    _eq(tri.vertex_boundaries, e["tess/out_vertex_offsets"][1:].reshape(s, -1)[:, -1], "vertex_boundaries")
    _eq(tri.face_boundaries, e["tess/out_face_offsets"][1:].reshape(s, -1)[:, -1] // 3, "face_boundaries")


@pytest.mark.parametrize("scene", goldens.RASTER_SCENES)
def test_raster_stages_match_reference(cuda_device, scene):
    g, d = goldens.raster(scene), cuda_device
    b, s, h, w, rows, cols = goldens.grid_dims(g)
    grid = tr.TileGrid((16, 16), (h, w), b, s)
    verts, faces = _t(g["vertices"], d), _t(g["faces"], d)
    sdf, sfb = _t(g["signed_distances"], d), _t(g["shell_face_boundaries"], d)
    xy, depth = tr.project_vertices(verts, _t(g["extrinsics"], d), _t(g["intrinsics"], d))
    _eq(xy, g["xy"], "xy")
    _eq(depth, g["depth"], "depth")
    bounds = tr.bound_triangles(xy, depth, faces, grid, float(g["near_plane"]))
    _eq(bounds.tile_minima, g["tile_minima"], "tile_minima")
    _eq(bounds.tile_maxima, g["tile_maxima"], "tile_maxima")
    _eq(bounds.num_tiles_overlapped, g["num_tiles_overlapped"], "num_tiles_overlapped")
    _eq(tr._camera_positions(_t(g["extrinsics"], d)), g["camera_positions"], "camera_positions")
    colors = tr.evaluate_spherical_harmonics(verts, _t(g["spherical_harmonics"], d), _t(g["extrinsics"], d),
                                             int(g["sh_degree"]))
    _eq(colors, g["colors"], "colors")

    stages = {}
    for mode, layout, separate in (("fused", FUSED_KEYS, False), ("explicit", EXPLICIT_KEYS, True)):
        kd = tr.create_key_defines(*layout)
        paired = tr.generate_keys(depth, faces, sfb, bounds.tile_minima, bounds.tile_maxima,
                                  bounds.num_tiles_overlapped, grid, kd)
        _eq(paired.keys, g[f"{mode}/keys"], f"{mode} keys")
        _eq(paired.triangle_indices, g[f"{mode}/triangles"], f"{mode} triangles")
        paired = tr.sort_keys(paired, grid)
        _eq(paired.keys, g[f"{mode}/sorted_keys"], f"{mode} sorted keys")
        _eq(paired.triangle_indices, g[f"{mode}/sorted_triangles"], f"{mode} sorted triangles")
        tb = tr.delineate_tiles(paired, grid, kd, separate)
        _eq(tb, g[f"{mode}/tile_boundaries"], f"{mode} tile boundaries")
        stages[mode] = (kd, paired, tb)

    kd, paired, tb = stages["fused"]
    image = tr.intersect_and_composite(xy, colors, sdf, faces, float(g["sharpness"]), paired.keys,
                                       paired.triangle_indices, tb.view(b, rows * cols, 2), s, grid, kd)
    _near(image, g["fused/image"], "fused image")

    kd, paired, tb = stages["explicit"]
    uv, index = tr.intersect(xy, faces, paired.triangle_indices, tb, grid, kd)
    _eq(index, g["explicit/index"], "hit index")
    _eq(uv, g["explicit/uv"], "hit uv")
    isdf, icol = tr.interpolate(uv, index, faces, sdf, colors)
    _eq(isdf, g["explicit/interp_sdf"], "interpolated sdf")
    _eq(icol, g["explicit/interp_colors"], "interpolated colours")
    psdf, pcol, mask = goldens.per_pixel_shells(g)
    out_c, out_t = tr.Composite.apply(_t(psdf, d), _t(pcol, d), _t(mask, d), float(g["sharpness"]))
    _near(out_c, g["explicit/composite_colors"], "composite colours")
    _near(out_t, g["explicit/composite_T"], "composite transmittance")


@pytest.mark.parametrize("scene", goldens.RASTER_SCENES)
@pytest.mark.parametrize("mode", ["fused", "explicit"])
def test_render_matches_reference_images(cuda_device, scene, mode):
    g, d = goldens.raster(scene), cuda_device
    b, s, h, w, rows, cols = goldens.grid_dims(g)
    image = tr.render(_t(g["extrinsics"], d), _t(g["intrinsics"], d), (h, w), _t(g["vertices"], d),
                      _t(g["faces"], d), _t(g["shell_face_boundaries"], d), _t(g["signed_distances"], d),
                      _t(g["spherical_harmonics"], d), int(g["sh_degree"]), float(g["sharpness"]),
                      _t(BACKGROUND, d), near_plane=float(g["near_plane"]), mode=mode)
    if mode == "fused":
        f = g["fused/image"]
        want = np.clip(f[:, :3] + f[:, 3:4] * BACKGROUND[:, None, None], 0, 1)
    else:
        rgb = g["explicit/composite_colors"] + BACKGROUND * g["explicit/composite_T"][:, None]
        want = rgb.reshape(b, h, w, 3).transpose(0, 3, 1, 2)
    np.testing.assert_allclose(_n(image), want, atol=IMAGE_ATOL, rtol=0)


@pytest.mark.parametrize("scene", goldens.RASTER_SCENES)
def test_fused_backward_matches_reference(cuda_device, scene):
    g, d = goldens.raster(scene), cuda_device
    b, s, h, w, rows, cols = goldens.grid_dims(g)
    grid = tr.TileGrid((16, 16), (h, w), b, s)
    kd = tr.create_key_defines(*FUSED_KEYS)
    colors = _t(g["colors"], d).requires_grad_(True)
    sdf = _t(g["signed_distances"], d).requires_grad_(True)
    sharp = torch.tensor(float(g["sharpness"]), device=d, requires_grad=True)
    out = tr.intersect_and_composite(_t(g["xy"], d), colors, sdf, _t(g["faces"], d), sharp,
                                     _t(g["fused/sorted_keys"], d), _t(g["fused/sorted_triangles"], d),
                                     _t(g["fused/tile_boundaries"].reshape(b, rows * cols, 2), d), s, grid, kd,
                                     gradient_mode="reference")
    out.backward(_t(g["fused/grad_image"], d))
    _close_grad(_n(colors.grad), g["fused/grad_colors"], "colours")
    _close_grad(_n(sdf.grad), g["fused/grad_signed_distances"], "signed distances")
    _close_grad([float(sharp.grad)], [g["fused/grad_sharpness"]], "sharpness")


@pytest.mark.parametrize("scene", goldens.RASTER_SCENES)
def test_explicit_composite_backward_matches_reference(cuda_device, scene):
    g, d = goldens.raster(scene), cuda_device
    psdf, pcol, mask = goldens.per_pixel_shells(g)
    sdf = _t(psdf, d).requires_grad_(True)
    col = _t(pcol, d).requires_grad_(True)
    sharp = torch.tensor(float(g["sharpness"]), device=d, requires_grad=True)
    out_c, out_t = tr.Composite.apply(sdf, col, _t(mask, d), sharp, "reference")
    torch.autograd.backward((out_c, out_t), (_t(g["explicit/grad_composite_colors"], d),
                                             _t(g["explicit/grad_composite_T"], d)))
    _close_grad(_n(sdf.grad), g["explicit/grad_shell_signed_distances"], "signed distances")
    _close_grad(_n(col.grad), g["explicit/grad_shell_colors"], "colours")
    _close_grad([float(sharp.grad)], [g["explicit/grad_sharpness"]], "sharpness")


@pytest.mark.parametrize("case", ["sphere", "random"])
def test_sdf_regularizers_match_reference(cuda_device, extraction, case):
    from oracle import oracle

    e, d = extraction, cuda_device
    grid = "sphere" if case == "sphere" else "random"
    args = [e[f"{grid}/neighbors"], e[f"{grid}/lower_corners"], e[f"{grid}/upper_corners"]]
    size = tuple(int(x) for x in e[f"reg_{case}/grid_size"])
    sdf = _t(e[f"reg_{case}/signed_distances"], d).requires_grad_(True)
    losses = te.compute_sdf_regularizers(sdf, *(_t(a, d) for a in args), size)
    for value, name in zip(losses, ("eikonal_loss_pos", "eikonal_loss_neg", "curvature_loss")):
        _eq(value, e[f"reg_{case}/{name}"], name)
    rng = np.random.default_rng(3)
    g = [rng.normal(0, 1, e[f"reg_{case}/curvature_loss"].shape).astype(np.float32) for _ in range(3)]
    torch.autograd.backward(list(losses), [_t(x, d) for x in g])
    want = oracle.compute_sdf_regularizers_backward(e[f"reg_{case}/signed_distances"], *args, size, *g)
    _close_grad(_n(sdf.grad), want, "signed distances")
