"""Pins the CPU oracle to the reference's own kernel outputs.

The fixtures in tests/golden/ were computed by the reference's compute
kernels (compiled on the host from its sources, see tests/golden/make_golden.py).
Every stage of the oracle must reproduce them bit for bit from the same
inputs: voxel extraction, dilation, marching-cubes tessellation, projection,
tile bounds, keys in both layouts, sorting, tile ranges, spherical harmonics,
the fused intersect-and-composite image, and the explicit intersect /
interpolate / composite chain.

Gradients: the oracle's default ("reference") routing must reproduce the
reference's two hand-written backward kernels (fused intersect-and-composite,
explicit composite) within 1e-4 of the largest gradient magnitude, and within 1e-4 relative on
every entry whose magnitude is at least 1e-3 of the largest.

When the reference tree is mounted, the fixtures are also regenerated in
memory and must equal the committed files (gradients, which the reference
accumulates with atomics in a thread-order-dependent sum, within 1e-5).
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle
from tests import goldens

GRAD_RTOL = 1e-4
ENTRY_FLOOR = 1e-3
ATOMIC_OUTPUTS = ("fused/grad_colors", "fused/grad_signed_distances", "fused/grad_sharpness",
                  "explicit/grad_shell_signed_distances", "explicit/grad_shell_colors", "explicit/grad_sharpness")


def close_grad(got, want, rtol=GRAD_RTOL, what="", entry_rtol=None):
    got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
    scale = max(float(np.abs(want).max()), 1e-30)
    err = float(np.abs(got - want).max())
    assert err <= rtol * scale, f"{what}: max abs err {err:.3e} > {rtol:g} x {scale:.3e}"
    # Per entry, relative, wherever the entry is not lost in the sum's
    # rounding: magnitude at least 1e-3 of the largest.
    big = np.abs(want) >= ENTRY_FLOOR * scale
    if big.any():
        entry_rtol = rtol if entry_rtol is None else entry_rtol
        rel = float((np.abs(got - want)[big] / np.abs(want[big])).max())
        assert rel <= entry_rtol, f"{what}: per-entry relative err {rel:.3e} > {entry_rtol:g}"


@pytest.fixture(scope="module")
def extraction():
    return goldens.load("extraction")


@pytest.mark.parametrize("grid", goldens.EXTRACTION_GRIDS)
def test_oracle_extract_voxels_matches_reference(extraction, grid):
    g = {k.split("/", 1)[1]: v for k, v in extraction.items() if k.startswith(grid + "/")}
    occ = g["occupancy"]
    vox = oracle.extract_voxels(occ)
    for field in ("vertices", "neighbors", "lower_corners", "upper_corners", "indices"):
        np.testing.assert_array_equal(getattr(vox, field), g[field], err_msg=field)
    vocc, vcounts = oracle.compute_vertex_occupancy(occ)
    np.testing.assert_array_equal(vocc, g["vertex_occupancy"])
    np.testing.assert_array_equal(vcounts, g["vertex_counts"])
    np.testing.assert_array_equal(oracle.count_occupancy(occ), g["voxel_counts"])
    for d in (1, 3):
        np.testing.assert_array_equal(oracle.dilate_occupancy(occ, d), g[f"dilated_{d}"], err_msg=f"dilation {d}")


def test_oracle_tessellation_matches_reference(extraction):
    e = extraction
    tri = oracle.tessellate_voxels(e["tess/signed_distances"], e["sphere/vertices"], e["tess/spherical_harmonics"],
                                   e["sphere/neighbors"], e["sphere/lower_corners"], e["sphere/upper_corners"],
                                   e["sphere/indices"], e["tess/level_sets"])
    assert e["tess/out_faces"].shape[0] > 0
    for field in goldens.TESS_FIELDS:
        np.testing.assert_array_equal(getattr(tri, field), e[f"tess/out_{field}"], err_msg=field)


@pytest.mark.parametrize("scene", goldens.RASTER_SCENES)
def test_oracle_raster_front_end_matches_reference(scene):
    g = goldens.raster(scene)
    b, s, h, w, rows, cols = goldens.grid_dims(g)
    xy, depth = oracle.project_vertices(g["vertices"], g["extrinsics"], g["intrinsics"])
    np.testing.assert_array_equal(xy, g["xy"])
    np.testing.assert_array_equal(depth, g["depth"])
    tmin, tmax, count = oracle.bound_triangles(xy, depth, g["faces"], (16, 16), (rows, cols), float(g["near_plane"]))
    np.testing.assert_array_equal(tmin, g["tile_minima"])
    np.testing.assert_array_equal(tmax, g["tile_maxima"])
    np.testing.assert_array_equal(count, g["num_tiles_overlapped"])
    np.testing.assert_array_equal(oracle.camera_positions(g["extrinsics"]), g["camera_positions"])
    colors = oracle.evaluate_spherical_harmonics(g["vertices"], g["spherical_harmonics"], g["extrinsics"],
                                                 int(g["sh_degree"]))
    np.testing.assert_array_equal(colors, g["colors"])
    for mode, kd, explicit in (("fused", oracle.fused_key_defines(), False),
                               ("explicit", oracle.explicit_key_defines(), True)):
        keys, tri = oracle.generate_keys(depth, g["faces"], g["shell_face_boundaries"], tmin, tmax, count, cols, kd)
        np.testing.assert_array_equal(keys, g[f"{mode}/keys"], err_msg=mode)
        np.testing.assert_array_equal(tri, g[f"{mode}/triangles"], err_msg=mode)
        sk, st = oracle.sort_pairs(keys, tri)
        np.testing.assert_array_equal(sk, g[f"{mode}/sorted_keys"], err_msg=mode)
        np.testing.assert_array_equal(st, g[f"{mode}/sorted_triangles"], err_msg=mode)
        bounds = oracle.delineate_tiles(sk, kd, explicit, b, s, rows * cols)
        np.testing.assert_array_equal(bounds.reshape(g[f"{mode}/tile_boundaries"].shape),
                                      g[f"{mode}/tile_boundaries"], err_msg=mode)


@pytest.mark.parametrize("scene", goldens.RASTER_SCENES)
def test_oracle_fused_image_matches_reference(scene):
    g = goldens.raster(scene)
    b, s, h, w, rows, cols = goldens.grid_dims(g)
    image = oracle.intersect_and_composite(g["xy"], g["colors"], g["signed_distances"], g["faces"],
                                           float(g["sharpness"]), g["fused/sorted_keys"], g["fused/sorted_triangles"],
                                           g["fused/tile_boundaries"].reshape(b, rows * cols, 2), s, (16, 16), (h, w),
                                           oracle.fused_key_defines())
    np.testing.assert_array_equal(image, g["fused/image"])


@pytest.mark.parametrize("scene", goldens.RASTER_SCENES)
def test_oracle_explicit_chain_matches_reference(scene):
    g = goldens.raster(scene)
    b, s, h, w, rows, cols = goldens.grid_dims(g)
    uv, index = oracle.intersect(g["xy"], g["faces"], g["explicit/sorted_triangles"], g["explicit/tile_boundaries"],
                                 s, (16, 16), (h, w))
    np.testing.assert_array_equal(index, g["explicit/index"])
    np.testing.assert_array_equal(uv, g["explicit/uv"])
    isdf, icol = oracle.interpolate(uv, index, g["faces"], g["signed_distances"], g["colors"])
    np.testing.assert_array_equal(isdf, g["explicit/interp_sdf"])
    np.testing.assert_array_equal(icol, g["explicit/interp_colors"])
    sdf, col, mask = goldens.per_pixel_shells(g)
    out_c, out_t = oracle.composite(sdf, col, mask, float(g["sharpness"]))
    np.testing.assert_array_equal(out_c, g["explicit/composite_colors"])
    np.testing.assert_array_equal(out_t, g["explicit/composite_T"])


@pytest.mark.parametrize("scene", goldens.RASTER_SCENES)
def test_oracle_fused_backward_matches_reference(scene):
    g = goldens.raster(scene)
    b, s, h, w, rows, cols = goldens.grid_dims(g)
    gc, gs, gsh = oracle.intersect_and_composite_backward(
        g["xy"], g["colors"], g["signed_distances"], g["faces"], float(g["sharpness"]), g["fused/sorted_keys"],
        g["fused/sorted_triangles"], g["fused/tile_boundaries"].reshape(b, rows * cols, 2), s, (16, 16), (h, w),
        oracle.fused_key_defines(), g["fused/image"], g["fused/grad_image"], exact=False)
    close_grad(gc, g["fused/grad_colors"], what="colours")
    close_grad(gs, g["fused/grad_signed_distances"], what="signed distances")
    close_grad([gsh], [g["fused/grad_sharpness"]], what="sharpness")


@pytest.mark.parametrize("scene", goldens.RASTER_SCENES)
def test_oracle_explicit_composite_backward_matches_reference(scene):
    g = goldens.raster(scene)
    sdf, col, mask = goldens.per_pixel_shells(g)
    gs, gc, gsh = oracle.composite_backward(sdf, col, mask, float(g["sharpness"]), g["explicit/composite_colors"],
                                            g["explicit/composite_T"], g["explicit/grad_composite_colors"],
                                            g["explicit/grad_composite_T"], exact=False)
    close_grad(gs, g["explicit/grad_shell_signed_distances"], what="signed distances")
    close_grad(gc, g["explicit/grad_shell_colors"], what="colours")
    close_grad([gsh], [g["explicit/grad_sharpness"]], what="sharpness")


def test_fixtures_regenerate_from_reference():
    """The committed fixtures are what the reference's kernels produce now."""
    from oracle import ref

    if not ref.available():
        pytest.skip("reference sources not mounted; the committed fixtures stand")
    from tests.golden import make_golden

    for name, arrays in make_golden.generate().items():
        committed = goldens.load(name)
        assert sorted(arrays) == sorted(committed), name
        for key, value in arrays.items():
            if key in ATOMIC_OUTPUTS:
                # Two runs of the reference's atomics differ by up to ~2e-5 of
                # an entry (summation order), so the per-entry bar is 1e-4.
                close_grad(value, committed[key], rtol=1e-5, what=f"{name}:{key}", entry_rtol=1e-4)
            else:
                np.testing.assert_array_equal(np.asarray(value), committed[key], err_msg=f"{name}:{key}")


@pytest.mark.parametrize("case", ["sphere", "random"])
def test_oracle_sdf_regularizers_match_reference(extraction, case):
    e = extraction
    grid = "sphere" if case == "sphere" else "random"
    got = oracle.compute_sdf_regularizers(e[f"reg_{case}/signed_distances"], e[f"{grid}/neighbors"],
                                          e[f"{grid}/lower_corners"], e[f"{grid}/upper_corners"],
                                          e[f"reg_{case}/grid_size"])
    for value, name in zip(got, ("eikonal_loss_pos", "eikonal_loss_neg", "curvature_loss")):
        np.testing.assert_array_equal(value, e[f"reg_{case}/{name}"], err_msg=name)


# ---------------------------------------------------------------------------
# Subdivision, occupancy mesh and vertex de-duplication
# ---------------------------------------------------------------------------
@pytest.fixture(scope="module")
def subdivision():
    return goldens.load("subdivision")


@pytest.mark.parametrize("case", goldens.SUBDIVISION_CASES)
def test_oracle_subdivision_matches_reference(subdivision, case):
    g = {k.split("/", 1)[1]: v for k, v in subdivision.items() if k.startswith(case + "/")}
    resolution = tuple(int(x) for x in g["resolution"])
    np.testing.assert_array_equal(oracle.upscale_occupancy(g["occupancy"], resolution), g["upscaled_occupancy"])
    sdf, sh, occ = oracle.upscale_parameters(g["signed_distances"], g["spherical_harmonics"], g["occupancy"],
                                             g["mask"], resolution)
    np.testing.assert_array_equal(occ, g["new_occupancy"])
    np.testing.assert_array_equal(sdf, g["new_signed_distances"])
    np.testing.assert_array_equal(sh, g["new_spherical_harmonics"])
    verts, colors = oracle.get_occupancy_mesh(g["occupancy"], g["mesh_colors_in"])
    np.testing.assert_array_equal(verts, g["mesh_vertices"])
    np.testing.assert_array_equal(colors, g["mesh_colors"])
    np.testing.assert_array_equal(oracle.write_occupancy(g["voxel_indices"], g["occupancy"].shape), g["written"])


@pytest.mark.parametrize("tol", goldens.INDEX_TOLERANCES)
def test_oracle_index_vertices_matches_reference(subdivision, tol):
    key = f"index_{tol:g}"
    np.testing.assert_array_equal(oracle.index_vertices(subdivision[f"{key}/points"], tol), subdivision[f"{key}/index"])


def test_oracle_index_keys_matches_reference(subdivision):
    np.testing.assert_array_equal(oracle.index_keys(subdivision["index_keys/keys"]), subdivision["index_keys/index"])


def test_oracle_index_vertices_groups_like_unstable_reference():
    """With the reference's default (unstable) CPU sort, each group's member
    is arbitrary but the grouping is the same as the oracle's."""
    from oracle import ref

    if not ref.available():
        pytest.skip("reference sources not mounted")
    import torch

    module = ref.python_module("triangle_extraction/index_vertices.py")
    keys = np.random.default_rng(2).integers(-30, 30, size=5000).astype(np.int64)
    got = module.index_keys(torch.from_numpy(keys)).numpy()
    want = oracle.index_keys(keys)
    assert np.array_equal(keys[got], keys)  # every index names an equal key
    assert len(set(zip(got.tolist(), want.tolist()))) == len(np.unique(want)) == len(np.unique(got))
