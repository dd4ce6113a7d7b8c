"""Parity of the timed form of the step with the oracle, at the benchmark sizes.

The benchmark times the fused training step as one CUDA-graph replay
(``graph.CapturedTrainingStep``: capacity-sized buffers, deferred SH,
capacity-mode keys, the tile-bucketed sort, stored hit bits, the MSE epilogue
inside the compositing kernels) at 8x8 tiles. These tests run that captured
step on the benchmark's scenes and compare it stage by stage with the CPU
oracle (the restatement of the reference kernels, pinned to them by the
golden fixtures) fed the same input arrays:

* mid (256^3 band around 8 spheres, SH degree 3, 8 shells, 4 x 800^2):
  vertex and face offsets, faces and voxel indices bit-exact; sorted keys,
  their triangles and the tile ranges bit-exact; the compositing output
  within 1e-5; the loss within 1e-5 relative; the grid SDF / SH gradients
  within 1e-4 of the largest gradient, and within 1e-4 relative on every
  entry whose magnitude is at least 1e-3 of the largest (reference gradient
  routing);
* uneven (the mid scene, 32 cameras of 200-1600 px per side in one ragged
  batch): every camera's compositing output within 1e-5 of the oracle
  rendering that camera alone, and the grid gradients of the batched loss
  against the sum of the per-camera oracle backwards;
* 40 same-size cameras: camera indices 32.. set the fused key's sign bit, so
  signed order puts them first; keys, tile ranges and images against the
  oracle's batched render;
* large (512^3 band around 32 spheres and a background sphere, 16 shells):
  extraction and tessellation bit-exact, one 1297x840 camera in both render
  modes within 1e-5;
* mid, exact gradient mode: grid SDF and SH gradients of the captured step
  against FP64 central finite differences on 64 random corners each
  (relative error <= 1e-3), with the hits and the marching-cubes weights held
  fixed as the adjoint holds them.

Clip decisions at exactly the clip boundary are a discontinuity of the
loss's derivative; where the GPU's and the oracle's composite values straddle
a boundary (within 1e-5 of it), the oracle's upstream gradient takes the
GPU's side, which both readings of the derivative allow.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from meshtryoshka_gb300 import graph, pipeline, synthetic
from meshtryoshka_gb300 import triangle_extraction as te
from meshtryoshka_gb300 import triangle_rasterization as tr
from oracle import oracle
from tests import fp64_model as m

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

IMAGE_ATOL = 1e-5
GRAD_TOL = 1e-4
FD_RTOL = 1e-3
TILE = (8, 8)


def _n(t: torch.Tensor) -> np.ndarray:
    return t.detach().cpu().numpy()


def _host_inputs(w: pipeline.Workload) -> dict:
    v = w.voxels
    return dict(sdf=_n(w.grid_sdf), sh=_n(w.grid_sh), vertices=_n(v.vertices), neighbors=_n(v.neighbors),
                lower=_n(v.lower_corners), upper=_n(v.upper_corners), indices=_n(v.indices), ls=_n(w.level_sets),
                ext=_n(w.extrinsics), intr=_n(w.intrinsics), bg=_n(w.background), target=_n(w.target))


def _tessellate(h: dict) -> oracle.Triangles:
    return oracle.tessellate_voxels(h["sdf"], h["vertices"], h["sh"], h["neighbors"], h["lower"], h["upper"],
                                    h["indices"], h["ls"])


def _render_vertices(tri) -> np.ndarray:
    # 2 v - 1 in float32, as the renderer's stand-in for uncontract() forms it.
    return (np.float32(2.0) * tri.vertices - np.float32(1.0)).astype(np.float32)


def _upstream(raw: np.ndarray, gpu_raw: np.ndarray, bg: np.ndarray, target: np.ndarray, n: int) -> np.ndarray:
    """d loss / d (rgb, T) of loss = sum((clip(rgb + T bg, 0, 1) - target)^2) / n,
    raw [B, 4, H, W] (oracle) -> [B, 4, H, W]."""
    bgc = bg.astype(np.float32)[None, :, None, None]
    x = (raw[:, :3] + raw[:, 3:4] * bgc).astype(np.float32)
    xg = (gpu_raw[:, :3] + gpu_raw[:, 3:4] * bgc).astype(np.float32)
    inside = (x >= 0) & (x <= 1)
    inside_gpu = (xg >= 0) & (xg <= 1)
    near = (np.abs(x) < 1e-5) | (np.abs(x - 1) < 1e-5)
    inside = np.where(near, inside_gpu, inside)
    img = np.clip(x, 0, 1)
    g = np.where(inside, (2.0 / n) * (img - target), 0.0).astype(np.float32)
    out = np.zeros_like(raw)
    out[:, :3] = g
    out[:, 3] = (g * bgc).sum(1)
    return out


def _grid_backward(h, tri, verts, r, tile, image_shape, graw, exact=False):
    b = h["ext"].shape[0]
    s = tri.face_boundaries.shape[0]
    gcol, gsdf_v, _ = oracle.intersect_and_composite_backward(
        r.xy, r.colors, tri.signed_distances, tri.faces, 50.0, r.sorted_keys, r.sorted_tri,
        r.tile_boundaries.reshape(b, -1, 2), s, tile, image_shape, oracle.fused_key_defines(), r.raw, graw,
        exact=exact)
    gsh_v = oracle.evaluate_spherical_harmonics_backward(verts, tri.spherical_harmonics.shape, h["ext"], 3,
                                                         r.colors, gcol)
    _, g_sdf, g_sh = oracle.create_triangle_vertices_backward(h["sdf"], h["sh"].shape, h["lower"], h["ls"],
                                                              tri.vertex_offsets, None, gsdf_v, gsh_v)
    return g_sdf, g_sh


def _assert_grads_close(got: np.ndarray, want: np.ndarray, what: str) -> None:
    scale = float(np.abs(want).max())
    assert scale > 0, what
    err = np.abs(got.astype(np.float64) - want)
    assert float(err.max()) <= GRAD_TOL * scale, f"{what}: max err {err.max():.3e} > {GRAD_TOL} x {scale:.3e}"
    big = np.abs(want) >= 1e-3 * scale
    rel = err[big] / np.abs(want[big])
    assert float(rel.max()) <= GRAD_TOL, f"{what}: per-entry relative error {rel.max():.3e} on {big.sum()} entries"


def _captured(w: pipeline.Workload, gradient_mode=None):
    step = graph.CapturedTrainingStep(w, gradient_mode=gradient_mode, record=True)
    for _ in range(3):
        loss = step()
        torch.cuda.synchronize()
        if step.check():
            break
    assert step.check()
    return step, float(loss)


@pytest.mark.parametrize("config", ["mid", "mid_band"])
def test_captured_mid_step_matches_oracle(cuda_device, config):
    """The timed step (and its band-matched variant, whose 4-voxel band
    gives every one of the 8 shells faces) against the oracle."""
    w = pipeline.build_workload(config, cuda_device)
    w.tile_shape = TILE
    step, loss = _captured(w)
    rec = step.records[0]
    h = _host_inputs(w)

    # Tessellation: bit-exact offsets, faces, voxel indices.
    tri = _tessellate(h)
    f = tri.faces.shape[0]
    np.testing.assert_array_equal(_n(rec["vertex_offsets"]), tri.vertex_offsets)
    np.testing.assert_array_equal(_n(rec["face_offsets"]), tri.face_offsets)
    np.testing.assert_array_equal(_n(rec["faces"])[:f], tri.faces)
    np.testing.assert_array_equal(_n(rec["voxel_indices"])[:f], tri.voxel_indices)
    np.testing.assert_array_equal(_n(rec["face_boundaries"]), tri.face_boundaries)

    # Keys, their triangles and the tile ranges: bit-exact.
    verts = _render_vertices(tri)
    r = oracle.render_fused(h["ext"], h["intr"], w.image_shape, verts, tri.faces, tri.face_boundaries,
                            tri.signed_distances, tri.spherical_harmonics, 3, 50.0, h["bg"], tile_shape=TILE)
    k = r.sorted_keys.shape[0]
    assert int(rec["key_count"]) == k
    np.testing.assert_array_equal(_n(rec["sorted_keys"])[:k], r.sorted_keys)
    np.testing.assert_array_equal(_n(rec["sorted_triangles"])[:k], r.sorted_tri)
    np.testing.assert_array_equal(_n(rec["tile_boundaries"]).reshape(-1, 2), r.tile_boundaries.reshape(-1, 2))

    # Compositing output and loss.
    gpu_raw = _n(rec["composite"])
    assert float(np.abs(gpu_raw - r.raw).max()) <= IMAGE_ATOL
    n = h["target"].size
    want_loss = float(((r.image.astype(np.float64) - h["target"]) ** 2).sum() / n)
    assert abs(loss - want_loss) <= 1e-5 * want_loss

    # Grid gradients through the whole chain.
    graw = _upstream(r.raw, gpu_raw, h["bg"], h["target"], n)
    g_sdf, g_sh = _grid_backward(h, tri, verts, r, TILE, w.image_shape, graw)
    _assert_grads_close(_n(w.grid_sdf.grad), g_sdf, "grid sdf")
    _assert_grads_close(_n(w.grid_sh.grad), g_sh, "grid sh")


def test_captured_uneven_cameras_match_oracle_per_camera(cuda_device):
    w = pipeline.build_workload("uneven", cuda_device)
    w.tile_shape = TILE
    step, loss = _captured(w)
    rec = step.records[0]
    h = _host_inputs(w)
    tri = _tessellate(h)
    verts = _render_vertices(tri)
    raws = [_n(x) for x in tr.split_cameras(rec["composite"], tr.TileGrid.for_cameras(TILE, w.image_shapes, 8))]
    targets = [_n(t) for t in w.targets()]
    n = 3 * w.num_pixels
    g_sdf = np.zeros(h["sdf"].shape, np.float64)
    g_sh = np.zeros(h["sh"].shape, np.float64)
    total = 0.0
    for b, (shape, gpu_raw, target) in enumerate(zip(w.image_shapes, raws, targets)):
        cam = dict(h, ext=h["ext"][b:b + 1], intr=h["intr"][b:b + 1])
        r = oracle.render_fused(cam["ext"], cam["intr"], shape, verts, tri.faces, tri.face_boundaries,
                                tri.signed_distances, tri.spherical_harmonics, 3, 50.0, h["bg"], tile_shape=TILE)
        err = float(np.abs(gpu_raw - r.raw[0]).max())
        assert err <= IMAGE_ATOL, f"camera {b} {shape}: {err:.3e}"
        total += float(((r.image[0].astype(np.float64) - target) ** 2).sum())
        graw = _upstream(r.raw, gpu_raw[None], h["bg"], target[None], n)
        a, c = _grid_backward(cam, tri, verts, r, TILE, shape, graw)
        g_sdf += a
        g_sh += c
    assert abs(loss - total / n) <= 1e-5 * (total / n)
    _assert_grads_close(_n(w.grid_sdf.grad), g_sdf, "grid sdf")
    _assert_grads_close(_n(w.grid_sh.grad), g_sh, "grid sh")


def test_sign_bit_cameras_match_oracle(cuda_device):
    """40 cameras in the 6-bit camera field: cameras 32..39 set bit 63 of the
    fused key, and the reference's signed stable sort puts them first."""
    d = cuda_device
    cfg = synthetic.CONFIGS["small"]
    occ = synthetic.make_occupancy(cfg, "cpu").numpy()
    vox = oracle.extract_voxels(occ)
    sdf = synthetic.corner_sdf(cfg, torch.from_numpy(vox.vertices)).numpy()
    sh = synthetic.corner_sh(cfg, sdf.shape[0]).numpy()
    ls = synthetic.level_sets(cfg).numpy()
    tri = oracle.tessellate_voxels(sdf, vox.vertices, sh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                   vox.indices, ls)
    verts = _render_vertices(tri)
    rng = np.random.default_rng(40)
    eyes = rng.normal(0, 1, (40, 3))
    eyes = 2.2 * eyes / np.linalg.norm(eyes, axis=1, keepdims=True)
    ext = np.stack([synthetic.look_at(e) for e in eyes]).astype(np.float32)
    intr = np.stack([synthetic.pinhole(48, 40, 60.0)] * 40).astype(np.float32)
    bg = np.array([0.1, 0.2, 0.3], np.float32)
    r = oracle.render_fused(ext, intr, (48, 40), verts, tri.faces, tri.face_boundaries, tri.signed_distances,
                            tri.spherical_harmonics, 0, 50.0, bg)
    assert (r.sorted_keys < 0).any()  # the sign bit is in use
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(d)  # noqa: E731
    store: dict = {}
    from meshtryoshka_gb300.record import recording

    with recording(store):
        image = tr.render_fused(t(ext), t(intr), (48, 40), t(verts), t(tri.faces), t(tri.face_boundaries),
                                t(tri.signed_distances), t(tri.spherical_harmonics), 0, 50.0, t(bg))
    np.testing.assert_array_equal(_n(store["sorted_keys"]), r.sorted_keys)
    np.testing.assert_array_equal(_n(store["sorted_triangles"]), r.sorted_tri)
    np.testing.assert_array_equal(_n(store["tile_boundaries"]).reshape(-1, 2), r.tile_boundaries.reshape(-1, 2))
    assert float(np.abs(_n(image) - r.image).max()) <= IMAGE_ATOL


def test_large_extraction_and_one_camera_in_both_modes(cuda_device):
    d = cuda_device
    cfg = synthetic.CONFIGS["large"]
    occ = synthetic.make_occupancy(cfg, "cpu")
    vox = te.extract_voxels(occ.to(d))
    want = oracle.extract_voxels(occ.numpy())
    for got, exp in zip((vox.vertices, vox.neighbors, vox.lower_corners, vox.upper_corners, vox.indices),
                        (want.vertices, want.neighbors, want.lower_corners, want.upper_corners, want.indices)):
        np.testing.assert_array_equal(_n(got), exp)
    sdf = synthetic.corner_sdf(cfg, vox.vertices)
    sh = synthetic.corner_sh(cfg, vox.num_vertices, d)
    ls = synthetic.level_sets(cfg, d)
    with torch.no_grad():
        tri = te.tessellate_voxels(sdf, vox.vertices, sh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                   vox.indices, ls)
    otri = oracle.tessellate_voxels(_n(sdf), want.vertices, _n(sh), want.neighbors, want.lower_corners,
                                    want.upper_corners, want.indices, _n(ls))
    np.testing.assert_array_equal(_n(tri.faces), otri.faces)
    np.testing.assert_array_equal(_n(tri.voxel_indices), otri.voxel_indices)
    np.testing.assert_array_equal(_n(tri.vertices), otri.vertices)
    np.testing.assert_array_equal(_n(tri.signed_distances), otri.signed_distances)
    np.testing.assert_array_equal(_n(tri.face_boundaries), otri.face_boundaries)
    del sh
    cams = synthetic.make_cameras(cfg)
    shape = tuple(cams.image_shapes[0])
    ext, intr = cams.extrinsics[:1].astype(np.float32), cams.intrinsics[:1].astype(np.float32)
    bg = np.array([0.2, 0.4, 0.6], np.float32)
    verts = _render_vertices(otri)
    args = (verts, otri.faces, otri.face_boundaries, otri.signed_distances, otri.spherical_harmonics, 3, 50.0, bg)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(d)  # noqa: E731
    with torch.no_grad():
        gpu_args = (pipeline.uncontract_stand_in(tri.vertices), tri.faces, tri.face_boundaries, tri.signed_distances,
                    tri.spherical_harmonics, 3, 50.0, t(bg))
        fused = tr.render(t(ext), t(intr), shape, *gpu_args, mode="fused")
        explicit = tr.render(t(ext), t(intr), shape, *gpu_args, mode="explicit")
    want_fused = oracle.render_fused(ext, intr, shape, *args).image
    assert float(np.abs(_n(fused) - want_fused).max()) <= IMAGE_ATOL
    want_explicit = oracle.render_explicit(ext, intr, shape, *args)
    assert float(np.abs(_n(explicit) - want_explicit).max()) <= IMAGE_ATOL


def test_captured_mid_step_exact_gradients_match_fd64(cuda_device):
    """FP64 central differences of the loss on 64 random grid corners (SDF)
    and 64 random grid SH entries, with the hits, barycentrics and
    marching-cubes weights held fixed. Only the pixels whose hits use a
    vertex of the perturbed corner change, so each difference is evaluated
    on those pixels."""
    w = pipeline.build_workload("mid", cuda_device)
    w.tile_shape = TILE
    step, _ = _captured(w, gradient_mode="exact")
    g_sdf_gpu, g_sh_gpu = _n(w.grid_sdf.grad), _n(w.grid_sh.grad)
    h = _host_inputs(w)
    tri = _tessellate(h)
    verts = _render_vertices(tri)
    b = h["ext"].shape[0]
    s = tri.face_boundaries.shape[0]
    hh, ww = w.image_shape
    r = oracle.render_fused(h["ext"], h["intr"], w.image_shape, verts, tri.faces, tri.face_boundaries,
                            tri.signed_distances, tri.spherical_harmonics, 3, 50.0, h["bg"])
    hf, huvw = oracle.fused_hits(r.xy, tri.faces, r.sorted_keys, r.sorted_tri, r.tile_boundaries.reshape(b, -1, 2),
                                 s, (16, 16), w.image_shape, oracle.fused_key_defines())
    hf, huvw = hf.reshape(b, -1, s), huvw.reshape(b, -1, s, 3)
    v = tri.vertices.shape[0]
    i0, i1, tw = oracle.triangle_vertex_sources(h["sdf"], h["lower"], h["ls"], tri.vertex_offsets, v)
    sdf64, sh64 = h["sdf"].astype(np.float64), h["sh"].astype(np.float64)
    target = h["target"].reshape(b, 3, -1).astype(np.float64)
    bg = h["bg"].astype(np.float64)
    n = h["target"].size

    def pixel_loss(pixels, vsdf, colors):
        # sum over the listed pixels [(camera, pixel index)] of the squared
        # clipped error, / n.
        total = 0.0
        for cam in range(b):
            p = pixels[cam]
            if p.size == 0:
                continue
            rgb, trans = m.composite_hits(tri.faces, hf[cam:cam + 1, p], huvw[cam:cam + 1, p], colors[cam:cam + 1],
                                          vsdf, 50.0)
            img = np.clip(rgb[0] + trans[0][:, None] * bg, 0.0, 1.0)
            total += float(((img - target[cam][:, p].T) ** 2).sum())
        return total / n

    def affected(corner):
        vmask = (i0 == corner) | (i1 == corner)
        fmask = vmask[tri.faces].any(axis=1)
        hit = np.where(hf >= 0, fmask[np.maximum(hf, 0)], False).any(axis=2)  # [B, P]
        return [np.nonzero(hit[cam])[0] for cam in range(b)], np.nonzero(vmask)[0]

    def vertex_values(sdf_grid, sh_grid, vids):
        vs = m.lerp_vertices(sdf_grid, i0[vids], i1[vids], tw[vids])
        vsh = m.lerp_vertices(sh_grid.transpose(1, 0, 2), i0[vids], i1[vids], tw[vids]).transpose(1, 0, 2)
        return vs, m.sh_colors(verts[vids], vsh, h["ext"], 3)

    # Every vertex's values in FP64 once; each perturbation recomputes only
    # the vertices of the perturbed corner.
    all_v = np.arange(v)
    base_sdf, base_col = vertex_values(sdf64, sh64, all_v)

    def fd(grid, index, pixels, vids):
        keep_sdf, keep_col = base_sdf[vids].copy(), base_col[:, vids].copy()

        def loss():
            base_sdf[vids], base_col[:, vids] = vertex_values(sdf64, sh64, vids)
            return pixel_loss(pixels, base_sdf, base_col)

        value = m.central_difference(loss, grid, index, 1e-6)
        base_sdf[vids], base_col[:, vids] = keep_sdf, keep_col
        return value

    rng = np.random.default_rng(64)
    hit_vertices = np.unique(tri.faces[hf[hf >= 0]].reshape(-1))
    corners = np.unique(np.concatenate([i0[hit_vertices], i1[hit_vertices]]))
    got_sdf, want_sdf, got_sh, want_sh = [], [], [], []
    for c in rng.choice(corners, 64, replace=False):
        pixels, vids = affected(int(c))
        want_sdf.append(fd(sdf64, (int(c),), pixels, vids))
        got_sdf.append(g_sdf_gpu[int(c)])
    for c in rng.choice(corners, 64, replace=False):
        pixels, vids = affected(int(c))
        k, ch = int(rng.integers(0, 16)), int(rng.integers(0, 3))
        want_sh.append(fd(sh64, (k, int(c), ch), pixels, vids))
        got_sh.append(g_sh_gpu[k, int(c), ch])
    for got, want, what in ((got_sdf, want_sdf, "sdf"), (got_sh, want_sh, "sh")):
        got, want = np.asarray(got, np.float64), np.asarray(want, np.float64)
        assert np.linalg.norm(want) > 0
        rel = float(np.linalg.norm(got - want) / np.linalg.norm(want))
        assert rel <= FD_RTOL, f"{what}: relative error {rel:.3e}"
