"""Adjoints against FP64 central finite differences (relative error <= 1e-3).

Finite differences are taken on the FP64 model in tests/fp64_model.py with
the geometry held fixed exactly where the reference's adjoint holds it fixed
(vertex positions are not differentiated, the marching-cubes weight t is
detached), so in the exact gradient mode the adjoint must equal the
derivative of that function:

* compositor level: d loss / d (per-vertex colours, per-vertex signed
  distances, sharpness) for the fused walk and for the explicit chain
  (intersect -> interpolate -> composite), from the CPU oracle's adjoint and
  from the GPU kernels;
* whole chain on the GPU: grid signed distances and grid SH coefficients
  (degree 3) -> tessellation -> SH evaluation -> fused render with the
  background blend and clip -> loss.

The loss is <image, G> for a fixed random G. The relative error is
||g - fd|| / ||fd|| over randomly chosen entries that the hits touch.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import oracle
from tests import fp64_model as m
from tests import semantics
from tests.scenes import SCENES, make_scene

FD_RTOL = 1e-3
STEP = 1e-6
N_ENTRIES = 24


def _rel(g, fd):
    g, fd = np.asarray(g, np.float64), np.asarray(fd, np.float64)
    return float(np.linalg.norm(g - fd) / max(np.linalg.norm(fd), 1e-30))


class FusedCase:
    """A fixed-geometry fused render of a test scene: hits, weights, target."""

    def __init__(self, name: str, seed: int = 0):
        sc = self.scene = make_scene(**SCENES[name])
        self.b = sc.extrinsics.shape[0]
        self.s = sc.face_boundaries.shape[0]
        self.h, self.w = sc.image_shape
        self.kd = oracle.fused_key_defines()
        r = self.render = oracle.render_fused(sc.extrinsics, sc.intrinsics, sc.image_shape, sc.vertices, sc.faces,
                                              sc.face_boundaries, sc.sdf, sc.sh, sc.sh_degree, sc.sharpness,
                                              sc.background)
        self.tb = r.tile_boundaries.reshape(self.b, -1, 2)
        hf, huvw = oracle.fused_hits(r.xy, sc.faces, r.sorted_keys, r.sorted_tri, self.tb, self.s, (16, 16),
                                     sc.image_shape, self.kd)
        self.hit_faces = hf.reshape(self.b, -1, self.s)
        self.hit_uvw = huvw.reshape(self.b, -1, self.s, 3)
        rng = np.random.default_rng(seed)
        self.target = rng.normal(0, 1, (self.b, 4, self.h, self.w)).astype(np.float32)
        self.colors64 = r.colors.astype(np.float64)
        self.sdf64 = sc.sdf.astype(np.float64)
        self.sharp64 = np.array([float(sc.sharpness)])
        hit = self.hit_faces >= 0
        self.touched = np.unique(sc.faces[self.hit_faces[hit]].reshape(-1))
        self.rng = rng

    def loss64(self) -> float:
        rgb, t = m.composite_hits(self.scene.faces, self.hit_faces, self.hit_uvw, self.colors64, self.sdf64,
                                  float(self.sharp64[0]))
        g = self.target.reshape(self.b, 4, -1).astype(np.float64)
        return float((rgb * g[:, :3].transpose(0, 2, 1)).sum() + (t * g[:, 3]).sum())

    def entries(self):
        cams = self.rng.integers(0, self.b, N_ENTRIES)
        verts = self.rng.choice(self.touched, N_ENTRIES)
        chans = self.rng.integers(0, 3, N_ENTRIES)
        col_idx = list(zip(cams, verts, chans))
        sdf_idx = [(int(v),) for v in self.rng.choice(self.touched, N_ENTRIES, replace=False)]
        return col_idx, sdf_idx

    def check(self, grad_colors, grad_sdf, grad_sharpness):
        col_idx, sdf_idx = self.entries()
        fd_c = [m.central_difference(self.loss64, self.colors64, i, STEP) for i in col_idx]
        fd_d = [m.central_difference(self.loss64, self.sdf64, i, STEP) for i in sdf_idx]
        fd_s = m.central_difference(self.loss64, self.sharp64, (0,), STEP)
        assert np.linalg.norm(fd_d) > 0 and np.linalg.norm(fd_c) > 0
        assert _rel([grad_colors[i] for i in col_idx], fd_c) <= FD_RTOL
        assert _rel([grad_sdf[i] for i in sdf_idx], fd_d) <= FD_RTOL
        assert _rel([grad_sharpness], [fd_s]) <= FD_RTOL


@pytest.mark.parametrize("name", ["front_128", "three_cams_odd"])
def test_fp64_model_matches_oracle_forward(name):
    c = FusedCase(name)
    rgb, t = m.composite_hits(c.scene.faces, c.hit_faces, c.hit_uvw, c.colors64, c.sdf64, float(c.sharp64[0]))
    raw = c.render.raw.reshape(c.b, 4, -1)
    assert np.abs(rgb - raw[:, :3].transpose(0, 2, 1)).max() < 1e-5
    assert np.abs(t - raw[:, 3]).max() < 1e-5


@pytest.mark.parametrize("name", ["front_128", "three_cams_odd"])
def test_oracle_fused_adjoint_matches_fd(name):
    c = FusedCase(name)
    sc, r = c.scene, c.render
    gcol, gsdf, gsharp = oracle.intersect_and_composite_backward(
        r.xy, r.colors, sc.sdf, sc.faces, sc.sharpness, r.sorted_keys, r.sorted_tri, c.tb, c.s, (16, 16),
        sc.image_shape, c.kd, r.raw, c.target, exact=True)
    c.check(gcol, gsdf, gsharp)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["front_128", "three_cams_odd"])
def test_gpu_fused_adjoint_matches_fd(cuda_device, name):
    import torch

    from meshtryoshka_gb300 import triangle_rasterization as tr

    c = FusedCase(name)
    sc, r, d = c.scene, c.render, cuda_device
    grid = tr.TileGrid((16, 16), sc.image_shape, c.b, c.s)
    kd = tr.create_key_defines(("camera", 6), ("tile", 20), ("depth", 32), ("shell", 6))
    colors = torch.from_numpy(r.colors).to(d).requires_grad_(True)
    sdf = torch.from_numpy(sc.sdf).to(d).requires_grad_(True)
    sharp = torch.tensor(float(sc.sharpness), device=d, requires_grad=True)
    out = tr.intersect_and_composite(torch.from_numpy(r.xy).to(d), colors, sdf, torch.from_numpy(sc.faces).to(d),
                                     sharp, torch.from_numpy(r.sorted_keys).to(d),
                                     torch.from_numpy(r.sorted_tri).to(d), torch.from_numpy(c.tb).to(d), c.s, grid,
                                     kd, gradient_mode="exact")
    (out * torch.from_numpy(c.target).to(d)).sum().backward()
    c.check(colors.grad.cpu().numpy(), sdf.grad.cpu().numpy(), float(sharp.grad))


class ExplicitCase(FusedCase):
    """Fixed first hits per shell; the explicit chain's loss is <rgb, G_rgb> + <T, G_T>."""

    def __init__(self, name: str, seed: int = 1):
        super().__init__(name, seed)
        sc = self.scene
        kd = oracle.explicit_key_defines()
        xy, depth = oracle.project_vertices(sc.vertices, sc.extrinsics, sc.intrinsics)
        rows, cols = -(-self.h // 16), -(-self.w // 16)
        tmin, tmax, count = oracle.bound_triangles(xy, depth, sc.faces, (16, 16), (rows, cols), 0.2)
        keys, tri = oracle.generate_keys(depth, sc.faces, sc.face_boundaries, tmin, tmax, count, cols, kd)
        sk, st = oracle.sort_pairs(keys, tri)
        tb = oracle.delineate_tiles(sk, kd, True, self.b, self.s, rows * cols)
        uv, index = oracle.intersect(xy, sc.faces, st, tb, self.s, (16, 16), sc.image_shape)
        self.uv, self.index = uv, index
        u, v = uv[..., 0], uv[..., 1]
        w = (np.float32(1.0) - u) - v  # as the interpolation kernel forms it, in float32
        # [B, S, H, W] -> [B, P, S] hit slots in shell order
        self.hit_faces = index.transpose(0, 2, 3, 1).reshape(self.b, -1, self.s)
        self.hit_uvw = np.stack([u, v, w], -1).transpose(0, 2, 3, 1, 4).reshape(self.b, -1, self.s, 3)
        hit = self.hit_faces >= 0
        self.touched = np.unique(sc.faces[self.hit_faces[hit]].reshape(-1))


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["front_128", "three_cams_odd"])
def test_gpu_explicit_adjoint_matches_fd(cuda_device, name):
    import torch

    from meshtryoshka_gb300 import triangle_rasterization as tr

    c = ExplicitCase(name)
    sc, d = c.scene, cuda_device
    colors = torch.from_numpy(c.render.colors).to(d).requires_grad_(True)
    sdf = torch.from_numpy(sc.sdf).to(d).requires_grad_(True)
    sharp = torch.tensor(float(sc.sharpness), device=d, requires_grad=True)
    uv, index = torch.from_numpy(c.uv).to(d), torch.from_numpy(c.index).to(d)
    isdf, icol = tr.interpolate(uv, index, torch.from_numpy(sc.faces).to(d), sdf, colors)
    b, s, h, w = isdf.shape
    psdf = isdf.permute(0, 2, 3, 1).reshape(b * h * w, s).contiguous()
    pcol = icol.permute(0, 2, 3, 1, 4).reshape(b * h * w, s, 3).contiguous()
    mask = (index != -1).permute(0, 2, 3, 1).reshape(b * h * w, s).contiguous()
    out_c, out_t = tr.Composite.apply(psdf, pcol, mask, sharp, "exact")
    g = torch.from_numpy(c.target).to(d).reshape(b, 4, h * w)
    loss = (out_c.reshape(b, h * w, 3) * g[:, :3].transpose(1, 2)).sum() + (out_t.reshape(b, h * w) * g[:, 3]).sum()
    loss.backward()
    c.check(colors.grad.cpu().numpy(), sdf.grad.cpu().numpy(), float(sharp.grad))


@pytest.mark.gpu
def test_gpu_grid_chain_matches_fd(cuda_device):
    """Grid SDF / SH (degree 3) -> tessellate -> SH -> fused render -> loss."""
    import torch

    from meshtryoshka_gb300 import triangle_extraction as te
    from meshtryoshka_gb300 import triangle_rasterization as tr
    from meshtryoshka_gb300 import synthetic

    d = cuda_device
    rng = np.random.default_rng(7)
    n = 32
    coords = -1 + (np.arange(n) + 0.5) * 2 / n
    z, y, x = np.meshgrid(coords, coords, coords, indexing="ij")
    occ = semantics.pack(np.abs(np.sqrt(x * x + y * y + z * z) - 0.5) < 2.5 * 2 / n)
    vox = oracle.extract_voxels(occ)
    p = 2 * vox.vertices.astype(np.float64) - 1
    gsdf = (np.linalg.norm(p, axis=1) - 0.5 + rng.normal(0, 0.002, len(p))).astype(np.float32)
    gsh = np.concatenate([rng.uniform(0, 1, (1, len(p), 3)), rng.normal(0, 0.1, (15, len(p), 3))]).astype(np.float32)
    ls = np.array([0.03, 0.01, -0.01, -0.03], np.float32)
    image_shape = (96, 96)
    ext = np.stack([synthetic.look_at(np.array(c)) for c in ((0.0, 0.0, 2.0), (1.2, 0.8, 1.3))]).astype(np.float32)
    intr = np.stack([synthetic.pinhole(96, 96, 55.0)] * 2).astype(np.float32)
    bg = np.array([0.2, 0.4, 0.6], np.float32)
    sharpness = 50.0
    target = rng.normal(0, 1, (2, 3) + image_shape).astype(np.float32)

    # GPU: the product path with autograd.
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(d)  # noqa: E731
    sdf_d = t(gsdf).requires_grad_(True)
    sh_d = t(gsh).requires_grad_(True)
    tri = te.tessellate_voxels(sdf_d, t(vox.vertices), sh_d, t(vox.neighbors), t(vox.lower_corners),
                               t(vox.upper_corners), t(vox.indices), t(ls))
    verts = 2.0 * tri.vertices - 1.0
    image = tr.render_fused(t(ext), t(intr), image_shape, verts, tri.faces, tri.face_boundaries, tri.signed_distances,
                            tri.spherical_harmonics, 3, sharpness, t(bg), gradient_mode="exact")
    (image * t(target)).sum().backward()
    g_sdf, g_sh = sdf_d.grad.cpu().numpy(), sh_d.grad.cpu().numpy()

    # FP64 model with the same fixed geometry.
    otri = oracle.tessellate_voxels(gsdf, vox.vertices, gsh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                    vox.indices, ls)
    i0, i1, tw = oracle.triangle_vertex_sources(gsdf, vox.lower_corners, ls, otri.vertex_offsets,
                                                otri.vertices.shape[0])
    vertices = (np.float32(2.0) * otri.vertices - np.float32(1.0)).astype(np.float32)
    np.testing.assert_array_equal(verts.detach().cpu().numpy(), vertices)
    s = ls.shape[0]
    r = oracle.render_fused(ext, intr, image_shape, vertices, otri.faces, otri.face_boundaries,
                            otri.signed_distances, otri.spherical_harmonics, 3, sharpness, bg)
    hf, huvw = oracle.fused_hits(r.xy, otri.faces, r.sorted_keys, r.sorted_tri, r.tile_boundaries.reshape(2, -1, 2),
                                 s, (16, 16), image_shape, oracle.fused_key_defines())
    hf, huvw = hf.reshape(2, -1, s), huvw.reshape(2, -1, s, 3)
    gsdf64, gsh64 = gsdf.astype(np.float64), gsh.astype(np.float64)
    g64 = target.reshape(2, 3, -1).astype(np.float64)

    def loss64():
        vsdf = m.lerp_vertices(gsdf64, i0, i1, tw)
        vsh = m.lerp_vertices(gsh64.transpose(1, 0, 2), i0, i1, tw).transpose(1, 0, 2)
        colors = m.sh_colors(vertices, vsh, ext, 3)
        rgb, trans = m.composite_hits(otri.faces, hf, huvw, colors, vsdf, sharpness)
        img = np.clip(rgb + trans[..., None] * bg, 0.0, 1.0)  # [B, P, 3]
        return float((img * g64.transpose(0, 2, 1)).sum())

    hit_vertices = np.unique(otri.faces[hf[hf >= 0]].reshape(-1))
    corners = np.unique(np.concatenate([i0[hit_vertices], i1[hit_vertices]]))
    sdf_idx = [(int(c),) for c in rng.choice(corners, N_ENTRIES, replace=False)]
    sh_idx = [(int(k), int(c), int(ch)) for k, c, ch in
              zip(rng.integers(0, 16, N_ENTRIES), rng.choice(corners, N_ENTRIES), rng.integers(0, 3, N_ENTRIES))]
    fd_sdf = [m.central_difference(loss64, gsdf64, i, STEP) for i in sdf_idx]
    fd_sh = [m.central_difference(loss64, gsh64, i, STEP) for i in sh_idx]
    assert np.linalg.norm(fd_sdf) > 0 and np.linalg.norm(fd_sh) > 0
    assert _rel([g_sdf[i] for i in sdf_idx], fd_sdf) <= FD_RTOL
    assert _rel([g_sh[i] for i in sh_idx], fd_sh) <= FD_RTOL


def test_oracle_sdf_regularizers_adjoint_matches_fd():
    """The hand-derived adjoint of the SDF regularizers (the reference
    differentiates them automatically) against FP64 central differences."""
    rng = np.random.default_rng(21)
    n = 32
    coords = -1 + (np.arange(n) + 0.5) * 2 / n
    z, y, x = np.meshgrid(coords, coords, coords, indexing="ij")
    occ = semantics.pack(np.abs(np.sqrt(x * x + y * y + z * z) - 0.5) < 2.5 * 2 / n)
    vox = oracle.extract_voxels(occ)
    p = 2 * vox.vertices.astype(np.float64) - 1
    sdf = (0.5 * (np.linalg.norm(p, axis=1) - 0.5) + rng.normal(0, 0.003, len(p))).astype(np.float32)
    grid_size = (n, n, n)
    nv = vox.upper_corners.shape[1]
    gp, gn, gc = (rng.normal(0, 1, nv).astype(np.float32) for _ in range(3))
    grad = oracle.compute_sdf_regularizers_backward(sdf, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                                    grid_size, gp, gn, gc)
    sdf64 = sdf.astype(np.float64)

    def loss64():
        pos, neg, curv = m.sdf_regularizers(sdf64, vox.neighbors, vox.lower_corners, vox.upper_corners, grid_size)
        return float((pos * gp).sum() + (neg * gn).sum() + (curv * gc).sum())

    pos, neg, curv = oracle.compute_sdf_regularizers(sdf, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                                     grid_size)
    p64, n64, c64 = m.sdf_regularizers(sdf64, vox.neighbors, vox.lower_corners, vox.upper_corners, grid_size)
    assert np.abs(pos - p64).max() < 1e-4 and np.abs(neg - n64).max() < 1e-4 and np.abs(curv - c64).max() < 1e-6
    idx = [(int(i),) for i in rng.choice(np.unique(vox.lower_corners[0]), N_ENTRIES, replace=False)]
    fd = [m.central_difference(loss64, sdf64, i, STEP) for i in idx]
    assert np.linalg.norm(fd) > 0
    assert _rel([grad[i] for i in idx], fd) <= FD_RTOL


@pytest.mark.gpu
def test_gpu_live_t_vertex_gradients_match_fd(cuda_device):
    """t_gradient="live": the marching-cubes weight t = (iso - d0) / (d1 - d0)
    is differentiated as a function of the edge's two corner SDFs (topology
    held fixed). Loss = <vertices, Gp> + <sdf, Gs> + <sh, Gsh> of the
    tessellation; its gradients with respect to the grid SDF, SH and
    positions against FP64 central differences (relative error <= 1e-3), on
    corners whose vertices all sit strictly inside their edges. The default
    mode stays the reference's (detached t) on the same inputs."""
    import torch

    from meshtryoshka_gb300 import triangle_extraction as te

    d = cuda_device
    rng = np.random.default_rng(11)
    n = 32
    coords = -1 + (np.arange(n) + 0.5) * 2 / n
    z, y, x = np.meshgrid(coords, coords, coords, indexing="ij")
    occ = semantics.pack(np.abs(np.sqrt(x * x + y * y + z * z) - 0.5) < 2.5 * 2 / n)
    vox = oracle.extract_voxels(occ)
    p = 2 * vox.vertices.astype(np.float64) - 1
    gsdf = (np.linalg.norm(p, axis=1) - 0.5 + rng.normal(0, 0.002, len(p))).astype(np.float32)
    gsh = np.concatenate([rng.uniform(0, 1, (1, len(p), 3)), rng.normal(0, 0.1, (3, len(p), 3))]).astype(np.float32)
    ls = np.array([0.02, 0.0, -0.02], np.float32)
    otri = oracle.tessellate_voxels(gsdf, vox.vertices, gsh, vox.neighbors, vox.lower_corners, vox.upper_corners,
                                    vox.indices, ls)
    v = otri.vertices.shape[0]
    gp = rng.normal(0, 1, (v, 3)).astype(np.float32)
    gs = rng.normal(0, 1, (v,)).astype(np.float32)
    gh = rng.normal(0, 1, (4, v, 3)).astype(np.float32)

    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(d)  # noqa: E731
    grads = {}
    for mode in ("live", "detached"):
        sdf_d = t(gsdf).requires_grad_(True)
        sh_d = t(gsh).requires_grad_(True)
        pos_d = t(vox.vertices).requires_grad_(True)
        tri = te.tessellate_voxels(sdf_d, pos_d, sh_d, t(vox.neighbors), t(vox.lower_corners),
                                   t(vox.upper_corners), t(vox.indices), t(ls), t_gradient=mode)
        loss = (tri.vertices * t(gp)).sum() + (tri.signed_distances * t(gs)).sum() + \
            (tri.spherical_harmonics * t(gh)).sum()
        loss.backward()
        grads[mode] = (sdf_d.grad.cpu().numpy(), sh_d.grad.cpu().numpy(), pos_d.grad.cpu().numpy())

    # Detached mode: the reference's adjoint (the oracle's restatement).
    want_pos, want_sdf, want_sh = oracle.create_triangle_vertices_backward(
        gsdf, gsh.shape, vox.lower_corners, ls, otri.vertex_offsets, gp, gs, gh)
    for got, want in zip(grads["detached"], (want_sdf, want_sh, want_pos)):
        assert np.abs(got - want).max() <= 1e-5 * max(np.abs(want).max(), 1e-30)

    # FP64 model with t live.
    i0, i1, tw = oracle.triangle_vertex_sources(gsdf, vox.lower_corners, ls, otri.vertex_offsets, v)
    shell = np.searchsorted(otri.vertex_boundaries, np.arange(v), side="right")
    iso = ls.astype(np.float64)[shell]
    sdf64, sh64, pos64 = gsdf.astype(np.float64), gsh.astype(np.float64), vox.vertices.astype(np.float64)

    def loss64():
        d0, d1 = sdf64[i0], sdf64[i1]
        tt = np.clip((iso - d0) / (d1 - d0), 0.0, 1.0)
        verts = pos64[i0] + tt[:, None] * (pos64[i1] - pos64[i0])
        vsdf = d0 + tt * (d1 - d0)
        vsh = sh64[:, i0] + tt[None, :, None] * (sh64[:, i1] - sh64[:, i0])
        return float((verts * gp).sum() + (vsdf * gs).sum() + (vsh * gh).sum())

    inside = (tw > 1e-3) & (tw < 1 - 1e-3) & (gsdf[i0] != gsdf[i1])
    bad = np.zeros(len(gsdf), bool)
    bad[i0[~inside]] = True
    bad[i1[~inside]] = True
    used = np.zeros(len(gsdf), bool)
    used[i0] = True
    used[i1] = True
    corners = np.nonzero(used & ~bad)[0]
    sdf_idx = [(int(c),) for c in rng.choice(corners, N_ENTRIES, replace=False)]
    sh_idx = [(int(k), int(c), int(ch)) for k, c, ch in
              zip(rng.integers(0, 4, N_ENTRIES), rng.choice(corners, N_ENTRIES), rng.integers(0, 3, N_ENTRIES))]
    pos_idx = [(int(c), int(ch)) for c, ch in zip(rng.choice(corners, N_ENTRIES), rng.integers(0, 3, N_ENTRIES))]
    g_sdf, g_sh, g_pos = grads["live"]
    for grid, idx, got in ((sdf64, sdf_idx, g_sdf), (sh64, sh_idx, g_sh), (pos64, pos_idx, g_pos)):
        fd = [m.central_difference(loss64, grid, i, STEP) for i in idx]
        assert np.linalg.norm(fd) > 0
        assert _rel([got[i] for i in idx], fd) <= FD_RTOL
    # The live weight changes the SDF gradient (and nothing else).
    assert _rel(g_sdf[[i[0] for i in sdf_idx]], want_sdf[[i[0] for i in sdf_idx]]) > 1e-2
    np.testing.assert_allclose(g_sh, want_sh, rtol=0, atol=1e-5 * np.abs(want_sh).max())
