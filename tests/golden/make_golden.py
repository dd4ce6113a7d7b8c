"""Generate the golden fixtures in this folder from the reference's own kernels.

Every output array is computed by the reference implementation's compute
kernels (its Slang sources, rewritten textually to C++ and compiled on the
host by ``oracle/build_ref.py``; see ``oracle/ref.py``). Gradients come from
the reference's two hand-written backward kernels (fused intersect-and-composite
and explicit composite), whose calls to automatically differentiated helpers
use hand-derived adjoints (``oracle/ref_shim/autodiff_*.h``). The glue between
kernels follows the reference's Python call sites:

* exclusive scans are numpy cumsums (triangle_extraction/__init__.py uses
  torch.cumsum),
* key sorting is a stable sort of the int64 keys (sort_keys.cu uses cub's
  stable radix sort over all 64 bits),
* camera centres are inverse(extrinsics)[:, :3, 3] in float64, rounded to
  float32 (evaluate_spherical_harmonics.py:38).

Inputs are seeded synthetic scenes: occupancy grids, a sphere band with a
noisy signed distance field, cameras looking at the origin.

Run from the repository root with the reference tree mounted:

    python tests/golden/make_golden.py [--reference PATH]

The output is deterministic; tests/test_golden_cpu.py regenerates it in
memory when the reference is present and checks it matches the committed
files.
"""

from __future__ import annotations

import argparse
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

NEAR_PLANE = 0.2
TILE = (16, 16)  # the reference's compiled tile shape


def _pack(bits: np.ndarray) -> np.ndarray:
    from tests import semantics

    return semantics.pack(bits)


def _sphere_band(n: int, radius: float = 0.5, width: float = 2.5) -> np.ndarray:
    c = -1 + (np.arange(n) + 0.5) * 2 / n
    z, y, x = np.meshgrid(c, c, c, indexing="ij")
    d = np.sqrt(x * x + y * y + z * z) - radius
    return _pack(np.abs(d) < width * 2 / n)


def _look_at(eye) -> np.ndarray:
    from meshtryoshka_gb300 import synthetic

    return synthetic.look_at(np.asarray(eye, np.float64))


def _pinhole(h, w, fov) -> np.ndarray:
    from meshtryoshka_gb300 import synthetic

    return synthetic.pinhole(h, w, fov)


# ---------------------------------------------------------------------------
# Extraction: voxels, dilation, tessellation
# ---------------------------------------------------------------------------
def extraction_fixture(ref) -> dict[str, np.ndarray]:
    rng = np.random.default_rng(3)
    out: dict[str, np.ndarray] = {}
    grids = {
        "random": _pack(rng.random((6, 5, 96)) < 0.3),
        "sphere": _sphere_band(32),
        "edges": _pack((np.arange(64)[None, None, :] % 32 >= 30) & (rng.random((3, 4, 64)) < 0.7)),
    }
    for name, occ in grids.items():
        vox = ref.extract_voxels(occ)
        out[f"{name}/occupancy"] = occ
        for field in ("vertices", "neighbors", "lower_corners", "upper_corners", "indices", "vertex_occupancy",
                      "vertex_counts", "voxel_counts"):
            out[f"{name}/{field}"] = vox[field]
        for d in (1, 3):
            out[f"{name}/dilated_{d}"] = ref.dilate_occupancy(occ, d)

    vox = ref.extract_voxels(grids["sphere"])
    p = 2 * vox["vertices"].astype(np.float64) - 1
    sdf = (np.linalg.norm(p, axis=1) - 0.5 + rng.normal(0, 0.002, len(p))).astype(np.float32)
    sh = rng.uniform(0, 1, (4, len(p), 3)).astype(np.float32)
    level_sets = np.array([0.02, 0.0, -0.02], np.float32)
    tri = ref.tessellate(sdf, vox["vertices"], sh, vox["neighbors"], vox["lower_corners"], vox["upper_corners"],
                         vox["indices"], level_sets)
    out["tess/signed_distances"] = sdf
    out["tess/spherical_harmonics"] = sh
    out["tess/level_sets"] = level_sets
    for field, value in tri.items():
        out[f"tess/out_{field}"] = value

    # SDF regularizers: the sphere grid with the SDF in the grid vertices'
    # [0, 1] units (Eikonal terms of both signs), and the random grid with a
    # random SDF and an anisotropic grid size.
    cases = {
        "sphere": (grids["sphere"], (0.5 * (np.linalg.norm(p, axis=1) - 0.5)
                                     + rng.normal(0, 0.003, len(p))).astype(np.float32)),
        "random": (grids["random"], None),
    }
    for name, (occ, reg_sdf) in cases.items():
        v = ref.extract_voxels(occ)
        if reg_sdf is None:
            reg_sdf = rng.normal(0, 0.05, v["vertices"].shape[0]).astype(np.float32)
        i, j, kp = occ.shape
        grid_size = np.array([i, j, 32 * kp], np.int32)
        pos, neg, curv = ref.compute_sdf_regularizers(reg_sdf, v["neighbors"], v["lower_corners"],
                                                      v["upper_corners"], grid_size)
        out.update({f"reg_{name}/signed_distances": reg_sdf, f"reg_{name}/grid_size": grid_size,
                    f"reg_{name}/eikonal_loss_pos": pos, f"reg_{name}/eikonal_loss_neg": neg,
                    f"reg_{name}/curvature_loss": curv})
    return out


# ---------------------------------------------------------------------------
# Subdivision: write / upscale occupancy, parameter upscaling, occupancy mesh,
# vertex de-duplication
# ---------------------------------------------------------------------------
SUBDIVISION_CASES = {
    # name: (old grid bits shape, new resolution, SH coefficients)
    "double": ((4, 4, 32), (8, 8, 64), 4),
    "odd": ((5, 3, 32), (9, 7, 96), 1),
    "same": ((3, 4, 32), (3, 4, 32), 9),
}


def _lattice_points(rng, n_unique: int, n: int, tol: float) -> np.ndarray:
    """Points within 0.3 tol of a lattice of multiples of tol: duplicates
    within the tolerance, and no coordinate near a rounding boundary, so that
    round(p / tol) is the same whether the division is exact or a
    multiplication by the reciprocal (as torch does on CUDA)."""
    cells = rng.integers(-2000, 2000, size=(n_unique, 3))
    pick = rng.integers(0, n_unique, size=n)
    jitter = rng.uniform(-0.3, 0.3, size=(n, 3))
    pts = ((cells[pick] + jitter) * tol).astype(np.float32)
    by_div = np.rint(pts / np.float32(tol))
    by_mul = np.rint(pts * (np.float32(1.0) / np.float32(tol)))
    assert np.array_equal(by_div, by_mul) and np.array_equal(by_div, cells[pick])
    return pts


def subdivision_fixture(ref) -> dict[str, np.ndarray]:
    import torch

    rng = np.random.default_rng(11)
    out: dict[str, np.ndarray] = {}
    for name, (shape, resolution, c) in SUBDIVISION_CASES.items():
        occ = _pack(rng.random(shape) < 0.35)
        mask = _pack(rng.random(shape) < 0.6)
        vox = ref.extract_voxels(occ)
        v = vox["vertices"].shape[0]
        sdf = rng.normal(0, 0.1, v).astype(np.float32)
        sh = rng.normal(0, 1, (c, v, 3)).astype(np.float32)
        new_sdf, new_sh, new_occ = ref.upscale_parameters(sdf, sh, occ, mask, resolution)
        out.update({f"{name}/occupancy": occ, f"{name}/mask": mask, f"{name}/resolution": np.array(resolution),
                    f"{name}/signed_distances": sdf, f"{name}/spherical_harmonics": sh,
                    f"{name}/upscaled_occupancy": ref.upscale_occupancy(occ, resolution),
                    f"{name}/new_signed_distances": new_sdf, f"{name}/new_spherical_harmonics": new_sh,
                    f"{name}/new_occupancy": new_occ})
        colors = rng.uniform(0, 1, (3, 2, 3)).astype(np.float32)
        verts, tcol = ref.get_occupancy_mesh(occ, colors)
        out.update({f"{name}/mesh_colors_in": colors, f"{name}/mesh_vertices": verts, f"{name}/mesh_colors": tcol})
        indices = rng.integers(0, occ.size * 32, size=300).astype(np.int32)
        out.update({f"{name}/voxel_indices": indices, f"{name}/written": ref.write_occupancy(indices, occ.shape)})

    # index_vertices / index_keys: the reference's Python run with a stable
    # sort, which is what torch's CUDA sort is above 4096 elements (a radix
    # sort); the CPU default sort chooses an arbitrary member of each group.
    module = ref.python_module("triangle_extraction/index_vertices.py")
    sort = torch.Tensor.sort
    torch.Tensor.sort = lambda self, *a, **k: sort(self, *a, **{**k, "stable": True})
    try:
        for tol in (1e-6, 1e-5):
            pts = _lattice_points(rng, 1500, 4000, tol)
            key = f"index_{tol:g}"
            out[f"{key}/points"] = pts
            out[f"{key}/index"] = module.index_vertices(torch.from_numpy(pts), tol).numpy()
        keys = rng.integers(-40, 40, size=3000).astype(np.int64) * (1 << 40) + rng.integers(0, 3, size=3000)
        out["index_keys/keys"] = keys
        out["index_keys/index"] = module.index_keys(torch.from_numpy(keys)).numpy()
    finally:
        torch.Tensor.sort = sort
    return out


# ---------------------------------------------------------------------------
# Tesseract assembly of a trainer checkpoint (meshtryoshka/model/tesseract.py)
# ---------------------------------------------------------------------------
def _reference_tesseract(ref):
    """The reference's tesseract module, imported with stand-ins for its
    package-relative imports (initializer, utils, scene type) and for the
    CUDA triangle_extraction package; its component geometry, voxel
    concatenation and duplicate re-indexing are plain torch and run as they
    are. index_vertices is the reference's own Python (stable sort)."""
    import importlib.util
    import types

    import torch

    from meshtryoshka_gb300 import triangle_extraction as ours

    index_module = ref.python_module("triangle_extraction/index_vertices.py")
    sort = torch.Tensor.sort

    def index_vertices(points, tol):
        torch.Tensor.sort = lambda self, *a, **k: sort(self, *a, **{**k, "stable": True})
        try:
            return index_module.index_vertices(points, tol)
        finally:
            torch.Tensor.sort = sort

    stubs = {
        "refpkg": {}, "refpkg.model": {},
        "refpkg.initializer": {"Initializer": object},
        "refpkg.utils": {"get_value_for_step": lambda step, schedule: schedule[max(k for k in schedule if k <= step)]},
        "refpkg.model.common": {"Scene": object},
        "triangle_extraction": {"UpscaledParameters": object, "Voxels": ours.Voxels, "dilate_occupancy": None,
                                "extract_voxels": None, "get_occupancy_mesh": None, "index_vertices": index_vertices,
                                "upscale_parameters": None, "write_occupancy": None},
    }
    saved = {name: sys.modules.get(name) for name in stubs}
    for name, attrs in stubs.items():
        module = types.ModuleType(name)
        if name in ("refpkg", "refpkg.model"):
            module.__path__ = []
        for key, value in attrs.items():
            setattr(module, key, value)
        sys.modules[name] = module
    try:
        path = ref.build_ref.reference_root() / "meshtryoshka" / "model" / "tesseract.py"
        spec = importlib.util.spec_from_file_location("refpkg.model.tesseract", path)
        module = importlib.util.module_from_spec(spec)
        module.__package__ = "refpkg.model"
        spec.loader.exec_module(module)
    finally:
        for name, old in saved.items():
            if old is None:
                sys.modules.pop(name, None)
            else:
                sys.modules[name] = old
    return module


TESSERACT = dict(center=32, arm=32, center_extent=0.5)


def tesseract_fixture(ref) -> dict[str, np.ndarray]:
    """A small tesseract (central cube 32^3, six arms 32 voxels deep) assembled
    by the reference's code from a seeded flat occupancy: per component the
    oracle's extract_voxels (pinned to the reference kernels), then the
    reference's corner mapping, concatenation and duplicate re-indexing; and
    the reference's contraction inverse on seeded points."""
    import torch

    from meshtryoshka_gb300 import triangle_extraction as ours
    from oracle import oracle

    tm = _reference_tesseract(ref)
    cm = ref.python_module("meshtryoshka/model/contraction.py")
    cfg = tm.TesseractCfg(center_resolution={0: TESSERACT["center"]}, arm_resolution={0: TESSERACT["arm"]},
                          center_extent=TESSERACT["center_extent"], parameter_init_seed=0, active_sh_degree={0: 0},
                          sh_lr_scale=1.0, disable_spherical_harmonics=False, disable_sparsity=False,
                          disable_tesseract=False)
    components = [tm.TesseractCenter(cfg)] + [tm.TesseractArm(cfg, d, s) for d in range(3) for s in range(2)]
    rng = np.random.default_rng(23)
    words, parts, out = [], [], {}
    for index, component in enumerate(components):
        i, j, k = component.shape(0)
        # A shell around the component's centre plus sparse noise, so voxels,
        # subvoxels and shared faces all occur.
        z, y, x = np.meshgrid(*(np.arange(n) + 0.5 for n in (i, j, k)), indexing="ij")
        r = np.sqrt(((x / k - 0.5) * 2) ** 2 + ((y / j - 0.5) * 2) ** 2 + ((z / i - 0.5) * 2) ** 2)
        bits = (np.abs(r - 0.8) < 0.05) | (rng.random((i, j, k)) < 0.002)
        occ = _pack(bits)
        words.append(occ.reshape(-1))
        v = oracle.extract_voxels(occ)
        t = ours.Voxels(*(torch.from_numpy(np.ascontiguousarray(a)) for a in
                          (v.vertices, v.neighbors, v.lower_corners, v.upper_corners, v.indices)), v.grid_shape)
        parts.append(t._replace(vertices=component.interpolate(t.vertices)))
        out[f"corners_{index}"] = component.corners.numpy()
    voxels = tm.Tesseract.concatenate_voxels(parts)
    voxels = tm.Tesseract.reindex_duplicate_vertices(voxels)
    out.update({"occupancy": np.concatenate(words).astype(np.int32), "vertices": voxels.vertices.numpy(),
                "neighbors": voxels.neighbors.numpy(), "lower_corners": voxels.lower_corners.numpy(),
                "upper_corners": voxels.upper_corners.numpy(), "indices": voxels.indices.numpy(),
                "layout": np.array([TESSERACT["center"], TESSERACT["arm"]], np.int32),
                "center_extent": np.array(TESSERACT["center_extent"], np.float32)})
    points = rng.uniform(-0.05, 1.05, (4000, 3)).astype(np.float32)
    contraction = cm.Contraction(cm.ContractionCfg(center_radius=0.6, arm_ratio=0.5, disable_exponential=False),
                                 TESSERACT["center_extent"])
    out["contraction_points"] = points
    out["uncontracted"] = contraction.uncontract(torch.from_numpy(points)).numpy()
    weights = rng.uniform(0, 1, (500, 3)).astype(np.float32)
    out["map_points"] = weights
    for index, component in enumerate(components):
        out[f"mapped_{index}"] = component.interpolate(torch.from_numpy(weights)).numpy()
    return out


# ---------------------------------------------------------------------------
# Rasterization: a tessellated sphere seen by a few cameras
# ---------------------------------------------------------------------------
SCENES = {
    "two_cams": dict(n=32, levels=(0.03, 0.0, -0.03), sh_degree=2, cameras=((0.0, 0.0, 2.0), (1.2, 0.8, 1.3)),
                     image_shape=(40, 56), fov=55.0, sharpness=40.0, seed=5),
    "close_up": dict(n=32, levels=(0.01, -0.01), sh_degree=1, cameras=((0.3, 0.2, 0.9),), image_shape=(48, 32),
                     fov=70.0, sharpness=80.0, seed=6),
}


def raster_fixture(ref, n, levels, sh_degree, cameras, image_shape, fov, sharpness, seed) -> dict[str, np.ndarray]:
    rng = np.random.default_rng(seed)
    vox = ref.extract_voxels(_sphere_band(n))
    p = 2 * vox["vertices"].astype(np.float64) - 1
    gsdf = (np.linalg.norm(p, axis=1) - 0.5 + rng.normal(0, 0.002, len(p))).astype(np.float32)
    c = (sh_degree + 1) ** 2
    gsh = np.empty((c, len(p), 3), np.float32)
    gsh[0] = rng.uniform(0, 1, (len(p), 3))
    gsh[1:] = rng.normal(0, 0.1, (c - 1, len(p), 3))
    ls = np.array(levels, np.float32)
    tri = ref.tessellate(gsdf, vox["vertices"], gsh, vox["neighbors"], vox["lower_corners"], vox["upper_corners"],
                         vox["indices"], ls)
    vertices = (2.0 * tri["vertices"] - 1.0).astype(np.float32)
    faces = tri["faces"]
    face_offsets = tri["face_offsets"]
    s = len(levels)
    # face_offsets[1:].view(S, -1)[:, -1] // 3 (triangle_extraction/__init__.py:146)
    sfb = np.ascontiguousarray(face_offsets[1:].reshape(s, -1)[:, -1] // 3).astype(np.int32)
    sdf = tri["signed_distances"]
    sh = tri["spherical_harmonics"]

    ext = np.stack([_look_at(cam) for cam in cameras]).astype(np.float32)
    intr = np.stack([_pinhole(image_shape[0], image_shape[1], fov) for _ in cameras]).astype(np.float32)
    h, w = image_shape
    b = len(cameras)
    rows, cols = -(-h // TILE[0]), -(-w // TILE[1])
    t = rows * cols

    xy, depth = ref.project_vertices(vertices, ext, intr)
    tmin, tmax, count = ref.bound_triangles(xy, depth, faces, TILE, (rows, cols), NEAR_PLANE)
    campos = np.linalg.inv(ext.astype(np.float64))[:, :3, 3].astype(np.float32)
    colors = ref.evaluate_sh(sh_degree, vertices, sh, campos)

    out = dict(vertices=vertices, faces=faces, shell_face_boundaries=sfb, signed_distances=sdf,
               spherical_harmonics=sh, sh_degree=np.int32(sh_degree), extrinsics=ext, intrinsics=intr,
               image_shape=np.array(image_shape, np.int32), sharpness=np.float32(sharpness),
               near_plane=np.float32(NEAR_PLANE), xy=xy, depth=depth, tile_minima=tmin, tile_maxima=tmax,
               num_tiles_overlapped=count, camera_positions=campos, colors=colors)

    for mode, explicit in (("fused", False), ("explicit", True)):
        keys, tri_idx = ref.generate_keys(explicit, depth, faces, sfb, tmin, tmax, count, cols)
        order = np.argsort(keys, kind="stable")
        sk, st = keys[order], tri_idx[order]
        bounds = ref.delineate_tiles(explicit, sk, b, s if explicit else 1, t, explicit)
        out.update({f"{mode}/keys": keys, f"{mode}/triangles": tri_idx, f"{mode}/sorted_keys": sk,
                    f"{mode}/sorted_triangles": st, f"{mode}/tile_boundaries": bounds})

    fused_args = (xy, colors, sdf, faces, sharpness, out["fused/sorted_keys"], out["fused/sorted_triangles"],
                  out["fused/tile_boundaries"].reshape(b, t, 2), s, (h, w))
    out["fused/image"] = ref.intersect_and_composite(*fused_args)
    grad_image = rng.normal(0, 1, out["fused/image"].shape).astype(np.float32)
    gc, gs, gsh = ref.intersect_and_composite_backward(*fused_args, out["fused/image"], grad_image)
    out.update({"fused/grad_image": grad_image, "fused/grad_colors": gc, "fused/grad_signed_distances": gs,
                "fused/grad_sharpness": np.float32(gsh)})
    uv, index = ref.intersect(xy, faces, out["explicit/sorted_triangles"], out["explicit/tile_boundaries"], s, (h, w))
    isdf, icol = ref.interpolate(uv, index, faces, sdf, colors)
    per_pixel_sdf = isdf.transpose(0, 2, 3, 1).reshape(-1, s)
    per_pixel_col = icol.transpose(0, 2, 3, 1, 4).reshape(-1, s, 3)
    mask = (index != -1).transpose(0, 2, 3, 1).reshape(-1, s)
    ccol, ct = ref.composite(per_pixel_sdf, per_pixel_col, mask, sharpness)
    out.update({"explicit/uv": uv, "explicit/index": index, "explicit/interp_sdf": isdf,
                "explicit/interp_colors": icol, "explicit/composite_colors": ccol, "explicit/composite_T": ct})
    g_col = rng.normal(0, 1, ccol.shape).astype(np.float32)
    g_t = rng.normal(0, 1, ct.shape).astype(np.float32)
    gs, gc, gsh = ref.composite_backward(per_pixel_sdf, per_pixel_col, mask, sharpness, ccol, ct, g_col, g_t)
    out.update({"explicit/grad_composite_colors": g_col, "explicit/grad_composite_T": g_t,
                "explicit/grad_shell_signed_distances": gs, "explicit/grad_shell_colors": gc,
                "explicit/grad_sharpness": np.float32(gsh)})
    return out


def generate(reference: str | None = None) -> dict[str, dict[str, np.ndarray]]:
    if reference:
        os.environ["MESHTRYOSHKA_REFERENCE"] = reference
    from oracle import ref

    if not ref.available():
        raise SystemExit("reference tree not found; cannot build its kernels")
    fixtures = {"extraction": extraction_fixture(ref), "subdivision": subdivision_fixture(ref),
                "tesseract": tesseract_fixture(ref)}
    for name, kw in SCENES.items():
        fixtures[f"raster_{name}"] = raster_fixture(ref, **kw)
    return fixtures


def main() -> None:
    parser = argparse.ArgumentParser()
    parser.add_argument("--reference", default=None)
    args = parser.parse_args()
    for name, arrays in generate(args.reference).items():
        path = HERE / f"{name}.npz"
        np.savez_compressed(path, **arrays)
        print(f"{path.name}: {len(arrays)} arrays, {path.stat().st_size / 1024:.0f} KiB")


if __name__ == "__main__":
    main()
