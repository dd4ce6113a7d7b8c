"""Loader for the golden fixtures in tests/golden/ (outputs of the reference's
own kernels, made by tests/golden/make_golden.py)."""

from __future__ import annotations

from pathlib import Path

import numpy as np

GOLDEN_DIR = Path(__file__).resolve().parent / "golden"
RASTER_SCENES = ("two_cams", "close_up")
EXTRACTION_GRIDS = ("random", "sphere", "edges")
SUBDIVISION_CASES = ("double", "odd", "same")
INDEX_TOLERANCES = (1e-6, 1e-5)
TESS_FIELDS = ("vertices", "signed_distances", "spherical_harmonics", "faces", "voxel_indices", "vertex_offsets",
               "face_offsets", "cell_codes", "vertex_types")


def load(name: str) -> dict[str, np.ndarray]:
    with np.load(GOLDEN_DIR / f"{name}.npz") as z:
        return {k: z[k] for k in z.files}


def raster(scene: str) -> dict[str, np.ndarray]:
    return load(f"raster_{scene}")


def grid_dims(g: dict[str, np.ndarray]) -> tuple[int, int, int, int, int, int]:
    """(B, S, H, W, rows, cols) of a raster fixture (16 x 16 tiles)."""
    b = g["extrinsics"].shape[0]
    s = g["shell_face_boundaries"].shape[0]
    h, w = (int(x) for x in g["image_shape"])
    return b, s, h, w, -(-h // 16), -(-w // 16)


def per_pixel_shells(g: dict[str, np.ndarray]):
    """The explicit-mode composite inputs as the reference lays them out:
    [pixel, shell] signed distances / colours / hit mask."""
    s = g["shell_face_boundaries"].shape[0]
    sdf = g["explicit/interp_sdf"].transpose(0, 2, 3, 1).reshape(-1, s)
    col = g["explicit/interp_colors"].transpose(0, 2, 3, 1, 4).reshape(-1, s, 3)
    mask = (g["explicit/index"] != -1).transpose(0, 2, 3, 1).reshape(-1, s)
    return np.ascontiguousarray(sdf), np.ascontiguousarray(col), np.ascontiguousarray(mask)
