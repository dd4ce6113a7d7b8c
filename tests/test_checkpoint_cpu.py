"""Scene ingest from reference checkpoints, against the reference's own
tesseract assembly (tests/golden/tesseract.npz, made by
tests/golden/make_golden.py from meshtryoshka/model/tesseract.py and
contraction.py): the components' corner geometry, the trilinear map onto
them, the contraction's inverse, and the concatenation plus duplicate
re-indexing of the components' voxels (voxels from the oracle's
extract_voxels, duplicates from the oracle's index_vertices). No GPU."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

from meshtryoshka_gb300 import checkpoint as ck
from meshtryoshka_gb300 import triangle_extraction as te
from oracle import oracle

GOLDEN = np.load(Path(__file__).parent / "golden" / "tesseract.npz")


def _layout():
    c, a = (int(x) for x in GOLDEN["layout"])
    return ck.TesseractLayout(c, a, float(GOLDEN["center_extent"]))


def test_component_corners_and_map_match_reference():
    layout = _layout()
    comps = layout.components()
    assert len(comps) == 7
    points = torch.from_numpy(GOLDEN["map_points"])
    for index, comp in enumerate(comps):
        corners = ck.component_corners(layout, comp, "cpu")
        np.testing.assert_array_equal(corners.numpy(), GOLDEN[f"corners_{index}"])
        mapped = ck.map_to_component(points, corners).numpy()
        np.testing.assert_allclose(mapped, GOLDEN[f"mapped_{index}"], rtol=0, atol=2e-7)


def test_uncontract_matches_reference():
    c = ck.Contraction(center_radius=0.6, arm_ratio=0.5, center_extent=float(GOLDEN["center_extent"]))
    got = c.uncontract(torch.from_numpy(GOLDEN["contraction_points"])).numpy()
    np.testing.assert_allclose(got, GOLDEN["uncontracted"], rtol=1e-6, atol=1e-7)


def test_concatenation_and_duplicates_match_reference():
    layout = _layout()
    occ = GOLDEN["occupancy"]
    parts, start = [], 0
    for comp in layout.components():
        i, j, k = layout.shape(comp)
        words = occ[start:start + i * j * k // 32].reshape(i, j, k // 32)
        start += words.size
        v = oracle.extract_voxels(words)
        t = te.Voxels(*(torch.from_numpy(np.ascontiguousarray(a)) for a in
                        (v.vertices, v.neighbors, v.lower_corners, v.upper_corners, v.indices)), v.grid_shape)
        parts.append(t._replace(vertices=ck.map_to_component(t.vertices, ck.component_corners(layout, comp, "cpu"))))
    assert start == occ.size
    voxels = ck.concatenate_voxels(parts)
    np.testing.assert_allclose(voxels.vertices.numpy(), GOLDEN["vertices"], rtol=0, atol=2e-7)
    np.testing.assert_array_equal(voxels.neighbors.numpy(), GOLDEN["neighbors"])
    np.testing.assert_array_equal(voxels.indices.numpy(), GOLDEN["indices"])
    first = oracle.index_vertices(GOLDEN["vertices"], 1e-6)
    np.testing.assert_array_equal(first[voxels.lower_corners.numpy()], GOLDEN["lower_corners"])
    np.testing.assert_array_equal(first[voxels.upper_corners.numpy()], GOLDEN["upper_corners"])


def test_layout_shapes():
    layout = ck.TesseractLayout(64, 32, 0.5)
    assert layout.shape(("center", -1, -1)) == (64, 64, 64)
    assert layout.shape(("arm", 2, 1)) == (64, 64, 32)
    assert layout.extent == (128, 128, 128)
    flat = ck.TesseractLayout(64, 32, 0.5, disable_tesseract=True)
    assert flat.components() == [("center", -1, -1)]
    assert flat.shape(("center", -1, -1)) == (128, 128, 128)


def test_checkpoint_layout_mismatch_is_rejected(tmp_path):
    if torch.cuda.is_available():
        pytest.skip("covered by the GPU test")
    path = tmp_path / "model.ckpt"
    torch.save({"model": {"tesseract.occupancy": torch.zeros(10, dtype=torch.int32)}}, path)
    with pytest.raises((RuntimeError, ValueError)):
        ck.load_tesseract_checkpoint(path, _layout(), "cpu")
