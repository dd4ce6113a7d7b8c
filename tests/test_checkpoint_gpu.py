"""A reference-format checkpoint (torch.save({"model": state_dict}) with the
tesseract's occupancy, raw signed distances and SH) loaded onto the GPU:
the assembled voxels equal the reference's assembly of the same occupancy
(tests/golden/tesseract.npz), the parameters come through unchanged, and the
scene serves render requests like a synthetic one."""

from __future__ import annotations

from pathlib import Path

import numpy as np
import pytest
import torch

from meshtryoshka_gb300 import checkpoint as ck
from meshtryoshka_gb300 import serving, synthetic
from meshtryoshka_gb300 import triangle_rasterization as tr

pytestmark = pytest.mark.gpu

GOLDEN = np.load(Path(__file__).parent / "golden" / "tesseract.npz")


def _save(tmp_path, sh_degree=1):
    g = GOLDEN["vertices"].shape[0]
    rng = np.random.default_rng(4)
    c = (sh_degree + 1) ** 2
    state = {
        "tesseract.step": torch.tensor(12000, dtype=torch.int32),
        "tesseract.occupancy": torch.from_numpy(GOLDEN["occupancy"]),
        "tesseract.signed_distances_raw": torch.from_numpy(rng.normal(0, 0.01, g).astype(np.float32)),
        "tesseract.sh_rgb": torch.from_numpy(rng.normal(0, 0.1, (1, g, 3)).astype(np.float32)),
        "tesseract.sh_rest": (torch.from_numpy(rng.normal(0, 0.05, (c - 1, g, 3)).astype(np.float32)) if c > 1
                              else torch.empty([], dtype=torch.float32)),
        "contraction_dummy": torch.zeros(1),
    }
    path = tmp_path / "checkpoint.ckpt"
    torch.save({"model": state, "step": 12000}, path)
    return path, state


def _layout():
    c, a = (int(x) for x in GOLDEN["layout"])
    return ck.TesseractLayout(c, a, float(GOLDEN["center_extent"]))


@pytest.mark.parametrize("sh_degree", [0, 1])
def test_checkpoint_loads_the_reference_assembly(cuda_device, tmp_path, sh_degree):
    path, state = _save(tmp_path, sh_degree)
    scene = ck.load_tesseract_checkpoint(path, _layout(), cuda_device)
    v = scene.voxels
    np.testing.assert_allclose(v.vertices.cpu().numpy(), GOLDEN["vertices"], rtol=0, atol=1e-6)
    for name in ("neighbors", "lower_corners", "upper_corners", "indices"):
        np.testing.assert_array_equal(getattr(v, name).cpu().numpy(), GOLDEN[name])
    assert v.grid_shape == (96, 96, 96)
    assert scene.step == 12000 and scene.sh_degree == sh_degree
    torch.testing.assert_close(scene.signed_distances.cpu(), state["tesseract.signed_distances_raw"], rtol=0,
                               atol=0)
    assert scene.spherical_harmonics.shape == ((sh_degree + 1) ** 2, v.vertices.shape[0], 3)
    torch.testing.assert_close(scene.spherical_harmonics[:1].cpu(), state["tesseract.sh_rgb"], rtol=0, atol=0)


def test_checkpoint_rejects_a_layout_that_does_not_match(cuda_device, tmp_path):
    path, _ = _save(tmp_path)
    with pytest.raises(ValueError):
        ck.load_tesseract_checkpoint(path, ck.TesseractLayout(32, 0, 0.5), cuda_device)


def test_checkpoint_scene_serves_requests(cuda_device, tmp_path):
    path, _ = _save(tmp_path)
    contraction = ck.Contraction(center_radius=0.6, arm_ratio=0.5, center_extent=float(GOLDEN["center_extent"]))
    levels = torch.tensor([0.01, 0.0, -0.01], device=cuda_device)
    scene = serving.Scene.from_checkpoint(path, _layout(), contraction, levels, cuda_device,
                                          sdf_offset=ck.sphere_initializer(0.3))
    vertices, faces, fb, sdf, sh = scene.mesh
    assert faces.shape[0] > 0
    ext = torch.from_numpy(synthetic.look_at(np.array([0.0, 0.3, 2.5]))[None]).to(cuda_device)
    intr = torch.from_numpy(synthetic.pinhole(96, 128, 60.0)[None]).to(cuda_device)
    req = serving.Request(0, 0, ext[0], intr[0], (96, 128), False, None, 0.0)
    done = serving.Server([scene]).run([req])
    want = tr.render_fused(ext, intr, (96, 128), vertices, faces, fb, sdf, sh, scene.sh_degree, scene.sharpness,
                           scene.background)[0]
    torch.testing.assert_close(done[0].image, want, rtol=0, atol=0)
    assert float(want.std()) > 0  # something is in view
