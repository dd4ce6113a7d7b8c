"""Cameras of different image sizes rendered in one pass (``render_cameras``).

Each camera's image must equal rendering that camera alone with
``render_fused`` (bit for bit: a camera's keys keep their relative order in
the batch, so every pixel sees the same hits in the same order), and the
gradients of a loss over all cameras must equal the sum of the single-camera
gradients (within 1e-5 of the largest: atomic accumulation order).
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from meshtryoshka_gb300 import synthetic
from meshtryoshka_gb300 import triangle_rasterization as tr
from tests.scenes import make_scene

pytestmark = pytest.mark.gpu

CAMERAS = (  # eye, (height, width), fov
    ((0.0, 0.0, 2.0), (75, 101), 55.0),
    ((1.2, 0.8, 1.3), (128, 64), 60.0),
    ((-1.5, -0.3, 1.1), (40, 200), 45.0),
    ((0.3, 1.6, 0.9), (33, 47), 70.0),
    ((0.0, -1.8, -1.0), (96, 96), 50.0),
)


def _t(a, device):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _scene(device):
    sc = make_scene(sh_degree=2, levels=(0.03, 0.01, -0.01, -0.03))
    ext = np.stack([synthetic.look_at(np.array(eye)) for eye, _, _ in CAMERAS]).astype(np.float32)
    intr = np.stack([synthetic.pinhole(h, w, fov) for _, (h, w), fov in CAMERAS]).astype(np.float32)
    shapes = [shape for _, shape, _ in CAMERAS]
    d = device
    args = dict(vertices=_t(sc.vertices, d), faces=_t(sc.faces, d), shell_face_boundaries=_t(sc.face_boundaries, d),
                signed_distances=_t(sc.sdf, d).requires_grad_(True),
                spherical_harmonics=_t(sc.sh, d).requires_grad_(True), sh_degree=sc.sh_degree,
                sharpness=float(sc.sharpness), background=_t(sc.background, d))
    return _t(ext, d), _t(intr, d), shapes, args


def _close(got, want, rtol=1e-5):
    scale = max(float(want.abs().max()), 1e-30)
    err = float((got - want).abs().max())
    assert err <= rtol * scale, f"max abs err {err:.3e} > {rtol:g} x {scale:.3e}"


@pytest.mark.parametrize("tile", [(16, 16), (8, 8), (12, 20)])
def test_cameras_match_single_camera_renders(cuda_device, tile):
    ext, intr, shapes, args = _scene(cuda_device)
    rng = np.random.default_rng(0)
    targets = [_t(rng.normal(0, 1, (3, h, w)).astype(np.float32), cuda_device) for h, w in shapes]

    images = tr.render_cameras(ext, intr, shapes, tile_shape=tile, **args)
    assert [tuple(i.shape) for i in images] == [(3, h, w) for h, w in shapes]
    sum(((img * t).sum() for img, t in zip(images, targets))).backward()
    g_sdf, g_sh = args["signed_distances"].grad.clone(), args["spherical_harmonics"].grad.clone()
    args["signed_distances"].grad = None
    args["spherical_harmonics"].grad = None

    loss = 0.0
    for b, (h, w) in enumerate(shapes):
        single = tr.render_fused(ext[b:b + 1], intr[b:b + 1], (h, w), tile_shape=tile, **args)[0]
        torch.testing.assert_close(images[b], single, rtol=0, atol=0)
        loss = loss + (single * targets[b]).sum()
    loss.backward()
    _close(g_sdf, args["signed_distances"].grad)
    _close(g_sh, args["spherical_harmonics"].grad)
    assert float(g_sdf.abs().max()) > 0


def test_cameras_in_a_captured_graph(cuda_device):
    """The ragged batch is capturable: no host reads with device counts."""
    ext, intr, shapes, args = _scene(cuda_device)
    want = [i.detach().clone() for i in tr.render_cameras(ext, intr, shapes, **args)]
    faces = args["faces"]
    nf = torch.tensor(faces.shape[0], dtype=torch.int32, device=cuda_device)
    kw = dict(args, signed_distances=args["signed_distances"].detach(),
              spherical_harmonics=args["spherical_harmonics"].detach())
    key_capacity = int(tr.LAST_RENDER_STATS["num_keys"]) + 1000
    stream = torch.cuda.Stream(cuda_device)
    stream.wait_stream(torch.cuda.current_stream(cuda_device))
    with torch.cuda.stream(stream):
        tr.render_cameras(ext, intr, shapes, num_faces=nf, key_capacity=key_capacity, **kw)
    torch.cuda.current_stream(cuda_device).wait_stream(stream)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        out = tr.render_cameras(ext, intr, shapes, num_faces=nf, key_capacity=key_capacity, **kw)
    graph.replay()
    torch.cuda.synchronize()
    for got, ref in zip(out, want):
        torch.testing.assert_close(got, ref, rtol=0, atol=0)


LOSS_RTOL = 1e-5


def test_uneven_workload_batched_equals_per_camera(cuda_device):
    """32 cameras of 200-1600 px: the batched training step (eager and as a
    CUDA graph) gives the per-camera form's loss and gradients."""
    from meshtryoshka_gb300 import graph, pipeline

    w = pipeline.build_workload("uneven", cuda_device)
    assert w.image_shapes is not None and len(set(w.image_shapes)) > 1

    def grads():
        out = w.grid_sdf.grad.clone(), w.grid_sh.grad.clone()
        w.grid_sdf.grad = None
        w.grid_sh.grad = None
        return out

    loss_plain = float(pipeline.per_camera_training_step(w).detach())
    g_plain = grads()
    loss_batched = float(pipeline.training_step(w).detach())
    g_batched = grads()
    # The loss is a float32 sum of ~3e7 squared errors, accumulated by
    # per-warp atomics in scheduling order: the two forms agree to the
    # rounding of such a sum, not bit for bit.
    assert abs(loss_batched - loss_plain) <= LOSS_RTOL * abs(loss_plain)
    _close(g_batched[0], g_plain[0])
    _close(g_batched[1], g_plain[1])

    step = graph.CapturedTrainingStep(w)
    loss_graph = float(step())
    assert step.check()
    assert abs(loss_graph - loss_plain) <= LOSS_RTOL * abs(loss_plain)
    _close(w.grid_sdf.grad, g_plain[0])
    _close(w.grid_sh.grad, g_plain[1])


@pytest.mark.parametrize("tile", [(8, 8), (12, 20)])
def test_tile_order_leaves_results_unchanged(cuda_device, tile, monkeypatch):
    """The longest-first tile order of the compositing kernels (cameras of
    different sizes: the tile's range is found through the camera table)
    changes only the order the work is taken in: identical images, the same
    gradients up to the order of their atomic sums."""
    results = []
    for ordered in (False, True):
        monkeypatch.setattr(tr, "TILE_ORDER", ordered)
        ext, intr, shapes, args = _scene(cuda_device)
        images = tr.render_cameras(ext, intr, shapes, tile_shape=tile, **args)
        rng = np.random.default_rng(3)
        loss = sum((img * _t(rng.normal(0, 1, tuple(img.shape)).astype(np.float32), cuda_device)).sum()
                   for img in images)
        loss.backward()
        results.append(([img.detach() for img in images], args["signed_distances"].grad.clone(),
                        args["spherical_harmonics"].grad.clone()))
    (i0, s0, h0), (i1, s1, h1) = results
    for a, b in zip(i0, i1):
        assert torch.equal(a, b)
    _close(s1, s0)
    _close(h1, h0)
    assert float(s0.abs().max()) > 0
