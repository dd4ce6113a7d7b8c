"""The MSE epilogue inside the compositing kernels against the unfused
composition (render, background blend, clip, mean squared error as tensor
ops): the same loss (within 1e-5 relative: summation order) and the same
gradients (within 1e-5 of the largest entry: atomic order), for cameras of
one size and of different sizes, in both gradient-routing modes, and through
the whole training step."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from meshtryoshka_gb300 import pipeline
from meshtryoshka_gb300 import triangle_rasterization as tr
from tests.scenes import SCENES, make_scene

pytestmark = pytest.mark.gpu


def _t(a, device):
    return torch.from_numpy(np.ascontiguousarray(a)).to(device)


def _close(got, want, rtol=1e-5):
    scale = max(float(want.abs().max()), 1e-30)
    err = float((got - want).abs().max())
    assert err <= rtol * scale, f"max abs err {err:.3e} > {rtol:g} x {scale:.3e}"


def _inputs(scene, d):
    return dict(vertices=_t(scene.vertices, d), faces=_t(scene.faces, d),
                shell_face_boundaries=_t(scene.face_boundaries, d),
                signed_distances=_t(scene.sdf, d).requires_grad_(True),
                spherical_harmonics=_t(scene.sh, d).requires_grad_(True), sh_degree=scene.sh_degree,
                sharpness=torch.tensor(float(scene.sharpness), device=d).requires_grad_(True),
                background=_t(scene.background, d))


def _grads(args):
    out = [args[k].grad.clone() for k in ("signed_distances", "spherical_harmonics", "sharpness")]
    for k in ("signed_distances", "spherical_harmonics", "sharpness"):
        args[k].grad = None
    return out


@pytest.mark.parametrize("name", ["three_cams_odd", "close_up"])
@pytest.mark.parametrize("mode", ["reference", "exact"])
def test_fused_loss_equals_unfused(cuda_device, name, mode):
    scene = make_scene(**SCENES[name])
    d = cuda_device
    args = _inputs(scene, d)
    ext, intr = _t(scene.extrinsics, d), _t(scene.intrinsics, d)
    b = scene.extrinsics.shape[0]
    target = _t(np.random.default_rng(0).uniform(0, 1, (b, 3, *scene.image_shape)).astype(np.float32), d)
    image = tr.render_fused(ext, intr, scene.image_shape, **args, gradient_mode=mode)
    loss = ((image - target) ** 2).mean()
    loss.backward()
    want = _grads(args)
    fused = tr.render_fused_loss(ext, intr, scene.image_shape, **args, target=target, gradient_mode=mode)
    assert abs(float(fused.detach()) - float(loss.detach())) <= 1e-5 * float(loss.detach())
    fused.backward()
    for got, ref in zip(_grads(args), want):
        _close(got, ref)


def test_fused_loss_cameras_of_different_sizes(cuda_device):
    scene = make_scene(**SCENES["three_cams_odd"])
    d = cuda_device
    args = _inputs(scene, d)
    ext, intr = _t(scene.extrinsics, d), _t(scene.intrinsics, d)
    shapes = [(75, 101), (40, 64), (96, 33)]
    rng = np.random.default_rng(1)
    targets = [_t(rng.uniform(0, 1, (3, h, w)).astype(np.float32), d) for h, w in shapes]
    images = tr.render_cameras(ext, intr, shapes, **args)
    total = sum(((img - t) ** 2).sum() for img, t in zip(images, targets))
    loss = total / sum(t.numel() for t in targets)
    loss.backward()
    want = _grads(args)
    flat = torch.cat([t.reshape(-1) for t in targets])
    fused = tr.render_fused_loss(ext, intr, None, **args, target=flat, camera_shapes=shapes)
    assert abs(float(fused.detach()) - float(loss.detach())) <= 1e-5 * float(loss.detach())
    fused.backward()
    for got, ref in zip(_grads(args), want):
        _close(got, ref)


@pytest.mark.parametrize("config", ["small", "uneven"])
def test_training_step_fused_loss_equals_unfused(cuda_device, config):
    w = pipeline.build_workload(config, cuda_device)
    results = []
    for fused in (False, True):
        w.fused_loss = fused
        loss = float(pipeline.training_step(w).detach())
        results.append((loss, w.grid_sdf.grad.clone(), w.grid_sh.grad.clone()))
        w.grid_sdf.grad = None
        w.grid_sh.grad = None
    (l0, s0, h0), (l1, s1, h1) = results
    assert abs(l1 - l0) <= 1e-5 * l0
    _close(s1, s0)
    _close(h1, h0)


@pytest.mark.parametrize("ssaa", [2, 3])
@pytest.mark.parametrize("name", ["three_cams_odd", "close_up"])
def test_fused_loss_with_ssaa_equals_unfused(cuda_device, name, ssaa):
    """SSAA (the trainer's train_ssaa): the image rendered at ssaa times the
    size, blended, averaged per ssaa x ssaa block and clipped, against the
    fused loss whose compositing backward takes 1 / ssaa^2 of each output
    pixel's gradient."""
    scene = make_scene(**SCENES[name])
    d = cuda_device
    args = _inputs(scene, d)
    ext, intr = _t(scene.extrinsics, d), _t(scene.intrinsics, d)
    b = scene.extrinsics.shape[0]
    target = _t(np.random.default_rng(ssaa).uniform(0, 1, (b, 3, *scene.image_shape)).astype(np.float32), d)
    image = tr.render_fused(ext, intr, scene.image_shape, **args, ssaa=ssaa, tile_shape=(8, 8))
    loss = ((image - target) ** 2).mean()
    loss.backward()
    want = _grads(args)
    fused = tr.render_fused_loss(ext, intr, scene.image_shape, **args, target=target, ssaa=ssaa, tile_shape=(8, 8))
    assert abs(float(fused.detach()) - float(loss.detach())) <= 1e-5 * float(loss.detach())
    fused.backward()
    for got, ref in zip(_grads(args), want):
        _close(got, ref)


def test_training_step_with_ssaa_uses_the_fused_loss(cuda_device):
    w = pipeline.build_workload("small", cuda_device)
    w.ssaa = 2
    results = []
    for fused in (False, True):
        w.fused_loss = fused
        loss = float(pipeline.training_step(w).detach())
        results.append((loss, w.grid_sdf.grad.clone(), w.grid_sh.grad.clone()))
        w.grid_sdf.grad = None
        w.grid_sh.grad = None
    (l0, s0, h0), (l1, s1, h1) = results
    assert abs(l1 - l0) <= 1e-5 * l0
    _close(s1, s0)
    _close(h1, h0)
