"""The CUDA-graph training step against the eager step.

* capacity-sized tessellation holds the eager tessellation as its live prefix
  (bit for bit);
* a captured fused step gives the eager step's loss and gradients (within
  1e-5 of the largest gradient: both accumulate with atomics), and repeated
  replays agree;
* capacities below the live sizes are detected by ``check()``, which
  re-captures; the replay after that matches the eager step. Undersized
  buffers are safe by construction: every writer is capacity-guarded and the
  readers clamp the device counts.
"""

from __future__ import annotations

import pytest
import torch

from meshtryoshka_gb300 import graph, pipeline
from meshtryoshka_gb300 import triangle_extraction as te
from meshtryoshka_gb300 import triangle_rasterization as tr

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-5
# Losses are float32 sums accumulated by per-warp atomics in scheduling order.
LOSS_RTOL = 1e-5


def _close(got, want, rtol=GRAD_RTOL):
    scale = max(float(want.abs().max()), 1e-30)
    err = float((got - want).abs().max())
    assert err <= rtol * scale, f"max abs err {err:.3e} > {rtol:g} x {scale:.3e}"


def _eager(w):
    w.grid_sdf.grad = None
    w.grid_sh.grad = None
    loss, stats = pipeline.forward(w, "fused")
    loss.backward()
    out = float(loss.detach()), w.grid_sdf.grad.clone(), w.grid_sh.grad.clone(), stats
    w.grid_sdf.grad = None
    w.grid_sh.grad = None
    return out


def test_counted_tessellation_prefix_is_eager(cuda_device):
    w = pipeline.build_workload("small", cuda_device)
    args = (w.grid_sdf.detach(), w.voxels.vertices, w.grid_sh.detach(), w.voxels.neighbors, w.voxels.lower_corners,
            w.voxels.upper_corners, w.voxels.indices, w.level_sets)
    eager = te.tessellate_voxels(*args)
    v, f = eager.vertices.shape[0], eager.faces.shape[0]
    tri, counts = te.tessellate_voxels_counted(*args, v + 1000, f + 777)
    assert int(counts.num_vertices) == v and int(counts.num_faces) == f
    assert tri.vertices.shape[0] == v + 1000 and tri.faces.shape[0] == f + 777
    torch.testing.assert_close(tri.vertices[:v], eager.vertices, rtol=0, atol=0)
    torch.testing.assert_close(tri.signed_distances[:v], eager.signed_distances, rtol=0, atol=0)
    torch.testing.assert_close(tri.spherical_harmonics[:, :v], eager.spherical_harmonics, rtol=0, atol=0)
    torch.testing.assert_close(tri.faces[:f], eager.faces, rtol=0, atol=0)
    torch.testing.assert_close(tri.face_boundaries, eager.face_boundaries, rtol=0, atol=0)


def test_captured_step_matches_eager(cuda_device):
    w = pipeline.build_workload("small", cuda_device)
    loss_e, gsdf_e, gsh_e, _ = _eager(w)
    step = graph.CapturedTrainingStep(w)
    assert step.launches_per_replay >= 15  # the whole step: tessellation, render, loss, backward
    for _ in range(3):
        loss = step()
        torch.cuda.synchronize()
        assert step.check()
        assert abs(float(loss) - loss_e) <= LOSS_RTOL * abs(loss_e)
        _close(w.grid_sdf.grad, gsdf_e)
        _close(w.grid_sh.grad, gsh_e)


def test_captured_step_recaptures_when_capacity_overflows(cuda_device):
    w = pipeline.build_workload("small", cuda_device)
    loss_e, gsdf_e, gsh_e, stats = _eager(w)
    small = pipeline.Capacities(stats["V"] // 2, stats["F"] // 2, stats["K"] // 2)
    step = graph.CapturedTrainingStep(w, capacities=small)
    step()
    torch.cuda.synchronize()
    assert not step.check()
    assert step.recaptures == 1
    c = step.capacities
    assert c.vertices >= stats["V"] and c.faces >= stats["F"] and c.keys >= stats["K"]
    loss = step()
    torch.cuda.synchronize()
    assert step.check()
    assert abs(float(loss) - loss_e) <= LOSS_RTOL * abs(loss_e)
    _close(w.grid_sdf.grad, gsdf_e)
    _close(w.grid_sh.grad, gsh_e)


def test_captured_step_follows_parameter_updates(cuda_device):
    """Parameters are read in place: an update between replays is seen."""
    w = pipeline.build_workload("small", cuda_device)
    step = graph.CapturedTrainingStep(w)
    step()
    with torch.no_grad():
        w.grid_sh.mul_(0.5)
    loss = step()
    torch.cuda.synchronize()
    assert step.check()
    loss_e, gsdf_e, gsh_e, _ = _eager(w)
    assert abs(float(loss) - loss_e) <= LOSS_RTOL * abs(loss_e)


def test_captured_step_input_sets_read_their_own_inputs(cuda_device):
    """With two input sets, each graph reads its own batch in place and the
    shared parameters; a replay of one set leaves the other set's outputs as
    they were."""
    w = pipeline.build_workload("small", cuda_device)
    step = graph.CapturedTrainingStep(w, input_sets=2)
    assert len(step.graphs) == 2 and step.launches_per_replay >= 15
    assert step.inputs[1]["grid_sh"] is w.grid_sh  # parameters are shared
    with torch.no_grad():
        step.inputs[1]["target"].mul_(0.75)
    loss0 = float(step(0))
    g0 = step.grad_sh.clone()
    loss1 = float(step(1))
    assert step.check()
    torch.cuda.synchronize()
    # Set 0's outputs survive the replay of set 1.
    torch.testing.assert_close(step._outputs[0][3], g0, rtol=0, atol=0)
    loss_e0, _, gsh_e0, _ = _eager(w)
    assert abs(loss0 - loss_e0) <= LOSS_RTOL * abs(loss_e0)
    _close(g0, gsh_e0)
    with torch.no_grad():
        w.target.mul_(0.75)
    loss_e1, gsdf_e1, gsh_e1, _ = _eager(w)
    assert abs(loss1 - loss_e1) <= LOSS_RTOL * abs(loss_e1)
    _close(step.grad_sdf, gsdf_e1)
    _close(step.grad_sh, gsh_e1)


@pytest.mark.parametrize("config", ["small", "mid", "large"])
def test_deferred_sh_matches_rows_bit_for_bit(cuda_device, config):
    """Colours from the grid SH (no per-vertex rows) equal the rows path, and
    so do the grid gradients: SH through the colours, signed distances and
    positions through the shared contribution list."""
    w = pipeline.build_workload(config, cuda_device)
    args = (w.voxels.vertices, None, w.voxels.neighbors, w.voxels.lower_corners, w.voxels.upper_corners,
            w.voxels.indices, w.level_sets)
    with torch.no_grad():
        _, stats = pipeline.forward(w)
    caps = pipeline.Capacities.around(stats)
    out = {}
    for defer in (False, True):
        gsdf = w.grid_sdf.detach().clone().requires_grad_(True)
        gsh = w.grid_sh.detach().clone().requires_grad_(True)
        a = list(args)
        a[1] = gsh
        tri, counts = te.tessellate_voxels_counted(gsdf, *a, caps.vertices, caps.faces, defer_sh=defer)
        assert isinstance(tri.spherical_harmonics, te.DeferredSH) == defer
        n = int(counts.num_vertices)
        verts = pipeline.uncontract_stand_in(tri.vertices.detach())
        colors = tr.evaluate_spherical_harmonics(verts, tri.spherical_harmonics, w.extrinsics, w.sh_degree)
        gen = torch.Generator(device=cuda_device).manual_seed(5)
        dcol = torch.randn(colors.shape, generator=gen, device=cuda_device)
        dcol[:, n:] = 0
        dsdf = torch.randn(tri.signed_distances.shape, generator=gen, device=cuda_device)
        dpos = torch.randn(tri.vertices.shape, generator=gen, device=cuda_device)
        dsdf[n:] = 0
        dpos[n:] = 0
        (g_sh,) = torch.autograd.grad(colors, gsh, dcol, retain_graph=True)
        g_sdf, = torch.autograd.grad((tri.signed_distances * dsdf).sum() + (tri.vertices * dpos).sum(), gsdf)
        out[defer] = (colors[:, :n].clone(), g_sh, g_sdf)
    for got, want in zip(out[True], out[False]):
        torch.testing.assert_close(got, want, rtol=0, atol=0)
    assert float(out[True][1].abs().max()) > 0


def test_grid_sh_backward_without_scratch_matches_two_pass(cuda_device, monkeypatch):
    """The one-pass grid SH backward (taken when the two-pass form's scratch
    would exceed its limit) gives the two-pass form's bits."""
    w = pipeline.build_workload("small", cuda_device)
    args = (w.voxels.vertices, None, w.voxels.neighbors, w.voxels.lower_corners, w.voxels.upper_corners,
            w.voxels.indices, w.level_sets)
    with torch.no_grad():
        _, stats = pipeline.forward(w)
    caps = pipeline.Capacities.around(stats)
    grads = []
    for limit in (te.GRID_SH_BACKWARD_SCRATCH_LIMIT, 0):
        monkeypatch.setattr(te, "GRID_SH_BACKWARD_SCRATCH_LIMIT", limit)
        gsh = w.grid_sh.detach().clone().requires_grad_(True)
        a = list(args)
        a[1] = gsh
        tri, counts = te.tessellate_voxels_counted(w.grid_sdf.detach(), *a, caps.vertices, caps.faces, defer_sh=True)
        verts = pipeline.uncontract_stand_in(tri.vertices.detach())
        colors = tr.evaluate_spherical_harmonics(verts, tri.spherical_harmonics, w.extrinsics, w.sh_degree)
        dcol = torch.randn(colors.shape, generator=torch.Generator(device=cuda_device).manual_seed(9),
                           device=cuda_device)
        dcol[:, int(counts.num_vertices):] = 0
        grads.append(torch.autograd.grad(colors, gsh, dcol)[0])
    torch.testing.assert_close(grads[1], grads[0], rtol=0, atol=0)
    assert float(grads[0].abs().max()) > 0


def test_captured_step_input_set_with_other_cameras(cuda_device):
    """A batch with other cameras in set 1 (more keys): the step detects an
    overflow if there is one, re-captures with capacities measured over every
    set, and then matches the eager step on that batch."""
    w = pipeline.build_workload("small", cuda_device)
    step = graph.CapturedTrainingStep(w, input_sets=2, margin=1.0)
    closer = w.extrinsics.clone()
    closer[:, 2, 3] *= 0.8  # cameras moved towards the scene: larger images of it, more keys
    with torch.no_grad():
        step.inputs[1]["extrinsics"].copy_(closer)
    for _ in range(3):
        loss1 = step(1)
        torch.cuda.synchronize()
        if step.check():
            break
    assert step.check()
    loss1 = float(loss1)
    g_sdf, g_sh = step.grad_sdf.clone(), step.grad_sh.clone()
    with torch.no_grad():
        w.extrinsics.copy_(closer)
    loss_e, gsdf_e, gsh_e, _ = _eager(w)
    assert abs(loss1 - loss_e) <= LOSS_RTOL * abs(loss_e)
    _close(g_sdf, gsdf_e)
    _close(g_sh, gsh_e)
