"""The serving loop: every request's result is the same alone and in the mix.

Requests for two resident scenes (render-only and render + gradient, images
of 256-1920 x 256-1080 px) arrive faster than they are served, so the server
batches render-only requests of a scene into one pass over cameras of
different sizes, batches render + gradient requests of a scene over one
shared tessellation, and overlaps batches on several streams. Each completed
request is then recomputed on its own: images must be identical, gradients
within 1e-4 of the largest entry (atomic accumulation order). The in-flight
byte estimate never exceeds the server's HBM budget (except for a request
served alone that exceeds it by itself).
"""

from __future__ import annotations

import pytest
import torch

from meshtryoshka_gb300 import serving

pytestmark = pytest.mark.gpu


def _close(got, want, rtol=1e-4):
    scale = max(float(want.abs().max()), 1e-30)
    err = float((got - want).abs().max())
    assert err <= rtol * scale, f"max abs err {err:.3e} > {rtol:g} x {scale:.3e}"


@pytest.fixture(scope="module")
def scenes(cuda_device):
    return [serving.Scene.build("serve_128", cuda_device), serving.Scene.build("serve_128", cuda_device, seed=3)]


def test_results_same_alone_and_in_the_mix(scenes):
    requests = serving.poisson_requests(scenes, rate=4000.0, duration=0.02, seed=11, gradient_fraction=0.25)
    assert len(requests) > 40 and any(r.gradient for r in requests)
    server = serving.Server(scenes, streams=3, max_batch=8, overlap_backlog=2)
    done = server.run(requests)
    torch.cuda.synchronize()
    assert sorted(c.request.id for c in done) == [r.id for r in requests]
    assert server.batches < len(requests)  # requests were batched
    for c in done:
        assert c.done >= c.request.arrival
        alone = serving.render_alone(scenes[c.request.scene], c.request)
        assert c.image.shape == (3, *c.request.shape)
        torch.testing.assert_close(c.image, alone.image, rtol=0, atol=0)
        if c.request.gradient:
            _close(c.grad_sdf, alone.grad_sdf)
            _close(c.grad_sh, alone.grad_sh)
        else:
            assert c.grad_sdf is None


def test_plain_form_serves_everything(scenes):
    requests = serving.poisson_requests(scenes, rate=500.0, duration=0.02, seed=5)
    done = serving.run_plain(scenes, requests)
    assert [c.request.id for c in done] == [r.id for r in requests]
    summary = serving.latency_summary(done)
    assert summary["requests"] == len(requests) and summary["p99_ms"] >= summary["p50_ms"] > 0


def test_gradient_requests_share_one_tessellation(scenes):
    """A batch of render + gradient requests of one scene gives each
    request's own gradients."""
    requests = [r for r in serving.poisson_requests(scenes, rate=4000.0, duration=0.05, seed=8,
                                                    gradient_fraction=1.0) if r.scene == 0][:3]
    assert len(requests) == 3
    batch = serving.render_gradient_batch(scenes[0], requests)
    for c in batch:
        alone = serving.render_alone(scenes[0], c.request)
        torch.testing.assert_close(c.image, alone.image, rtol=0, atol=0)
        _close(c.grad_sdf, alone.grad_sdf)
        _close(c.grad_sh, alone.grad_sh)


def test_memory_budget_bounds_the_bytes_in_flight(scenes):
    """With a budget of a few requests' worth of bytes, the in-flight
    estimate stays within it and every request is served."""
    requests = serving.poisson_requests(scenes, rate=4000.0, duration=0.02, seed=2, gradient_fraction=0.2)
    sizes = [scenes[r.scene].request_bytes(r) for r in requests]
    budget = 3 * max(sizes)
    server = serving.Server(scenes, streams=4, max_batch=16, hbm_budget=budget)
    done = server.run(requests)
    assert len(done) == len(requests)
    assert 0 < server.peak_inflight_bytes <= budget
    # A budget below one request still serves (one request at a time).
    tight = serving.Server(scenes, streams=4, max_batch=16, hbm_budget=min(sizes) // 2)
    assert len(tight.run(requests[:10])) == 10
    assert tight.peak_inflight_bytes <= max(sizes[:10])
