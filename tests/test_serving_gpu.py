"""The serving loop: every request's result is the same alone and in the mix.

Requests for two resident scenes (render-only and render + gradient, images
of 256-1920 x 256-1080 px) arrive faster than they are served, so the server
batches render-only requests of a scene into one pass over cameras of
different sizes and overlaps batches on several streams. Each completed
request is then recomputed on its own: images must be identical, gradients
within 1e-4 of the largest entry (atomic accumulation order).
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
    server = serving.Server(scenes, streams=3, max_batch=8)
    done = server.run(requests)
    torch.cuda.synchronize()
    assert sorted(c.request.id for c in done) == [r.id for r in requests]
    assert server.batches < len(requests)  # render-only requests were batched
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


def test_memory_budget_limits_inflight_pixels(scenes):
    """A pixel budget of one large image still serves every request."""
    requests = serving.poisson_requests(scenes, rate=4000.0, duration=0.01, seed=2, gradient_fraction=0.0)
    server = serving.Server(scenes, streams=4, max_batch=16, max_pixels=1920 * 1080)
    done = server.run(requests)
    assert len(done) == len(requests)
