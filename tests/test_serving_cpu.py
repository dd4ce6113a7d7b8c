"""Host logic of the serving loop: how the next batch is formed.

``Server._form_batch`` takes requests of the queue head's scene and kind
(render-only, or render + gradient) in arrival order, up to the batch limit of
that kind, while their estimated bytes fit the budget left by the batches in
flight; the head goes alone when nothing is in flight even if it exceeds the
budget; the requests it passes over keep their order at the front of the
queue, and it looks ahead a bounded distance. No GPU: the scenes are stubs
that estimate a request's bytes from its pixels.
"""

from __future__ import annotations

from collections import deque

from meshtryoshka_gb300 import serving

BYTES_PER_PIXEL = 10


class _StubScene:
    def measure_keys_per_pixel(self) -> float:
        return 1.0

    def request_bytes(self, r: serving.Request) -> int:
        return BYTES_PER_PIXEL * r.pixels


def _server(**kw) -> serving.Server:
    return serving.Server([_StubScene(), _StubScene()], **kw)


def _req(i: int, scene: int, gradient: bool = False, shape=(10, 10)) -> serving.Request:
    return serving.Request(i, scene, None, None, shape, gradient, None, float(i))


def _ids(requests) -> list[int]:
    return [r.id for r in requests]


def test_batch_takes_the_heads_scene_and_kind_in_order():
    s = _server(max_batch=4)
    q = deque([_req(0, 0), _req(1, 0, True), _req(2, 1), _req(3, 0), _req(4, 0), _req(5, 0), _req(6, 0)])
    batch, used = s._form_batch(q, budget=1 << 30, idle=True)
    assert _ids(batch) == [0, 3, 4, 5]  # max_batch render requests of scene 0
    assert used == 4 * BYTES_PER_PIXEL * 100
    assert _ids(q) == [1, 2, 6]  # the passed-over requests stay in front, in order


def test_gradient_batches_have_their_own_limit():
    s = _server(max_batch=8, max_gradient_batch=2)
    q = deque([_req(0, 1, True), _req(1, 1, True), _req(2, 1, True), _req(3, 1)])
    batch, _ = s._form_batch(q, budget=1 << 30, idle=True)
    assert _ids(batch) == [0, 1]
    assert _ids(q) == [2, 3]


def test_budget_bounds_the_batch():
    s = _server(max_batch=8)
    one = BYTES_PER_PIXEL * 100
    q = deque([_req(i, 0) for i in range(5)])
    batch, used = s._form_batch(q, budget=2 * one + one // 2, idle=False)
    assert _ids(batch) == [0, 1] and used == 2 * one
    assert _ids(q) == [2, 3, 4]


def test_head_over_budget_goes_alone_only_when_idle():
    s = _server(max_batch=8)
    big = _req(0, 0, shape=(100, 100))  # 100,000 bytes
    q = deque([big, _req(1, 0)])
    batch, used = s._form_batch(q, budget=5_000, idle=False)
    assert batch == [] and used == 0
    assert _ids(q) == [0, 1]  # nothing taken, order kept
    batch, used = s._form_batch(q, budget=5_000, idle=True)
    assert _ids(batch) == [0] and used == BYTES_PER_PIXEL * 10_000
    assert _ids(q) == [1]


def test_look_ahead_is_bounded():
    s = _server(max_batch=2)
    others = [_req(i, 1) for i in range(1, 1 + 4 * 2 + 1)]  # one more than the look-ahead allows
    late = _req(100, 0)
    q = deque([_req(0, 0), *others, late])
    batch, _ = s._form_batch(q, budget=1 << 30, idle=True)
    assert _ids(batch) == [0]  # the scan stopped before reaching the late request of scene 0
    assert _ids(q) == [r.id for r in others] + [100]
