"""Optional recording of a step's intermediate buffers.

Inside ``with recording(store):`` the tessellation and render entry points
put references to their intermediate device tensors into ``store`` (no copies,
no host reads): vertex and face offsets, faces and voxel indices, the sorted
keys and their triangles, the tile ranges and the compositing output. A
captured training step records once at capture time; its buffers belong to
the graph and every replay overwrites them in place, so after a replay the
recorded tensors hold that replay's values. Used by the parity tests to
compare the timed form of the step with the oracle stage by stage.
"""

from __future__ import annotations

from contextlib import contextmanager

_ACTIVE: list[dict] = []


@contextmanager
def recording(store: dict):
    _ACTIVE.append(store)
    try:
        yield store
    finally:
        _ACTIVE.pop()


def note(**tensors) -> None:
    """Adds ``tensors`` to the innermost active store, if any."""
    if _ACTIVE:
        _ACTIVE[-1].update(tensors)
