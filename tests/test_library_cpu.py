"""The C-ABI library builds, loads, and exports every symbol the header
declares (no GPU needed, no compute calls)."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_symbols() -> list[str]:
    names = []
    for h in HEADERS:
        text = h.read_text()
        names += re.findall(r"^MT_API\s+[\w\s\*]+?\b(mt_\w+)\s*\(", text, re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "mt_exclusive_scan_i32" in names
    assert len(names) >= 10


def test_library_exports_every_declared_symbol():
    from meshtryoshka_gb300 import build

    path = build.build()
    lib = ctypes.CDLL(str(path))
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_header():
    from meshtryoshka_gb300 import _native

    missing = [n for n in declared_symbols() if n not in _native._SIGNATURES]
    assert not missing, f"declared but not bound in _native: {missing}"


def test_status_strings_without_gpu():
    from meshtryoshka_gb300 import _native

    lib = _native.library()
    assert lib.mt_status_string(0) == b"ok"
    assert lib.mt_status_string(5) == b"device spin-wait timed out"
    assert lib.mt_version() >= 1
    assert lib.mt_scan_workspace_bytes(0) >= 256


def test_cpu_tensors_are_rejected():
    import torch

    from meshtryoshka_gb300 import triangle_extraction as te

    with pytest.raises(ValueError, match="CUDA"):
        te.count_occupancy(torch.zeros((2, 2, 1), dtype=torch.int32))


def test_ragged_camera_table():
    """Per-camera grids, first tiles and first output elements of a batch of
    cameras with different image sizes."""
    from meshtryoshka_gb300 import triangle_rasterization as tr

    grid = tr.TileGrid.for_cameras((16, 16), [(75, 101), (128, 64), (40, 200)], 4)
    assert grid.image_shape == (128, 200) and grid.grid_shape == (8, 13)
    assert grid.camera_grids() == [(5, 7), (8, 4), (3, 13)]
    assert grid.camera_tiles == 35 + 32 + 39
    assert grid.output_numel == 4 * (75 * 101 + 128 * 64 + 40 * 200)
    table = tr._camera_table(grid, "cpu").tolist()
    assert table == [[5, 7, 75, 101, 0, 0], [8, 4, 128, 64, 35, 4 * 75 * 101],
                     [3, 13, 40, 200, 67, 4 * (75 * 101 + 128 * 64)]]
    assert tr._camera_table(tr.TileGrid((16, 16), (64, 64), 2, 3), "cpu") is None


def test_compositing_buffer_sizes_without_gpu():
    """The compositing scratch sizes (host-only calls): the hit-bit store is a
    header (the bump counter and one int32 first batch per work item, rounded
    to 128 bytes) plus a 128-byte line per batch; the tile order holds 512
    int32 bucket counts and cursors plus one index per tile; the staging
    scratch a 128-byte header plus a 32-byte record per (camera, vertex)."""
    from meshtryoshka_gb300 import _native

    lib = _native.library()
    for tiles, th, tw, batches in ((40_000, 8, 8, 95_000), (1, 16, 16, 1), (10_001, 4, 8, 3)):
        items = tiles * ((th * tw + 31) // 32)
        header = (8 + 4 * items + 127) // 128 * 128
        assert lib.mt_composite_hit_bits_bytes(tiles, th, tw, batches) == header + 128 * batches
    assert lib.mt_composite_hit_bits_bytes(0, 8, 8, 10) == 0
    assert lib.mt_composite_hit_bits_bytes(10, 8, 8, 0) == 0
    assert lib.mt_composite_tile_order_bytes(40_000) == (512 + 40_000) * 4
    assert lib.mt_composite_tile_order_bytes(0) == 512 * 4
    assert lib.mt_composite_staging_bytes(4, 1000) == 128 + 32 * 4 * 1000
    assert lib.mt_composite_staging_bytes(0, 1000) == 0
