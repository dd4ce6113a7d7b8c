"""ctypes binding of ``libmtgb.so`` (the C ABI in ``include/meshtryoshka_gb300.h``).

This module is the only place Python touches the native library. It

* loads the library (building it first with nvcc if it is missing or stale),
* declares every entry point's argument types,
* turns a non-zero ``mt_status`` into ``RuntimeError`` (the library's
  equivalent of the reference's ``TORCH_CHECK`` failures), and
* owns the per-device scratch workspaces the library asks callers to supply.

There is no fallback: if the CUDA library cannot be loaded, importing the
render path fails.
"""

from __future__ import annotations

import contextlib
import ctypes
import threading
from ctypes import c_float, c_int32, c_int64, c_size_t, c_uint64, c_void_p

import torch

from . import build as _build

P = c_void_p
I32 = c_int32
I64 = c_int64

# name -> (restype, argtypes)
_SIGNATURES: dict[str, tuple[object, list[object]]] = {
    "mt_status_string": (ctypes.c_char_p, [I32]),
    "mt_version": (I32, []),
    "mt_scan_workspace_bytes": (c_size_t, [I64]),
    "mt_exclusive_scan_i32": (I32, [P, I64, P, c_size_t, P]),
    "mt_exclusive_scan_i64": (I32, [P, I64, P, c_size_t, P]),
    "mt_inclusive_scan_i32_to_i64": (I32, [P, P, I64, P, c_size_t, P]),
    "mt_exclusive_scan_i32_static": (I32, [P, I64, P]),
    "mt_exclusive_scan_i32_static_max_elements": (I64, []),
    "mt_exclusive_scan_i32_static_status": (I32, [P, P]),
    "mt_test_lookback_timeout": (I32, [I32, P, P, c_size_t, P]),
    "mt_compute_vertex_occupancy": (I32, [P, I32, I32, I32, P, P, P]),
    "mt_count_occupancy": (I32, [P, I32, I32, I32, P, P]),
    "mt_create_voxels": (I32, [P, P, P, P, I32, I32, I32, I64, I64, P, P, P, P, P, P]),
    "mt_dilate_occupancy": (I32, [P, I32, I32, I32, I32, P, P]),
    "mt_write_occupancy": (I32, [P, I64, P, I64, P]),
    "mt_upscale_occupancy": (I32, [P, P, I32, I32, I32, I32, I32, I32, P, P]),
    "mt_upscale_parameters": (I32, [P, P, P, P, I32, I64, I32, I32, I32, P, P, I32, I32, I32, I64, P, P, P]),
    "mt_count_occupancy_mesh_triangles": (I32, [P, I32, I32, I32, P, P]),
    "mt_create_occupancy_mesh_triangles": (I32, [P, I32, I32, I32, P, I64, P, P, P, P]),
    "mt_quantize_points": (I32, [P, I64, c_float, P, P, P]),
    "mt_pack_point_keys": (I32, [P, I64, I32, P, P, P]),
    "mt_iota_i32": (I32, [I64, P, P]),
    "mt_index_sorted_runs": (I32, [P, P, I64, P, P]),
    "mt_count_triangle_vertices": (I32, [P, P, I64, P, I32, P, P]),
    "mt_create_triangle_vertices": (
        I32,
        [P, P, P, I32, P, I64, P, I32, P, I64, P, P, P, P, P, P, P],
    ),
    "mt_create_triangle_vertices_live_t_backward": (I32, [P, P, P, I32, I64, P, I64, P, P, P, P, P]),
    "mt_create_triangle_vertices_backward": (
        I32,
        [P, I32, P, I64, P, I32, P, P, P, P, I64, P, P, P, P, P, c_size_t, P],
    ),
    "mt_create_triangle_vertices_backward_workspace_bytes": (c_size_t, [I64, I64]),
    "mt_count_triangle_faces": (I32, [P, P, I64, P, I64, P, I32, P, P, P]),
    "mt_compute_sdf_regularizers": (I32, [P, P, P, I64, P, I64, I32, I32, I32, P, P, P, P]),
    "mt_compute_sdf_regularizers_backward": (I32, [P, P, P, I64, P, I64, I32, I32, I32, P, P, P, P, P]),
    "mt_create_triangle_faces": (
        I32,
        [P, P, I64, I64, I64, P, P, P, I32, P, I64, P, P, P],
    ),
    "mt_shell_boundaries": (I32, [P, I64, P, I64, I32, P, P, P, P]),
    "mt_vertex_grad_list_max_shells": (I32, []),
    "mt_build_vertex_grad_list_workspace_bytes": (c_size_t, [I64]),
    "mt_build_vertex_grad_list": (I32, [P, P, I64, P, I32, P, I64, P, P, P, P, c_size_t, P]),
    "mt_vertex_grads_from_list": (I32, [P, P, I64, P, P, P, P, P]),
    "mt_grid_sh_colors": (I32, [P, I32, I64, P, I64, P, P, I32, P, I32, P, P]),
    "mt_grid_sh_colors_backward_workspace_bytes": (c_size_t, [I64]),
    "mt_grid_sh_colors_backward": (I32, [P, P, I64, I64, P, I32, I32, P, I32, P, P, P, P, P, c_size_t, P]),
    "mt_capacity_overflow": (I32, [P, I64, P, I64, P, I64, P, P]),
    "mt_sort_pairs_workspace_bytes": (c_size_t, [I64]),
    "mt_sort_pairs_i64_i32": (I32, [P, P, P, P, I64, P, I32, I32, P, c_size_t, P]),
    "mt_camera_positions": (I32, [P, I32, P, P]),
    "mt_project_vertices": (I32, [P, I64, P, P, I32, P, P, P]),
    "mt_evaluate_spherical_harmonics": (I32, [P, I64, P, I32, I32, P, I32, P, P]),
    "mt_evaluate_spherical_harmonics_backward": (I32, [P, I64, I32, I32, P, I32, P, P, P, P]),
    "mt_bound_triangles": (I32, [P, P, I64, P, I64, P, I32, I32, I32, I32, I32, P, c_float, P, P, P, P]),
    "mt_generate_keys": (I32, [P, I64, P, I64, P, I32, P, P, P, I32, I32, P, P, I64, P, P, P]),
    "mt_bound_and_generate_keys_workspace_bytes": (c_size_t, [I64]),
    "mt_bound_and_generate_keys": (
        I32,
        [P, P, I64, P, I64, P, P, I32, I32, I32, I32, I32, I32, P, c_float, P, I64, P, P, P, P, c_size_t, P],
    ),
    "mt_delineate_tiles": (I32, [P, I64, P, P, I32, I32, I32, I64, P, P]),
    "mt_sort_keys_by_tile_supported": (I32, [P, I32, I32, I64]),
    "mt_sort_keys_by_tile_workspace_bytes": (c_size_t, [I64, I64]),
    "mt_sort_keys_by_tile": (I32, [P, P, I64, P, P, I32, I32, I32, I64, P, P, P, P, c_size_t, P]),
    "mt_intersect_and_composite_forward": (
        I32,
        [P, P, P, I64, P, P, P, P, I64, P, P, I32, I32, I32, I32, I32, I32, I32, I32, P, P, I64, P, P, P, P, P,
         c_float, P, P, c_size_t, P, c_size_t, I32, P],
    ),
    "mt_composite_hit_bits_bytes": (c_size_t, [I64, I32, I32, I64]),
    "mt_composite_tile_order_bytes": (c_size_t, [I64]),
    "mt_intersect_and_composite_backward": (
        I32,
        [P, P, P, I64, P, P, P, P, I64, P, I32, I32, I32, I32, I32, I32, I32, I32, P, P, I64, P, P, P, P, P, P,
         c_float, P, I32, P, P, P, I32, P, c_size_t, P, c_size_t, P, c_size_t, I32, P],
    ),
    "mt_composite_staging_bytes": (c_size_t, [I32, I64]),
    "mt_ssaa_loss": (I32, [P, I32, I32, I32, I32, P, P, c_float, P, P, P]),
    "mt_intersect": (I32, [P, I64, P, P, P, I32, I32, I32, I32, I32, I32, I32, I32, P, P, P]),
    "mt_interpolate": (I32, [P, P, I32, I32, I32, I32, P, P, P, I64, P, P, P]),
    "mt_interpolate_backward": (I32, [P, P, I32, I32, I32, I32, P, I64, P, P, P, P, P]),
    "mt_composite": (I32, [P, P, P, I64, I32, P, P, P, P]),
    "mt_composite_backward": (I32, [P, P, P, I64, I32, P, P, P, P, P, P, P, P, I32, P]),
}

_lib = None
_lock = threading.Lock()


def _load():
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        path = _build.LIBRARY
        if not path.exists() or _build._stale(path, _build.sources() + _build.headers()):
            _build.build()
        lib = ctypes.CDLL(str(path))
        for name, (restype, argtypes) in _SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = restype
            fn.argtypes = argtypes
        _lib = lib
        return lib


def library():
    """The loaded ctypes library (loads / builds on first use)."""
    return _load()


def library_path() -> str:
    return str(_build.LIBRARY)


# Kernels each entry point enqueues (memsets excluded); used to count this
# library's launches, e.g. inside a benchmark's timed region.
KERNELS_PER_CALL = {
    "mt_sort_pairs_i64_i32": 11,  # histogram, plan, 8 digit passes, copy
    "mt_create_voxels": 1,
    "mt_create_triangle_vertices": 2,  # vertices + source records, SH rows (1 without the rows)
    "mt_create_triangle_vertices_backward": 5,  # corner inverse, count, scan, list + grads, SH gather
    "mt_intersect_and_composite_forward": 4,  # warp masks, tile-order histogram and scatter, composite
    "mt_sort_keys_by_tile": 7,  # count, scan, tile ranges, scatter, tiny / medium / small / large bin sorts
    "mt_bound_and_generate_keys": 3,  # rectangles + chunk counts, chunk scan, keys
    "mt_build_vertex_grad_list": 4,  # corner inverse, count, scan, fill
    "mt_grid_sh_colors_backward": 2,  # per-vertex SH gradients, per-grid-vertex sums
}


class LaunchRecorder:
    """Counts library kernel launches and optionally times every entry point
    with CUDA events on the stream it was enqueued on. A timed call is
    preceded by a short device-side sleep on that stream, so that the start
    event fires only once the host has enqueued the call's kernels: the
    recorded time is device time, without the host's enqueue overhead."""

    SLEEP_CYCLES = 200_000  # about 0.1 ms at 2 GHz, more than one call's host overhead

    def __init__(self, timed: bool = False):
        self.launches = 0
        self.calls: dict[str, int] = {}
        self.timed = timed
        self.events: dict[str, list[tuple[torch.cuda.Event, torch.cuda.Event]]] = {}

    def times_ms(self) -> dict[str, list[float]]:
        return {k: [a.elapsed_time(b) for a, b in v] for k, v in self.events.items()}


_recorder: LaunchRecorder | None = None


@contextlib.contextmanager
def record_launches(timed: bool = False):
    global _recorder
    previous = _recorder
    _recorder = LaunchRecorder(timed)
    try:
        yield _recorder
    finally:
        _recorder = previous


def call(name: str, *args, launches: int | None = None) -> None:
    """Call an entry point and raise RuntimeError on a non-zero status.
    ``launches``: kernels this call enqueues, when it differs from the entry
    point's usual count (``KERNELS_PER_CALL``)."""
    lib = _load()
    rec = _recorder
    if rec is not None:
        rec.launches += KERNELS_PER_CALL.get(name, 1) if launches is None else launches
        rec.calls[name] = rec.calls.get(name, 0) + 1
        if rec.timed:
            start = torch.cuda.Event(enable_timing=True)
            end = torch.cuda.Event(enable_timing=True)
            torch.cuda._sleep(rec.SLEEP_CYCLES)
            start.record()
    status = getattr(lib, name)(*args)
    if rec is not None and rec.timed:
        end.record()
        rec.events.setdefault(name, []).append((start, end))
    if status != 0:
        msg = lib.mt_status_string(status).decode()
        raise RuntimeError(f"{name} failed: {msg} (status {status})")


def ptr(t: torch.Tensor | None) -> int | None:
    """Device pointer of a contiguous tensor (None -> NULL)."""
    if t is None:
        return None
    if not t.is_contiguous():
        raise ValueError("meshtryoshka_gb300 kernels require contiguous tensors")
    return t.data_ptr() if t.numel() > 0 else None


def stream(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def require_cuda(*tensors: torch.Tensor) -> torch.device:
    device = None
    for t in tensors:
        if t is None:
            continue
        if t.device.type != "cuda":
            raise ValueError(
                "meshtryoshka_gb300 runs on CUDA tensors only (got a tensor on "
                f"{t.device}); there is no CPU path"
            )
        if device is None:
            device = t.device
        elif t.device != device:
            raise ValueError("all tensors must be on the same CUDA device")
    if device is None:
        raise ValueError("no CUDA tensor given")
    return device


class Workspace:
    """Growable per-device scratch buffer handed to the library.

    Byte 0 holds the library's device status word, zeroed on allocation.
    Calls that use a workspace are stream-ordered, so one workspace per device
    is shared by all calls on that device's current stream.
    """

    def __init__(self, device: torch.device):
        self.device = device
        self.buffer = torch.zeros(0, dtype=torch.uint8, device=device)

    def get(self, nbytes: int) -> tuple[int, int]:
        nbytes = max(int(nbytes), 256)
        if self.buffer.numel() < nbytes:
            grow = max(nbytes, int(self.buffer.numel() * 1.5))
            grow = (grow + 4095) // 4096 * 4096
            self.buffer = torch.zeros(grow, dtype=torch.uint8, device=self.device)
        return self.buffer.data_ptr(), self.buffer.numel()

    def status(self) -> int:
        """Device status word (synchronizes the current stream)."""
        if self.buffer.numel() < 4:
            return 0
        return int(self.buffer[:4].view(torch.int32).item())

    def check(self) -> None:
        code = self.status()
        if code != 0:
            self.buffer[:4].zero_()
            msg = _load().mt_status_string(code).decode()
            raise RuntimeError(f"device-side failure: {msg} (status {code})")


_workspaces: dict[tuple[int, int], Workspace] = {}


def workspace(device: torch.device) -> Workspace:
    index = device.index if device.index is not None else torch.cuda.current_device()
    key = (index, torch.cuda.current_stream(device).cuda_stream)
    ws = _workspaces.get(key)
    if ws is None:
        ws = Workspace(device)
        _workspaces[key] = ws
    return ws


__all__ = [
    "library",
    "library_path",
    "call",
    "ptr",
    "stream",
    "require_cuda",
    "workspace",
    "Workspace",
    "c_float",
    "c_uint64",
]
