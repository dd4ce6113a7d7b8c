"""Bounded device waits give up with a status instead of hanging.

The single-pass scans wait on their predecessors' descriptors with a bounded
spin. A test entry point makes one warp look back over a predecessor that
never publishes; with a small spin limit it must return promptly, record
MT_ERR_DEVICE_TIMEOUT in the workspace status word (where every scan records
it) and fall back to an empty prefix. The context stays usable: a normal scan
on the same stream afterwards is correct.
"""

from __future__ import annotations

import time

import pytest
import torch

pytestmark = pytest.mark.gpu

MT_ERR_DEVICE_TIMEOUT = 5


def test_lookback_wait_times_out_with_status(cuda_device):
    from meshtryoshka_gb300 import _native as nt

    lib = nt.library()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    ws = torch.zeros(4096, dtype=torch.uint8, device=cuda_device)
    prefix = torch.full((1,), -7, dtype=torch.int64, device=cuda_device)
    t0 = time.perf_counter()
    assert lib.mt_test_lookback_timeout(1000, prefix.data_ptr(), ws.data_ptr(), ws.numel(), stream) == 0
    torch.cuda.synchronize(cuda_device)
    elapsed = time.perf_counter() - t0
    status = int(ws[:4].view(torch.int32).item())
    assert status == MT_ERR_DEVICE_TIMEOUT
    assert lib.mt_status_string(status) == b"device spin-wait timed out"
    assert int(prefix) == 0
    assert elapsed < 5.0

    # The context is still usable: a scan on the same stream is correct.
    x = torch.arange(1, 10_001, dtype=torch.int32, device=cuda_device)
    ws2 = torch.zeros(lib.mt_scan_workspace_bytes(x.numel()), dtype=torch.uint8, device=cuda_device)
    assert lib.mt_exclusive_scan_i32(x.data_ptr(), x.numel(), ws2.data_ptr(), ws2.numel(), stream) == 0
    torch.cuda.synchronize(cuda_device)
    assert int(ws2[:4].view(torch.int32).item()) == 0
    assert int(x[-1]) == 9999 * 10000 // 2


def test_lookback_test_entry_rejects_bad_limits(cuda_device):
    from meshtryoshka_gb300 import _native as nt

    lib = nt.library()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    ws = torch.zeros(4096, dtype=torch.uint8, device=cuda_device)
    prefix = torch.zeros(1, dtype=torch.int64, device=cuda_device)
    assert lib.mt_test_lookback_timeout(0, prefix.data_ptr(), ws.data_ptr(), ws.numel(), stream) == 1
    assert lib.mt_test_lookback_timeout((1 << 20) + 1, prefix.data_ptr(), ws.data_ptr(), ws.numel(), stream) == 1
    assert lib.mt_test_lookback_timeout(10, prefix.data_ptr(), ws.data_ptr(), 100, stream) == 3
