"""The allocation-free scan entry point, called through the C ABI.

``mt_exclusive_scan_i32_static`` serves callers that cannot allocate device
memory for scratch (a C/C++ host without its own device allocator, or a host
framework that forbids new device allocations); its scratch is a fixed
``__device__`` array inside the library. It must give exactly the same result
as ``mt_exclusive_scan_i32`` (integer scan: bit-exact), on repeated calls that
reuse the shared array, and must reject sizes beyond its limit.

This file is named to be collected last, so a run that stops at the first
failure has already run every other test.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

MT_ERR_TOO_LARGE = 7


def test_static_scan_matches_workspace_scan_on_consecutive_calls(cuda_device):
    from meshtryoshka_gb300 import _native as nt

    lib = nt.library()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    rng = np.random.default_rng(20)
    # Two calls in a row: a large one, then a smaller one that reuses the
    # shared scratch left behind by the first.
    for n in (3_000_001, 4_097):
        x = torch.from_numpy(rng.integers(0, 16, n).astype(np.int32)).to(cuda_device)
        with_workspace = x.clone()
        without = x.clone()
        ws = torch.zeros(lib.mt_scan_workspace_bytes(n), dtype=torch.uint8, device=cuda_device)
        assert lib.mt_exclusive_scan_i32(with_workspace.data_ptr(), n, ws.data_ptr(), ws.numel(), stream) == 0
        assert lib.mt_exclusive_scan_i32_static(without.data_ptr(), n, stream) == 0
        torch.cuda.synchronize(cuda_device)
        assert torch.equal(with_workspace, without)
        expect = np.concatenate(([0], np.cumsum(x.cpu().numpy().astype(np.int64))[:-1])).astype(np.int32)
        np.testing.assert_array_equal(without.cpu().numpy(), expect)


def test_static_scan_at_its_maximum_size(cuda_device):
    """n equal to the limit uses the last descriptor slot of the fixed array."""
    from meshtryoshka_gb300 import _native as nt

    lib = nt.library()
    n = lib.mt_exclusive_scan_i32_static_max_elements()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    gen = torch.Generator(device=cuda_device).manual_seed(3)
    x = torch.randint(0, 4, (n,), dtype=torch.int32, device=cuda_device, generator=gen)
    host_in = x.cpu().numpy()
    without = x.clone()
    assert lib.mt_exclusive_scan_i32_static(without.data_ptr(), n, stream) == 0
    ws = torch.zeros(lib.mt_scan_workspace_bytes(n), dtype=torch.uint8, device=cuda_device)
    assert lib.mt_exclusive_scan_i32(x.data_ptr(), n, ws.data_ptr(), ws.numel(), stream) == 0  # in place
    torch.cuda.synchronize(cuda_device)
    assert torch.equal(x, without)
    del x, ws
    expect = np.cumsum(host_in, dtype=np.int64)
    expect = np.concatenate(([0], expect[:-1])).astype(np.int32)
    np.testing.assert_array_equal(without.cpu().numpy(), expect)


def test_static_scan_status_word_reads_ok(cuda_device):
    from meshtryoshka_gb300 import _native as nt

    lib = nt.library()
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    x = torch.ones(100_000, dtype=torch.int32, device=cuda_device)
    assert lib.mt_exclusive_scan_i32_static(x.data_ptr(), x.numel(), stream) == 0
    status = torch.full((1,), -1, dtype=torch.int32, device=cuda_device)
    assert lib.mt_exclusive_scan_i32_static_status(status.data_ptr(), stream) == 0
    torch.cuda.synchronize(cuda_device)
    assert int(status) == 0
    assert int(x[-1]) == x.numel() - 1


def test_static_scan_rejects_sizes_beyond_its_limit(cuda_device):
    from meshtryoshka_gb300 import _native as nt

    lib = nt.library()
    limit = lib.mt_exclusive_scan_i32_static_max_elements()
    assert limit == 1 << 26
    x = torch.zeros(16, dtype=torch.int32, device=cuda_device)
    stream = torch.cuda.current_stream(cuda_device).cuda_stream
    status = lib.mt_exclusive_scan_i32_static(x.data_ptr(), limit + 1, stream)
    assert status == MT_ERR_TOO_LARGE
    assert lib.mt_status_string(status) == b"size exceeds the static scratch limit"
    torch.cuda.synchronize(cuda_device)
    assert int(x.abs().sum()) == 0  # nothing was launched
