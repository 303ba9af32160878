"""The allocation-free exclusive scan, edpp_scan_exclusive_i32_noalloc.

Some callers cannot allocate device memory where they call the scan (inside
a host callback, in a loop that must never touch the allocator, or as a
plugin whose host application owns every device allocation).  This entry
point keeps its look-back state in a fixed 1 MiB device array inside the
library instead of a caller workspace.  The test calls it through the C ABI
twice in a row, with different lengths so that the second call must clear
what the first left in the shared array, and compares each result with the
workspace-taking edpp_scan_exclusive_i32 (LOOKBACK) on the same input.
Integer scans are compared exactly.  This file is named to be collected
last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scan_with_workspace(edpp, torch, x):
    lib = edpp.lib()
    out = torch.empty_like(x)
    n = x.numel()
    ws = edpp.workspace(lib.edpp_scan_workspace_size(n, 0, 0), x.device)
    st = lib.edpp_scan_exclusive_i32(ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(out.data_ptr()),
                                     n, 0, ctypes.c_void_p(ws.data_ptr()), ws.numel(),
                                     edpp.current_stream_handle())
    assert st == 0
    return out


def _scan_noalloc(edpp, torch, x):
    lib = edpp.lib()
    out = torch.full_like(x, -1)
    st = lib.edpp_scan_exclusive_i32_noalloc(ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(out.data_ptr()), x.numel(),
                                             edpp.current_stream_handle())
    assert st == 0
    return out


def test_noalloc_matches_workspace_scan_twice(cuda, edpp):
    torch = cuda
    # first call: a long input (many tiles of look-back state); second call:
    # a shorter one that reuses the front of the same state.
    for n, seed, lo, hi in ((3_000_017, 1, 0, 15), (123_457, 2, 2**30, 2**31 - 1)):
        x = torch.from_numpy(edpp.gen_uniform_i32(n, seed, lo, hi)).cuda()
        ref = _scan_with_workspace(edpp, torch, x)
        got = _scan_noalloc(edpp, torch, x)
        torch.cuda.synchronize()
        assert edpp.sync_status() == edpp.EDPP_OK
        assert torch.equal(got, ref), f"mismatch at n={n}"


def test_noalloc_limit_and_arguments(cuda, edpp):
    lib = edpp.lib()
    max_len = lib.edpp_scan_exclusive_i32_noalloc_max_length()
    assert max_len == ((1 << 20) - 256) // 8 * 4096
    fake = ctypes.c_void_p(16)  # never dereferenced: the size check fails first
    assert lib.edpp_scan_exclusive_i32_noalloc(fake, fake, max_len + 1, None) == edpp.EDPP_EINVAL
    assert lib.edpp_scan_exclusive_i32_noalloc(fake, fake, -1, None) == edpp.EDPP_EINVAL
    assert lib.edpp_scan_exclusive_i32_noalloc(None, None, 0, None) == edpp.EDPP_OK
