"""The allocation-free exclusive scan, edpp_scan_exclusive_i32_noalloc.

Some callers cannot allocate device memory where they call the scan: a host
thread that must never enter the device allocator (a real-time loop that
cannot afford its latency or implicit synchronisation), or a plugin whose
host application owns every device allocation.  This entry point keeps its
look-back state in a fixed 1 MiB device array inside the library instead of
a caller workspace.

The tests call it through the C ABI twice in a row, with different lengths
so that the second call must clear what the first left in the shared array,
and compare each result with the oracle's sequential scan and with the
workspace-taking edpp_scan_exclusive_i32 (LOOKBACK) on the same input.
Integer scans are compared exactly.  A further test checks the defining
property: after a warm-up call, calls at the maximum length leave the
device's free memory unchanged; another captures one call in a CUDA graph
and replays it.  This file is named to be collected last.
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


def _scan_noalloc(edpp, torch, x, out=None):
    lib = edpp.lib()
    if out is None:
        out = torch.full_like(x, -1)
    st = lib.edpp_scan_exclusive_i32_noalloc(ctypes.c_void_p(x.data_ptr()),
                                             ctypes.c_void_p(out.data_ptr()), x.numel(),
                                             edpp.current_stream_handle())
    assert st == 0
    return out


def test_noalloc_matches_oracle_and_workspace_scan_twice(cuda, edpp, orc):
    torch = cuda
    # first call: a long input (many tiles of look-back state); second call:
    # a shorter one that reuses the front of the same state.
    for n, seed, lo, hi in ((3_000_017, 1, 0, 15), (123_457, 2, 2**30, 2**31 - 1)):
        h = edpp.gen_uniform_i32(n, seed, lo, hi)
        x = torch.from_numpy(h).cuda()
        ref = _scan_with_workspace(edpp, torch, x)
        got = _scan_noalloc(edpp, torch, x)
        torch.cuda.synchronize()
        assert edpp.sync_status() == edpp.EDPP_OK
        expect = orc.scan(h, False)
        assert np.array_equal(got.cpu().numpy(), expect), f"differs from the oracle at n={n}"
        assert torch.equal(got, ref), f"differs from the workspace scan at n={n}"


def test_noalloc_leaves_free_memory_unchanged(cuda, edpp, orc):
    torch = cuda
    lib = edpp.lib()
    n = lib.edpp_scan_exclusive_i32_noalloc_max_length()
    h = edpp.gen_uniform_i32(n, 3, 0, 7)
    x = torch.from_numpy(h).cuda()
    out = torch.empty_like(x)
    _scan_noalloc(edpp, torch, x, out)  # warm-up: module load, fault word, address lookup
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(3):
        _scan_noalloc(edpp, torch, x, out)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert edpp.sync_status() == edpp.EDPP_OK
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    # the full-length result, checked through its closed form on the device:
    # consecutive differences give back the input, and the last element plus
    # the last input is the wrapping total
    assert torch.equal(out[1:] - out[:-1], x[:-1])
    total = int(np.sum(h.astype(np.int64))) & 0xFFFFFFFF
    last = (int(out[-1].item()) + int(h[-1])) & 0xFFFFFFFF
    assert out[0].item() == 0 and last == total


def test_noalloc_in_cuda_graph(cuda, edpp, orc):
    # after a warm-up call, one call is captured in a CUDA graph (its look-back
    # state clear and its kernel); each replay must give the workspace scan's
    # result again, on fresh input written into the same buffer
    torch = cuda
    n = 2_000_003
    x = torch.from_numpy(edpp.gen_uniform_i32(n, 4, -1000, 1000)).cuda()
    out = torch.full_like(x, -1)
    _scan_noalloc(edpp, torch, x, out)  # warm-up outside the capture
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        with torch.cuda.graph(g):
            _scan_noalloc(edpp, torch, x, out)
    torch.cuda.current_stream().wait_stream(s)
    for seed in (5, 6):
        h = edpp.gen_uniform_i32(n, seed, -1000, 1000)
        x.copy_(torch.from_numpy(h))
        out.fill_(-1)
        g.replay()
        torch.cuda.synchronize()
        assert edpp.sync_status() == edpp.EDPP_OK
        assert np.array_equal(out.cpu().numpy(), orc.scan(h, False)), f"replay with seed {seed}"
        assert torch.equal(out, _scan_with_workspace(edpp, torch, x))


def test_noalloc_limit_and_arguments(cuda, edpp):
    lib = edpp.lib()
    max_len = lib.edpp_scan_exclusive_i32_noalloc_max_length()
    assert max_len == ((1 << 20) - 256) // 8 * 4096
    fake = ctypes.c_void_p(16)  # never dereferenced: the size check fails first
    assert lib.edpp_scan_exclusive_i32_noalloc(fake, fake, max_len + 1, None) == edpp.EDPP_EINVAL
    assert lib.edpp_scan_exclusive_i32_noalloc(fake, fake, -1, None) == edpp.EDPP_EINVAL
    assert lib.edpp_scan_exclusive_i32_noalloc(None, None, 0, None) == edpp.EDPP_OK
