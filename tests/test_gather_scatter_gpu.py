"""GPU multi-pass gather / scatter against the oracle (bit-exact), and against
the reference's own CUDA kernels where their cubins were built."""
import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

PASSES = [1, 2, 4, 8, 16]


METHODS = ["sweep", "partition", "tiled", "auto"]


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("n", [1, 2, 3, 5, 17, 1000, 4096 + 3, 100003, (1 << 20) + 1])
@pytest.mark.parametrize("passes", PASSES)
def test_permutation(cuda, edpp, orc, method, n, passes):
    loc = edpp.gen_permutation(n, 2)
    inp = edpp.gen_uniform_i32(n, 4, -2**31, 2**31 - 1)
    g = to_host(edpp.gather(to_dev(inp), to_dev(loc), passes, method=method))
    np.testing.assert_array_equal(g, orc.gather(inp, loc, passes))
    s = to_host(edpp.scatter(to_dev(inp), to_dev(loc), passes, method=method))
    np.testing.assert_array_equal(s, orc.scatter(inp, loc, passes))


@pytest.mark.parametrize("n", [1, 1000, 1 << 22, (1 << 22) + 13])
@pytest.mark.parametrize("passes", [0, 3, 64, 2048, 5000])
def test_partition_window_counts(cuda, edpp, orc, n, passes):
    # pass 0 sizes windows to L2; large pass counts clamp the window count
    loc = edpp.gen_permutation(n, 5)
    inp = edpp.gen_uniform_i32(n, 4, -2**31, 2**31 - 1)
    g = to_host(edpp.gather(to_dev(inp), to_dev(loc), passes, method="partition"))
    np.testing.assert_array_equal(g, inp[loc])
    s = to_host(edpp.scatter(to_dev(inp), to_dev(loc), passes, method="partition"))
    e = np.zeros(n, np.int32)
    e[loc] = inp
    np.testing.assert_array_equal(s, e)


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("passes", [1, 3, 16])
def test_non_permutation_and_invalid_indices(cuda, edpp, orc, method, passes):
    # repeated indices (gather only: a scatter with duplicates races, as in
    # the reference) and indices outside [0,n), which every pass skips
    n = 70001
    loc = edpp.gen_uniform_i32(n, 6, -50, n + 50)
    inp = np.arange(n, dtype=np.int32)
    out0 = np.full(n, -7, np.int32)
    g = to_host(edpp.gather(to_dev(inp), to_dev(loc), passes, out=to_dev(out0), method=method))
    np.testing.assert_array_equal(g, orc.gather(inp, loc, passes, out=out0))
    # scatter through a permutation with some indices made invalid
    perm = edpp.gen_permutation(n, 8)
    perm[::13] = -1
    perm[5::17] = n + 3
    s = to_host(edpp.scatter(to_dev(inp), to_dev(perm), passes, out=to_dev(out0), method=method))
    np.testing.assert_array_equal(s, orc.scatter(inp, perm, passes, out=out0))


@pytest.mark.parametrize("method", METHODS)
def test_unaligned(cuda, edpp, orc, method):
    n = 40009
    loc = edpp.gen_permutation(n, 2)
    inp = np.arange(n, dtype=np.int32)
    b_loc = cuda.zeros(n + 4, dtype=cuda.int32, device="cuda")
    b_in = cuda.zeros(n + 4, dtype=cuda.int32, device="cuda")
    b_out = cuda.zeros(n + 4, dtype=cuda.int32, device="cuda")
    b_loc[1:n + 1] = to_dev(loc)
    b_in[2:n + 2] = to_dev(inp)
    for passes in (1, 4):
        o = b_out[3:n + 3]
        edpp.gather(to_dev(inp), b_loc[1:n + 1], passes, out=o, method=method)
        np.testing.assert_array_equal(to_host(o), orc.gather(inp, loc, passes))
        edpp.scatter(b_in[2:n + 2], b_loc[1:n + 1], passes, out=o, method=method)
        np.testing.assert_array_equal(to_host(o), orc.scatter(inp, loc, passes))


@pytest.mark.parametrize("method", METHODS)
def test_config2a_full_size_properties(cuda, edpp, method):
    # 2^28 int32, in[i] = i, Fisher-Yates permutation (seed 2): gather gives
    # loc itself, scatter gives the inverse permutation, and gathering the
    # scatter result through loc gives back the identity, for every pass count.
    n = 1 << 28
    loc = to_dev(edpp.gen_permutation(n, 2))
    inp = cuda.arange(n, dtype=cuda.int32, device="cuda")
    ws = None
    if method != "sweep":
        ws = edpp.workspace(max(edpp.gs_workspace_bytes("gather", n, p, method) for p in PASSES))
    for passes in PASSES:
        g = edpp.gather(inp, loc, passes, method=method, ws=ws)
        assert cuda.equal(g, loc), passes
        del g
        s = edpp.scatter(inp, loc, passes, method=method, ws=ws)
        back = edpp.gather(s, loc, passes, method=method, ws=ws)
        assert cuda.equal(back, inp), passes
        del s, back


@pytest.mark.parametrize("n", [16384, 16385, (1 << 21) + 7, 3 * (1 << 20) + 1])
def test_tiled_skewed_indices(cuda, edpp, orc, n):
    # every index in a few windows (one window's pairs exceed a refine tile's
    # span, the per-pair cursor path), plus invalid ones
    rng = np.random.default_rng(n)
    loc = rng.integers(0, min(n, 3000), n).astype(np.int32)
    loc[::7] = rng.integers(0, n, len(loc[::7])).astype(np.int32)
    loc[3::11] = -5
    inp = edpp.gen_uniform_i32(n, 4, -2**31, 2**31 - 1)
    out0 = np.full(n, 99, np.int32)
    g = to_host(edpp.gather(to_dev(inp), to_dev(loc), 1, out=to_dev(out0), method="tiled"))
    np.testing.assert_array_equal(g, orc.gather(inp, loc, 1, out=out0))
    # scatter through a permutation, destinations drawn from two windows first
    perm = edpp.gen_permutation(n, 9)
    order = np.argsort(perm % 5, kind="stable")
    perm = perm[order]
    s = to_host(edpp.scatter(to_dev(inp), to_dev(perm), 4, out=to_dev(out0), method="tiled"))
    np.testing.assert_array_equal(s, orc.scatter(inp, perm, 4, out=out0))


def test_tiled_wide_windows(cuda, edpp):
    # above 2^28 elements the windows grow to 2^15 (128 KB of shared memory)
    n = (1 << 28) + 5
    loc = to_dev(edpp.gen_permutation(n, 2))
    inp = cuda.arange(n, dtype=cuda.int32, device="cuda")
    ws = edpp.workspace(edpp.gs_workspace_bytes("gather", n, 1, "tiled"))
    g = edpp.gather(inp, loc, 1, method="tiled", ws=ws)
    assert cuda.equal(g, loc)
    s = edpp.scatter(inp, loc, 1, method="tiled", ws=ws)
    assert cuda.equal(edpp.gather(s, loc, 1, method="tiled", ws=ws), inp)


def test_against_reference_cuda_kernels(cuda, edpp, orc):
    rc = orc.ref_cuda()
    if rc is None:
        pytest.skip("reference CUDA cubins not available on this machine")
    import ctypes
    n = 300001
    loc = edpp.gen_permutation(n, 2)
    inp = edpp.gen_uniform_i32(n, 4, -2**31, 2**31 - 1)
    P = lambda a: ctypes.c_void_p(a.ctypes.data)
    for scatter in (0, 1):
        ref = np.zeros(n, np.int32)
        assert rc.refcu_gather_scatter(scatter, P(inp), P(ref), P(loc), n) == 0
        f = edpp.scatter if scatter else edpp.gather
        for passes in (1, 8):
            for method in METHODS:
                mine = to_host(f(to_dev(inp), to_dev(loc), passes, method=method))
                np.testing.assert_array_equal(mine, ref)


def test_tiled_above_2p29_takes_the_l2_window_path(cuda, edpp):
    # beyond 2^29 elements the tiled entry points hand over to the L2-window
    # partition (pass 0) inside the same workspace; identity properties
    n = (1 << 29) + 7
    loc = to_dev(edpp.gen_permutation(n, 2))
    inp = cuda.arange(n, dtype=cuda.int32, device="cuda")
    ws = edpp.workspace(edpp.gs_workspace_bytes("gather", n, 1, "tiled"))
    g = edpp.gather(inp, loc, 1, method="tiled", ws=ws)
    assert cuda.equal(g, loc)
    del g
    s = edpp.scatter(inp, loc, 1, method="tiled", ws=ws)
    assert cuda.equal(edpp.gather(s, loc, 1, method="tiled", ws=ws), inp)
