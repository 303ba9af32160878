"""Access-pattern and single-block scan microbenchmark kernels: each one's
output against the oracle (the scale kernels touch exactly the reference's
index set, the block-order sweep sums every chunk once, the matrix scans are
exclusive scans as opencl/test/test_scan_local.cpp checks them)."""
import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("pattern", ["column", "row", "mixed", "vec"])
@pytest.mark.parametrize("local,grid,repeat", [(512, 64, 1), (512, 96, 7), (64, 3, 20),
                                               (96, 5, 3)])
def test_scale_patterns(cuda, edpp, pattern, local, grid, repeat):
    n = local * grid * repeat
    inp = edpp.gen_uniform_i32(n + 37, 5, -2**28, 2**28)
    d_in = to_dev(inp)
    d_out = cuda.full((n + 37,), -7, dtype=cuda.int32, device="cuda")
    edpp.access_scale(d_in, d_out, repeat, pattern, local, grid)
    got = to_host(d_out)
    np.testing.assert_array_equal(got[:n], inp[:n] * 3)
    assert np.all(got[n:] == -7)  # nothing past the index range is written


@pytest.mark.parametrize("local", [1, 32, 256])
@pytest.mark.parametrize("shuffled", [False, True])
def test_block_order_sweep(cuda, edpp, local, shuffled):
    grid, chunk = 256, 1000
    inp = edpp.gen_uniform_i32(grid * chunk + 5, 6, 0, 1000)
    order = np.arange(grid, dtype=np.int32)
    if shuffled:
        order = np.random.default_rng(1).permutation(grid).astype(np.int32)
    out = to_host(edpp.access_wg(to_dev(inp), to_dev(order), local))
    want = (inp[:grid * chunk] & 1).reshape(grid, chunk).sum(axis=1)
    np.testing.assert_array_equal(out, want)


@pytest.mark.parametrize("length", [1, 1000, 512 * 64 * 3 + 17])
def test_cache_heat(cuda, edpp, length):
    d = cuda.full((length,), -1, dtype=cuda.int32, device="cuda")
    edpp.cache_heat(d, 512, 64)
    np.testing.assert_array_equal(to_host(d), np.arange(length, dtype=np.int32))


@pytest.mark.parametrize("scheme", ["lm", "reg", "lm_reg", "warp"])
@pytest.mark.parametrize("tile", [1, 2, 7, 16, 33, 49])
def test_local_scan(cuda, edpp, orc, scheme, tile):
    n = 512 * tile
    inp = edpp.gen_uniform_i32(n, 7, 0, 15)  # the reference's rand() & 0xf range
    out = to_host(edpp.local_scan(to_dev(inp), tile, scheme, repeat=3))
    np.testing.assert_array_equal(out, orc.scan(inp, inclusive=False))
