"""GPU scans against the oracle: bit-exact for int32 / int64 (wrapping), f32
within a stated tolerance of an f64 accumulation."""
import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

ALGOS = ["lookback", "rts", "ssa"]
# Tile sizes of the kernels: 4096 int32/f32, 2048 int64 elements.
SIZES = [1, 2, 3, 4, 5, 31, 32, 33, 1000, 2047, 2048, 2049, 4095, 4096, 4097, 8193,
         65536 * 3 + 17, (1 << 20) + 7]


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("n", SIZES)
@pytest.mark.parametrize("inclusive", [False, True])
def test_int32(cuda, edpp, orc, algo, n, inclusive):
    x = edpp.gen_uniform_i32(n, 1, 0, 15)
    y = to_host(edpp.scan(to_dev(x), inclusive=inclusive, algo=algo))
    np.testing.assert_array_equal(y, orc.scan(x, inclusive))


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("n", [1, 2049, 100003, (1 << 20) + 3])
@pytest.mark.parametrize("inclusive", [False, True])
def test_int64(cuda, edpp, orc, algo, n, inclusive):
    x = edpp.gen_uniform_i64(n, 1, 0, 100)
    x[::7] = np.int64(2**62)  # forces 64-bit wrap-around
    y = to_host(edpp.scan(to_dev(x), inclusive=inclusive, algo=algo))
    np.testing.assert_array_equal(y, orc.scan(x, inclusive))


@pytest.mark.parametrize("algo", ALGOS)
def test_int32_wraps_like_reference(cuda, edpp, orc, algo):
    # values near 2^31: the prefix overflows int32 many times
    n = 300007
    x = edpp.gen_uniform_i32(n, 7, 2**30, 2**31 - 1)
    for inc in (False, True):
        y = to_host(edpp.scan(to_dev(x), inclusive=inc, algo=algo))
        np.testing.assert_array_equal(y, orc.scan(x, inc))


@pytest.mark.parametrize("algo", ALGOS)
def test_all_ones_closed_form(cuda, edpp, algo):
    # cuda/test_scan.cu:52-58: exclusive scan of ones gives out[i] == i
    n = (1 << 22) + 5
    x = cuda.ones(n, dtype=cuda.int32, device="cuda")
    y = edpp.scan(x, algo=algo)
    assert cuda.equal(y, cuda.arange(n, dtype=cuda.int32, device="cuda"))


@pytest.mark.parametrize("algo", ALGOS)
def test_config1_bit_exact(cuda, edpp, orc, algo):
    # 2^24 int32 uniform in [0,15], seed 1, exclusive
    n = 1 << 24
    x = edpp.gen_uniform_i32(n, 1, 0, 15)
    y = to_host(edpp.scan(to_dev(x), algo=algo))
    np.testing.assert_array_equal(y, orc.scan(x))


@pytest.mark.parametrize("algo", ALGOS)
def test_in_place(cuda, edpp, orc, algo):
    n = 123457
    x = edpp.gen_uniform_i32(n, 9, -1000, 1000)
    t = to_dev(x)
    edpp.scan(t, out=t, algo=algo)
    np.testing.assert_array_equal(to_host(t), orc.scan(x))


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("shift_in,shift_out", [(1, 0), (0, 1), (3, 2)])
def test_unaligned_pointers(cuda, edpp, orc, algo, shift_in, shift_out):
    n = 50003
    x = edpp.gen_uniform_i32(n, 11, 0, 1 << 20)
    buf_in = cuda.zeros(n + 8, dtype=cuda.int32, device="cuda")
    buf_out = cuda.zeros(n + 8, dtype=cuda.int32, device="cuda")
    buf_in[shift_in:shift_in + n] = to_dev(x)
    vin, vout = buf_in[shift_in:shift_in + n], buf_out[shift_out:shift_out + n]
    edpp.scan(vin, inclusive=True, algo=algo, out=vout)
    np.testing.assert_array_equal(to_host(vout), orc.scan(x, True))
    assert int(buf_out[:shift_out].abs().sum()) == 0  # nothing written outside


F32_RTOL = 1e-3  # |gpu - f64| / max(|f64|, 1.0)


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("n", [1, 4097, 1 << 20])
def test_f32_within_tolerance(cuda, edpp, orc, algo, n):
    x = edpp.gen_uniform_f32(n, 1, -1.0, 1.0)
    for inc in (False, True):
        y = to_host(edpp.scan(to_dev(x), inclusive=inc, algo=algo)).astype(np.float64)
        ref = orc.scan(x, inc)
        err = np.abs(y - ref) / np.maximum(np.abs(ref), 1.0)
        assert err.max() < F32_RTOL, err.max()


def test_empty(cuda, edpp):
    x = cuda.empty(0, dtype=cuda.int32, device="cuda")
    assert edpp.scan(x).numel() == 0


def test_bounded_wait_times_out_and_context_survives(cuda, edpp, orc):
    # tile 0 never publishes; every waiting tile gives up after 20 ms
    st = edpp.selftest_lookback_timeout(5 * 4096, 20_000_000)
    assert st == edpp.EDPP_ETIMEOUT
    # the context is still usable and the fault word was cleared
    x = edpp.gen_uniform_i32(100000, 1, 0, 15)
    y = to_host(edpp.scan(to_dev(x)))
    np.testing.assert_array_equal(y, orc.scan(x))
    assert edpp.sync_status() == edpp.EDPP_OK


def test_against_reference_cub_exclusive_sum(cuda, edpp, orc):
    # the reference's CUDA scan is cub::DeviceScan::ExclusiveSum
    # (cuda/test_scan.cu:45-47); same call, same seeded input
    rc = orc.ref_cuda()
    if rc is None:
        pytest.skip("reference CUDA runner not built on this machine")
    import ctypes
    for n, lo, hi in ((1 << 24, 0, 15), (1000003, 2**30, 2**31 - 1)):
        x = edpp.gen_uniform_i32(n, 1, lo, hi)
        ref = np.zeros(n, np.int32)
        assert rc.refcu_cub_exclusive_sum_i32(ctypes.c_void_p(x.ctypes.data),
                                              ctypes.c_void_p(ref.ctypes.data), n) == 0
        for algo in ALGOS:
            np.testing.assert_array_equal(to_host(edpp.scan(to_dev(x), algo=algo)), ref)


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("dt,n", [("int32", (1 << 25) + 3), ("int64", (1 << 24) + 5)])
def test_beyond_l2_bit_exact(cuda, edpp, orc, algo, dt, n):
    # larger than 60% of L2: the three-launch RTS/SSA paths and many look-back tiles
    x = (edpp.gen_uniform_i32(n, 4, -5000, 5000) if dt == "int32"
         else edpp.gen_uniform_i64(n, 4, -2**40, 2**40))
    for inclusive in (False, True):
        y = to_host(edpp.scan(to_dev(x), inclusive=inclusive, algo=algo))
        np.testing.assert_array_equal(y, orc.scan(x, inclusive=inclusive))


@pytest.mark.parametrize("algo", ALGOS)
def test_config4_full_size_differences(cuda, edpp, algo):
    # 2^30 int32 in [0,100] (seed 1): consecutive differences of the
    # exclusive scan give back the input, the inclusive scan is the
    # exclusive one shifted by the input, and the total matches a
    # sum in int64 taken modulo 2^32
    torch = cuda
    n = 1 << 30
    x = torch.from_numpy(edpp.gen_uniform_i32(n, 1, 0, 100)).to("cuda")
    ex = edpp.scan(x, inclusive=False, algo=algo)
    assert int(ex[0]) == 0
    assert bool(torch.equal(ex[1:] - ex[:-1], x[:-1]))
    inc = edpp.scan(x, inclusive=True, algo=algo)
    assert bool(torch.equal(inc - ex, x))
    total = int(x.sum(dtype=torch.int64)) & 0xFFFFFFFF
    assert (int(inc[-1]) & 0xFFFFFFFF) == total
