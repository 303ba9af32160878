"""Every tunable variant gives the oracle's results: each look-back tile shape
and each slice length of the chunked reduce-then-scan (forced through the
tuning table), int32 and int64, exclusive and inclusive, ragged lengths; the
gather under both choices; and the autotuner records a valid choice."""
import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.fixture
def tuned(edpp):
    yield edpp
    edpp.tune_load(None)  # the committed table again


def _ref(x, inclusive):
    c = np.cumsum(x.astype(np.int64)).astype(x.dtype)  # wraps like the device sums
    return c if inclusive else np.concatenate([np.zeros(1, x.dtype), c[:-1]])


@pytest.mark.parametrize("dt", ["int32", "int64"])
@pytest.mark.parametrize("variant", [0, 1, 2, 3])
def test_lookback_shapes(cuda, tuned, dt, variant):
    edpp = tuned
    elem = 4 if dt == "int32" else 8
    for n in (1, 3, 4095, 4097, 8191, 8193, 65537, (1 << 20) + 3, (1 << 23) + 11, (1 << 26) + 5):
        edpp.lib().edpp_tune_clear()
        edpp.tune_set(edpp.TUNE_SCAN_LOOKBACK, elem, n.bit_length() - 1, variant)
        x = (edpp.gen_uniform_i32(n, 5, -2**31, 2**31 - 1) if dt == "int32"
             else edpp.gen_uniform_i64(n, 5, -2**62, 2**62))
        d = to_dev(x)
        for inc in (False, True):
            y = to_host(edpp.scan(d, inclusive=inc, algo="lookback"))
            np.testing.assert_array_equal(y, _ref(x, inc), err_msg=f"n={n} v={variant}")
    assert edpp.sync_status() == edpp.EDPP_OK


@pytest.mark.parametrize("dt", ["int32", "int64"])
@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4])
def test_chunked_rts_slices(cuda, tuned, dt, variant):
    edpp = tuned
    torch = cuda
    elem = 4 if dt == "int32" else 8
    # larger than 60% of L2, so the chunked form runs (variant 4 also below
    # that, where the others take the one-launch fused form); ragged ends
    for n in ((1 << 25) + 5, (3 << 24) + 4097, (1 << 20) + 3, 4097, 1):
        edpp.lib().edpp_tune_clear()
        edpp.tune_set(edpp.TUNE_SCAN_RTS, elem, n.bit_length() - 1, variant)
        tdt = torch.int32 if dt == "int32" else torch.int64
        x = torch.randint(-1000, 1000, (n,), dtype=tdt, device="cuda")
        ref = torch.cumsum(x.to(torch.int64), 0).to(tdt)
        for inc in (False, True):
            y = edpp.scan(x, inclusive=inc, algo="rts")
            r = ref if inc else torch.cat([ref.new_zeros(1), ref[:-1]])
            assert torch.equal(y, r), f"n={n} v={variant} inclusive={inc}"
        del x, ref
    assert edpp.sync_status() == edpp.EDPP_OK


@pytest.mark.parametrize("variant", [0, 1])
def test_gather_choice(cuda, tuned, orc, variant):
    edpp = tuned
    n = (1 << 20) + 7
    edpp.lib().edpp_tune_clear()
    edpp.tune_set(edpp.TUNE_GATHER, 4, n.bit_length() - 1, variant)
    assert edpp.lib().edpp_gather_prefers_direct(n) == variant
    loc = edpp.gen_permutation(n, 2)
    inp = edpp.gen_uniform_i32(n, 4, -2**31, 2**31 - 1)
    y = to_host(edpp.gather(to_dev(inp), to_dev(loc), 1, method="auto"))
    np.testing.assert_array_equal(y, orc.gather(inp, loc, 1))


def test_autotune_records_a_choice(cuda, tuned):
    edpp = tuned
    torch = cuda
    edpp.lib().edpp_tune_clear()
    n = 1 << 22
    x = torch.randint(0, 100, (n,), dtype=torch.int32, device="cuda")
    y = torch.empty_like(x)
    ws = edpp.workspace(edpp.scan_workspace_bytes(n, "int32", "lookback"), x.device)
    v, ms, each = edpp.autotune_plain(edpp.TUNE_SCAN_LOOKBACK, x, y, ws, reps=3)
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 4, n) == (v, True)
    flush = torch.empty(64 << 20, dtype=torch.int32, device="cuda")  # 256 MB > L2
    v, ms, each = edpp.autotune_plain(edpp.TUNE_SCAN_LOOKBACK, x, y, ws, reps=3, flush=flush)
    assert 0 <= v < 4 and ms > 0 and len(each) == 4 and each[v] == ms
    assert v == 0 or ms <= 0.99 * each[0]  # the default stays unless beaten by over 1%
    assert edpp.tune_get(edpp.TUNE_SCAN_LOOKBACK, 4, n) == (v, True)
    loc = torch.from_numpy(edpp.gen_permutation(n, 2)).cuda()
    gws = edpp.workspace(edpp.gs_workspace_bytes("gather", n, 1, "tiled"), x.device)
    v, ms, _ = edpp.autotune_plain(edpp.TUNE_GATHER, x, y, gws, loc=loc, reps=3)
    assert v in (0, 1) and ms > 0
    assert torch.equal(y, x[loc.long()])  # the last candidate's result


@pytest.mark.parametrize("variant", [0, 1, 2, 3, 4])
def test_chunked_rts_unaligned_and_in_place(cuda, tuned, variant):
    """The chunked reduce-then-scan with pointers off 16-byte alignment (its
    plain-load path) and in place (in == out), int32, at a size that takes
    the chunked form."""
    edpp = tuned
    torch = cuda
    n = (1 << 25) + 3
    edpp.lib().edpp_tune_clear()
    edpp.tune_set(edpp.TUNE_SCAN_RTS, 4, n.bit_length() - 1, variant)
    base = torch.randint(-1000, 1000, (n + 2,), dtype=torch.int32, device="cuda")
    x = base[1:n + 1]  # 4 bytes past a 16-byte boundary
    ref = torch.cumsum(x.to(torch.int64), 0).to(torch.int32)
    out_base = torch.empty(n + 3, dtype=torch.int32, device="cuda")
    y = out_base[3:n + 3]
    assert y.data_ptr() % 16 != 0 and x.data_ptr() % 16 != 0
    edpp.scan(x, inclusive=True, algo="rts", out=y)
    assert torch.equal(y, ref)
    z = x.clone()
    edpp.scan(z, inclusive=True, algo="rts", out=z)  # in place, aligned
    assert torch.equal(z, ref)
    w = base.clone()[1:n + 1]
    edpp.scan(w, inclusive=True, algo="rts", out=w)  # in place, unaligned
    assert torch.equal(w, ref)
    assert edpp.sync_status() == edpp.EDPP_OK
