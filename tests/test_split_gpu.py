"""GPU stable multi-split against the oracle (bit-exact, every layout), and
against the reference's own CUDA split kernels where their cubins were built."""
import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu

BUCKETS = [1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 2048, 4096, 8192]


def _run(edpp, keys, B, layout, vals=None, start=True):
    if layout == "aos":
        ko, _, st = edpp.split(to_dev(keys), B, layout="aos", bucket_start=start)
        return to_host(ko), None, (to_host(st) if start else None)
    ko, vo, st = edpp.split(to_dev(keys), B, values=None if vals is None else to_dev(vals),
                            layout=layout, bucket_start=start)
    return to_host(ko), (None if vo is None else to_host(vo)), (to_host(st) if start else None)


@pytest.mark.parametrize("B", BUCKETS)
@pytest.mark.parametrize("n", [1, 7, 8191, 8192, 8193, 100003])
@pytest.mark.parametrize("layout", ["ko", "soa", "aos"])
def test_uniform_keys(cuda, edpp, orc, B, n, layout):
    keys = edpp.gen_keys_uniform(n, 3)
    vals = np.arange(n, dtype=np.int32)
    if layout == "aos":
        pairs = np.stack([keys, vals], axis=1)
        ko, _, st = _run(edpp, pairs, B, "aos")
        ek, _, es = orc.split(pairs, B, layout="aos")
        np.testing.assert_array_equal(ko, ek)
    else:
        ko, vo, st = _run(edpp, keys, B, layout, vals if layout == "soa" else None)
        ek, ev, es = orc.split(keys, B, vals if layout == "soa" else None, layout=layout)
        np.testing.assert_array_equal(ko, ek)
        if layout == "soa":
            np.testing.assert_array_equal(vo, ev)
    np.testing.assert_array_equal(st, es)


@pytest.mark.parametrize("B", [2, 8, 16, 32, 64, 256, 1024, 2048, 4096, 8192])  # 2048+: two passes
def test_zipf_keys_large(cuda, edpp, orc, B):
    n = (1 << 22) + 77
    keys = edpp.gen_keys_zipf(n, 3, B, 1.0)
    vals = np.arange(n, dtype=np.int32)
    ko, vo, st = _run(edpp, keys, B, "soa", vals)
    ek, ev, es = orc.split(keys, B, vals)
    np.testing.assert_array_equal(ko, ek)
    np.testing.assert_array_equal(vo, ev)
    np.testing.assert_array_equal(st, es)


@pytest.mark.parametrize("B", [4, 8, 16, 256, 1024])
@pytest.mark.parametrize("layout", ["ko", "soa", "aos"])
def test_one_bucket_holds_every_key(cuda, edpp, orc, B, layout):
    # every lane of every warp ranks into the same bucket (the ranking's
    # same-address worst case): the output is the input order and every
    # bucket starts at 0 (all buckets below the last one are empty)
    n = 3 * 8192 + 555
    keys = (edpp.gen_uniform_i32(n, 8, 0, 1 << 20) * B + (B - 1)).astype(np.int32)
    vals = np.arange(n, dtype=np.int32)
    if layout == "aos":
        pairs = np.stack([keys, vals], axis=1)
        ko, _, st = _run(edpp, pairs, B, "aos")
        ek, _, es = orc.split(pairs, B, layout="aos")
        np.testing.assert_array_equal(ko, pairs.reshape(-1) if ko.ndim == 1 else pairs)
    else:
        ko, vo, st = _run(edpp, keys, B, layout, vals if layout == "soa" else None)
        ek, ev, es = orc.split(keys, B, vals if layout == "soa" else None, layout=layout)
        np.testing.assert_array_equal(ko, keys)
        if layout == "soa":
            np.testing.assert_array_equal(vo, vals)
    np.testing.assert_array_equal(ko, ek)
    np.testing.assert_array_equal(st, es)
    assert not st.any()


def test_negative_keys_and_unaligned(cuda, edpp, orc):
    n, B = 50021, 32
    keys = edpp.gen_uniform_i32(n, 5, -2**31, 2**31 - 1)
    vals = edpp.gen_uniform_i32(n, 6, -2**31, 2**31 - 1)
    bk = cuda.zeros(n + 4, dtype=cuda.int32, device="cuda")
    bv = cuda.zeros(n + 4, dtype=cuda.int32, device="cuda")
    bk[1:n + 1] = to_dev(keys)
    bv[3:n + 3] = to_dev(vals)
    ok = cuda.zeros(n + 4, dtype=cuda.int32, device="cuda")
    ov = cuda.zeros(n + 4, dtype=cuda.int32, device="cuda")
    edpp.split(bk[1:n + 1], B, values=bv[3:n + 3], keys_out=ok[2:n + 2], values_out=ov[1:n + 1])
    ek, ev, _ = orc.split(keys, B, vals)
    np.testing.assert_array_equal(to_host(ok[2:n + 2]), ek)
    np.testing.assert_array_equal(to_host(ov[1:n + 1]), ev)


@pytest.mark.parametrize("bits", [1, 3, 5, 8])
def test_against_reference_cuda_split(cuda, edpp, orc, bits):
    rc = orc.ref_cuda()
    if rc is None:
        pytest.skip("reference CUDA cubins not available on this machine")
    import ctypes
    n = 1 << 20  # the reference needs n % 256 == 0 and keys < 2^bits
    keys = edpp.gen_uniform_i32(n, 3, 0, (1 << bits) - 1)
    ref = np.zeros(n, np.int32)
    assert rc.refcu_split(ctypes.c_void_p(keys.ctypes.data), ctypes.c_void_p(ref.ctypes.data), n,
                          bits) == 0
    ko, _, _ = _run(edpp, keys, 1 << bits, "ko", start=False)
    np.testing.assert_array_equal(ko, ref)


def test_config3_full_size_properties(cuda, edpp):
    # 2^28 pairs, value = index: stable <=> within each bucket values ascend;
    # keys are a permutation of the input keys taken in that order.
    n = 1 << 28
    torch = cuda
    for B, kind in ((256, "uniform"), (1024, "zipf")):
        keys = edpp.gen_keys_uniform(n, 3) if kind == "uniform" else edpp.gen_keys_zipf(n, 3, B)
        kd = to_dev(keys)
        del keys
        vd = torch.arange(n, dtype=torch.int32, device="cuda")
        ko, vo, st = edpp.split(kd, B, values=vd, bucket_start=True)
        assert torch.equal(ko, kd[vo.long()])  # values point at their keys
        b = (ko & (B - 1)).long()
        assert bool((b[1:] >= b[:-1]).all())
        same = b[1:] == b[:-1]
        assert bool((vo[1:][same] > vo[:-1][same]).all())  # stable
        counts = torch.bincount((kd & (B - 1)).long(), minlength=B)
        exp_start = torch.cumsum(counts, 0) - counts
        assert torch.equal(st.long(), exp_start)
        del kd, vd, ko, vo, b, same


@pytest.mark.parametrize("layout", ["ko", "soa", "aos"])
@pytest.mark.parametrize("n,local,grid", [(100003, 256, 32768), (100003, 32, 16), (77777, 64, 7),
                                          (5000, 16, 3), (1 << 20, 256, 128)])
@pytest.mark.parametrize("B", [2, 64, 1024])
def test_wi_split_order(cuda, edpp, orc, layout, n, local, grid, B):
    # the reference WI_split's lane-strided order, bit-exact with the
    # literal restatement of WI_histogram / WI_shuffle
    keys = edpp.gen_keys_uniform(n, 3)
    vals = np.arange(n, dtype=np.int32)
    if layout == "aos":
        pairs = np.stack([keys, vals], axis=1)
        ko, _ = edpp.split_wi(to_dev(pairs), B, layout="aos", local_size=local, grid_size=grid)
        ek, _ = orc.split_wi(pairs, B, aos=True, local_size=local, grid_size=grid)
        np.testing.assert_array_equal(to_host(ko), ek)
    else:
        v = vals if layout == "soa" else None
        ko, vo = edpp.split_wi(to_dev(keys), B, None if v is None else to_dev(v), layout=layout,
                               local_size=local, grid_size=grid)
        ek, ev = orc.split_wi(keys, B, v, local_size=local, grid_size=grid)
        np.testing.assert_array_equal(to_host(ko), ek)
        if v is not None:
            np.testing.assert_array_equal(to_host(vo), ev)


@pytest.mark.parametrize("layout", ["ko", "soa", "aos"])
def test_wi_split_matches_reference_kernel_vectors(cuda, edpp, layout):
    """edpp_split_i32_wi against the output of the reference's own OpenCL
    WI_split kernels (tests/golden/reference_cl_wi_split.npz)."""
    from test_golden import wi_cases
    for n, local, grid, B, keys, perm in wi_cases(edpp):
        vals = np.arange(n, dtype=np.int32)
        if layout == "aos":
            ko, _ = edpp.split_wi(to_dev(np.stack([keys, vals], axis=1)), B, layout="aos",
                                  local_size=local, grid_size=grid)
            np.testing.assert_array_equal(to_host(ko), np.stack([keys[perm], perm], axis=1))
        else:
            v = vals if layout == "soa" else None
            ko, vo = edpp.split_wi(to_dev(keys), B, None if v is None else to_dev(v),
                                   layout=layout, local_size=local, grid_size=grid)
            np.testing.assert_array_equal(to_host(ko), keys[perm])
            if v is not None:
                np.testing.assert_array_equal(to_host(vo), perm)
