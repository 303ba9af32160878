"""The oracle's restatement against the reference's own OpenMP code.

oracle/_ref/libref_omp.so is the reference's openmp/*.cpp compiled from the
reference tree (oracle/build.py); it exists only where that tree is present
and the host is x86 (the reference uses AVX2).  Elsewhere these tests skip
and the committed golden vectors (test_oracle_golden.py) pin the oracle.
"""
import ctypes

import numpy as np
import pytest


@pytest.fixture(scope="module")
def ref(orc):
    r = orc.ref_omp()
    if r is None:
        pytest.skip("reference OpenMP library not built on this host")
    return r


def P(a):
    return ctypes.c_void_p(a.ctypes.data)


@pytest.mark.parametrize("n", [1, 2, 31, 1000, 65537])
def test_gather_scatter_match_reference(orc, edpp, ref, n):
    loc = edpp.gen_permutation(n, 2)
    inp = np.arange(n, dtype=np.int32)
    out_ref = np.zeros(n, np.int32)
    ref.ref_gather(P(inp), P(out_ref), P(loc), n)
    for passes in (1, 2, 4, 8, 16):
        np.testing.assert_array_equal(orc.gather(inp, loc, passes), out_ref)
    out_ref = np.zeros(n, np.int32)
    ref.ref_scatter(P(inp), P(out_ref), P(loc), n)
    for passes in (1, 2, 4, 8, 16):
        np.testing.assert_array_equal(orc.scatter(inp, loc, passes), out_ref)


@pytest.mark.parametrize("n,lo,hi", [(1, 0, 15), (4099, 0, 15), (100003, 0, 100),
                                     (20000, 2**30, 2**31 - 1), (3000, -2**31, 2**31 - 1)])
def test_scans_match_reference(orc, edpp, ref, n, lo, hi):
    x = edpp.gen_uniform_i32(n, 1, lo, hi)
    ex = orc.scan(x)
    for name in ("ref_scan_ssa", "ref_scan_rts", "ref_scan_tbb"):
        out = np.zeros(n, np.int32)
        getattr(ref, name)(P(x), P(out), n)
        np.testing.assert_array_equal(out, ex, err_msg=name)
    for scheme in ("ssa", "rts"):
        for nt in (1, 3, 8):
            out, _ = orc.scan_omp(x, scheme, nt)
            np.testing.assert_array_equal(out, ex, err_msg=f"{scheme}/{nt}")
    np.testing.assert_array_equal(orc.scan(x, inclusive=True), ex + x)


def test_all_ones_scan_closed_form(orc, ref):
    # cuda/test_scan.cu:52-58 and openmp/test_scan_CPU.cpp:39-49: out[i] == i
    n = 1 << 16
    x = np.ones(n, np.int32)
    np.testing.assert_array_equal(orc.scan(x), np.arange(n, dtype=np.int32))
    out = np.zeros(n, np.int32)
    ref.ref_scan_rts(P(x), P(out), n)
    np.testing.assert_array_equal(out, np.arange(n, dtype=np.int32))


def test_stream_copy_scale_match_reference(orc, ref, edpp):
    n = 12345
    a = edpp.gen_uniform_i32(n, 5, -2**31, 2**31 - 1)
    for name, op in (("ref_copy", "copy"), ("ref_scale", "scale")):
        out = np.zeros(n, np.int32)
        getattr(ref, name)(P(a), P(out), n)
        mine, _ = orc.stream(op, a, scalar=3)
        np.testing.assert_array_equal(mine, out, err_msg=op)


@pytest.mark.parametrize("xs", [[1.0, 2.0, 3.0, 100.0, 2.5], [5.0, 5.0, 5.0, 5.0, 9.0],
                                [1.0, 1.1, 1.2, 1.3], [7.0]])
def test_hampel_matches_reference(orc, ref, xs):
    a = np.array(xs, np.float64)
    assert orc.average_hampel(a) == pytest.approx(ref.ref_average_hampel(P(a), len(a)), rel=1e-12)


def test_compute_bandwidth_matches_reference(orc, ref):
    for num, w, ms in ((1 << 28, 4, 3.5), (12345, 8, 0.25)):
        assert orc.compute_bandwidth(num, w, ms) == pytest.approx(
            ref.ref_compute_bandwidth(num, w, ms), rel=1e-15)


@pytest.mark.parametrize("n,local,grid,B", [(1, 32, 2, 4), (100003, 32, 16, 64), (77777, 64, 7, 2),
                                            (5000, 16, 3, 1024), (65536, 128, 64, 256),
                                            (999, 1, 39, 16)])
def test_wi_split_restatement_matches_reference_kernels(orc, edpp, n, local, grid, B):
    """The reference's own OpenCL WI_split, compiled as C (oracle/_ref), on
    the same seeded keys as the restatement, every layout."""
    if orc.ref_cl_split("ko") is None:
        pytest.skip("reference OpenCL split not built on this host")
    keys = edpp.gen_keys_uniform(n, 11)
    vals = np.arange(n, dtype=np.int32)
    rk, _ = orc.ref_wi_split(keys, B, local_size=local, grid_size=grid)
    ek, _ = orc.split_wi(keys, B, local_size=local, grid_size=grid)
    np.testing.assert_array_equal(rk, ek)
    rk, rv = orc.ref_wi_split(keys, B, vals, local_size=local, grid_size=grid)
    ek, ev = orc.split_wi(keys, B, vals, local_size=local, grid_size=grid)
    np.testing.assert_array_equal(rk, ek)
    np.testing.assert_array_equal(rv, ev)
    pairs = np.stack([keys, vals], axis=1)
    ra, _ = orc.ref_wi_split(pairs, B, aos=True, local_size=local, grid_size=grid)
    ea, _ = orc.split_wi(pairs, B, aos=True, local_size=local, grid_size=grid)
    np.testing.assert_array_equal(ra, ea)
