"""Split oracle: the counting-sort restatement against literal restatements
of the reference's own split algorithms, and the reference's own checks.

  orc.split               stable partition (counting sort)
  orc.split_cuda_ballot   cuda/test_split.cu pre_scan/ExclusiveSum/post_scan,
                          ballots emulated lane by lane
  orc.split_single        opencl single_split (single_histogram, scan,
                          single_shuffle), 39 groups as in splitImpl.cpp:371
"""
import numpy as np
import pytest


@pytest.mark.parametrize("bits", [1, 2, 3, 5, 8])
@pytest.mark.parametrize("n", [32, 256, 4096, 32 * 777])
def test_counting_sort_equals_cuda_ballot_split(orc, edpp, bits, n):
    keys = edpp.gen_uniform_i32(n, 3, 0, (1 << bits) - 1)  # CUDA split needs key < B
    ko, _, _ = orc.split(keys, 1 << bits)
    np.testing.assert_array_equal(orc.split_cuda_ballot(keys, bits), ko)
    # the reference's own check, cuda/test_split.cu:196-204
    np.testing.assert_array_equal(ko, np.sort(keys))


@pytest.mark.parametrize("buckets", [1, 2, 16, 256, 1024, 4096, 8192])
@pytest.mark.parametrize("n", [1, 38, 39, 1000, 100003])
def test_counting_sort_equals_single_split(orc, edpp, buckets, n):
    keys = edpp.gen_keys_uniform(n, 3)
    ko, _, start = orc.split(keys, buckets)
    np.testing.assert_array_equal(orc.split_single(keys, buckets, aos=False), ko)
    # AOS: pairs keyed on .x, value = index makes stability visible
    pairs = np.stack([keys, np.arange(n, dtype=np.int32)], axis=1)
    pk, _, _ = orc.split(pairs, buckets, layout="aos")
    np.testing.assert_array_equal(orc.split_single(pairs, buckets, aos=True), pk)
    # the reference's OpenCL checks (opencl/test/test_split.cpp:164-203)
    b = (ko.astype(np.int64) & (buckets - 1))
    assert np.all(np.diff(b) >= 0)
    assert b.sum() == (keys.astype(np.int64) & (buckets - 1)).sum()
    # bucket starts (gatherStartPos)
    counts = np.bincount(keys & (buckets - 1), minlength=buckets)
    np.testing.assert_array_equal(start, np.concatenate([[0], np.cumsum(counts)[:-1]]))


def test_soa_stability(orc, edpp):
    n, B = 50000, 64
    keys = edpp.gen_keys_zipf(n, 3, B)
    vals = np.arange(n, dtype=np.int32)
    ko, vo, _ = orc.split(keys, B, vals)
    b = ko & (B - 1)
    # within a bucket, values (= input positions) ascend: stable
    for bb in range(B):
        v = vo[b == bb]
        assert np.all(np.diff(v) > 0)
    np.testing.assert_array_equal(keys[vo], ko)


@pytest.mark.parametrize("r_len,s_len,hi", [(0, 5, 3), (5, 0, 3), (1, 1, 0), (1000, 700, 50),
                                            (3000, 4000, 100000)])
def test_join_count_equals_pair_count(orc, edpp, r_len, s_len, hi):
    # the join oracle (sort-merge) against the definition: sum over keys of
    # count_R(key) * count_S(key), here by brute-force pair comparison
    r = edpp.gen_uniform_i32(r_len, 11, -hi, hi)
    s = edpp.gen_uniform_i32(s_len, 12, -hi, hi)
    want = int((r[:, None] == s[None, :]).sum()) if r_len and s_len else 0
    assert orc.join_count(r, s) == want
