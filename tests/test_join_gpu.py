"""Partitioned hash join match count against the oracle (sort-merge count)."""
import numpy as np
import pytest

from conftest import to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("r_len,s_len,key_range", [(1, 1, 10), (1000, 3000, 500),
                                                   (1 << 20, 1 << 20, 1 << 20),
                                                   ((1 << 22) + 7, (1 << 21) + 3, 1 << 23)])
@pytest.mark.parametrize("buckets", [0, 1, 64, 4096, 8192, "np"])
def test_uniform_keys(cuda, edpp, orc, r_len, s_len, key_range, buckets):
    r = edpp.gen_uniform_i32(r_len, 7, 0, key_range - 1)
    s = edpp.gen_uniform_i32(s_len, 8, 0, key_range - 1)
    if buckets == "np":
        got = edpp.hash_join_count(to_dev(r), to_dev(s), partitioned=False)
    else:
        got = edpp.hash_join_count(to_dev(r), to_dev(s), buckets)
    assert got == orc.join_count(r, s)


def test_skewed_and_negative_keys(cuda, edpp, orc):
    # one hot key (partition far larger than a table build) and negative keys
    n = 200000
    r = edpp.gen_uniform_i32(n, 9, -1000, 1000)
    s = edpp.gen_uniform_i32(n, 10, -1000, 1000)
    s[: n // 2] = 42
    r[::3] = 42
    want = orc.join_count(r, s)
    assert edpp.hash_join_count(to_dev(r), to_dev(s), 256) == want
    assert edpp.hash_join_count(to_dev(r), to_dev(s), partitioned=False) == want
    assert edpp.hash_join_count(to_dev(r), to_dev(s[:0].copy())) == 0
    assert edpp.hash_join_count(to_dev(r[:0].copy()), to_dev(s), partitioned=False) == 0
