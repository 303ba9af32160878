"""LSD radix sort on the stable split, against numpy's stable argsort of the
keys' unsigned bit patterns (the reference's radix sort order)."""
import numpy as np
import pytest

from conftest import to_dev, to_host

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [1, 2, 1000, 8193, (1 << 20) + 3, 1 << 24])
@pytest.mark.parametrize("bits", [(0, 32), (0, 16), (8, 24), (0, 5), (3, 3)])
def test_pairs(cuda, edpp, n, bits):
    keys = edpp.gen_uniform_i32(n, 3, -2**31, 2**31 - 1)
    vals = np.arange(n, dtype=np.int32)
    ko, vo = edpp.radix_sort(to_dev(keys), to_dev(vals), *bits)
    lo, hi = bits
    digit = (keys.view(np.uint32).astype(np.uint64) >> lo) & ((1 << (hi - lo)) - 1)
    order = np.argsort(digit, kind="stable")
    np.testing.assert_array_equal(to_host(vo), vals[order])
    np.testing.assert_array_equal(to_host(ko), keys[order])


def test_keys_only_and_duplicates(cuda, edpp):
    n = 300001
    keys = edpp.gen_uniform_i32(n, 5, 0, 1000)  # many duplicates
    ko, _ = edpp.radix_sort(to_dev(keys))
    np.testing.assert_array_equal(to_host(ko), np.sort(keys.view(np.uint32)).view(np.int32))
