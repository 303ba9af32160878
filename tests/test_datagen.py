"""Seeded generators (csrc/host/datagen.cpp): reproducible, thread-count
independent, and with the distributions the benchmark configs name."""
import hashlib

import numpy as np


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:16]


def test_splitmix64_known_values(edpp):
    # splitmix64 with state 0: published first outputs of the generator.
    lib = edpp.lib()
    assert lib.edpp_gen_draw(0, 0) == 0xE220A8397B1DCDAF
    assert lib.edpp_gen_draw(0, 1) == 0x6E789E6AA1B965F4
    assert lib.edpp_gen_draw(0, 2) == 0x06C45D188009454F


def test_deterministic_and_parallel_independent(edpp):
    a = edpp.gen_uniform_i32(1 << 18, 1, 0, 15)  # threaded fill
    b = np.array([edpp.gen_uniform_i32(1, 0, 0, 0)[0]])  # smoke
    assert b.shape == (1,)
    c = edpp.gen_uniform_i32(1 << 18, 1, 0, 15)
    np.testing.assert_array_equal(a, c)
    # a short fill (single thread) is a prefix of the long one
    np.testing.assert_array_equal(edpp.gen_uniform_i32(1000, 1, 0, 15), a[:1000])
    assert a.min() == 0 and a.max() == 15
    assert abs(a.mean() - 7.5) < 0.05


def test_permutation_is_fisher_yates_permutation(edpp):
    n = 100000
    p = edpp.gen_permutation(n, 2)
    assert np.array_equal(np.sort(p), np.arange(n, dtype=np.int32))
    np.testing.assert_array_equal(p, edpp.gen_permutation(n, 2))
    assert not np.array_equal(p, edpp.gen_permutation(n, 3))
    # Durstenfeld with the documented draw order, restated in Python for small n
    lib = edpp.lib()
    m = 257
    ref = list(range(m))
    for i in range(m - 1, 0, -1):
        x = lib.edpp_gen_draw(2, m - 1 - i)
        j = ((x >> 32) * (i + 1)) >> 32
        ref[i], ref[j] = ref[j], ref[i]
    np.testing.assert_array_equal(edpp.gen_permutation(m, 2), np.array(ref, np.int32))


def test_zipf_keys(edpp):
    B, n = 64, 1 << 20
    k = edpp.gen_keys_zipf(n, 3, B, 1.0)
    assert k.min() >= 0
    b = k & (B - 1)
    cnt = np.bincount(b, minlength=B) / n
    h = sum(1.0 / (i + 1) for i in range(B))
    expect = np.array([1.0 / (i + 1) / h for i in range(B)])
    assert np.max(np.abs(cnt - expect)) < 0.003
    # high bits are random: many distinct keys per bucket
    assert len(np.unique(k[b == 0])) > 0.9 * (b == 0).sum()


def test_uniform_keys_and_floats(edpp):
    k = edpp.gen_keys_uniform(1 << 16, 3)
    assert k.min() >= 0 and k.max() > 2**30
    f = edpp.gen_uniform_f32(1 << 16, 1, -1.0, 1.0)
    assert f.min() >= -1.0 and f.max() < 1.0 and abs(f.mean()) < 0.02
    g = edpp.gen_uniform_i64(1000, 1, 0, 100)
    assert g.min() >= 0 and g.max() <= 100


def test_oracle_permutation_equals_library_generator(edpp, orc):
    """The reference arm of the benchmark makes its index array with the
    oracle's generator (it must not load the library); it is the same array."""
    for n, seed in ((0, 2), (1, 2), (2, 2), (1000, 2), (1 << 20, 2), ((1 << 20) + 7, 5)):
        np.testing.assert_array_equal(orc.gen_permutation(n, seed), edpp.gen_permutation(n, seed))
