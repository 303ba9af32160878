"""Golden vectors produced by the reference itself (tests/golden/make_golden.py).

reference_omp.npz   the reference's OpenMP functions (gather, scatter,
                    scan_SSA_omp, scan_RTS_omp, scan_tbb, copy_omp,
                    scale_omp, average_Hampel)
reference_cuda.npz  the reference's CUDA kernels (warp-ballot split,
                    gather_kernel, scatter_kernel, int32 STREAM) and the CUB
                    ExclusiveSum call of its scan test
reference_cl_wi_split.npz  the reference's OpenCL WI_split (WI_histogram /
                    WI_shuffle compiled as C), as the permutation it applies

The oracle must reproduce every vector (CPU tests); the GPU primitives must
too (gpu tests).
"""
from pathlib import Path

import numpy as np
import pytest

from conftest import to_dev, to_host

G = Path(__file__).resolve().parent / "golden"


def load(name):
    p = G / name
    if not p.exists():
        pytest.skip(f"{name} not generated")
    return dict(np.load(p))


def wi_cases(edpp):
    """(n, local, grid, buckets, keys, perm) of every WI_split fixture; the
    keys are regenerated from their seed and checked against the stored sum."""
    g = load("reference_cl_wi_split.npz")
    out = []
    for c in range(len([k for k in g if k.endswith("_params")])):
        n, local, grid, B, seed, ksum = (int(v) for v in g[f"wi{c}_params"])
        keys = edpp.gen_keys_uniform(n, seed)
        assert int(keys.astype(np.int64).sum()) == ksum
        out.append((n, local, grid, B, keys, g[f"wi{c}_perm"]))
    return out


def test_oracle_wi_split_vectors(orc, edpp):
    """The restated WI_split order equals the reference's own kernels' output
    in every layout."""
    for n, local, grid, B, keys, perm in wi_cases(edpp):
        vals = np.arange(n, dtype=np.int32)
        ko, _ = orc.split_wi(keys, B, local_size=local, grid_size=grid)
        np.testing.assert_array_equal(ko, keys[perm])
        sk, sv = orc.split_wi(keys, B, vals, local_size=local, grid_size=grid)
        np.testing.assert_array_equal(sk, keys[perm])
        np.testing.assert_array_equal(sv, perm)
        ak, _ = orc.split_wi(np.stack([keys, vals], axis=1), B, aos=True, local_size=local,
                             grid_size=grid)
        np.testing.assert_array_equal(ak, np.stack([keys[perm], perm], axis=1))


# ---- oracle against the reference's vectors ----------------------------------
def test_oracle_omp_vectors(orc, edpp):
    g = load("reference_omp.npz")
    # the inputs are the package's seeded generators: pin them too
    np.testing.assert_array_equal(g["gs_loc"], edpp.gen_permutation(len(g["gs_loc"]), 2))
    for p in (1, 2, 4, 8, 16):
        np.testing.assert_array_equal(orc.gather(g["gs_in"], g["gs_loc"], p), g["gather_out"])
        np.testing.assert_array_equal(orc.scatter(g["gs_in"], g["gs_loc"], p), g["scatter_out"])
    for tag in ("small", "wrap", "signed"):
        x = g[f"scan_{tag}_in"]
        for name in ("ssa", "rts", "tbb"):
            np.testing.assert_array_equal(orc.scan(x), g[f"scan_{tag}_{name}"])
        for scheme in ("ssa", "rts"):
            np.testing.assert_array_equal(orc.scan_omp(x, scheme, 4)[0], g[f"scan_{tag}_{scheme}"])
    np.testing.assert_array_equal(orc.stream("copy", g["stream_a"])[0], g["stream_copy"])
    np.testing.assert_array_equal(orc.stream("scale", g["stream_a"], scalar=3)[0],
                                  g["stream_scale"])
    for i in range(4):
        assert orc.average_hampel(g[f"hampel_{i}_in"]) == pytest.approx(
            float(g[f"hampel_{i}_out"][0]), rel=1e-12)


def test_oracle_cuda_vectors(orc):
    g = load("reference_cuda.npz")
    for bits in (1, 3, 5, 8):
        k = g[f"split_b{bits}_in"]
        ko, _, _ = orc.split(k, 1 << bits)
        np.testing.assert_array_equal(ko, g[f"split_b{bits}_out"])
        np.testing.assert_array_equal(orc.split_cuda_ballot(k, bits), g[f"split_b{bits}_out"])
    np.testing.assert_array_equal(orc.gather(g["gs_in"], g["gs_loc"]), g["gather_out"])
    np.testing.assert_array_equal(orc.scatter(g["gs_in"], g["gs_loc"]), g["scatter_out"])
    for name in ("copy", "scale", "add", "triad"):
        np.testing.assert_array_equal(orc.stream(name, g["stream_a"], g["stream_b"], 3)[0],
                                      g[f"stream_{name}"])
    np.testing.assert_array_equal(orc.scan(g["cub_scan_in"]), g["cub_scan_out"])


# ---- GPU primitives against the reference's vectors -----------------------------
@pytest.mark.gpu
def test_gpu_omp_vectors(cuda, edpp):
    g = load("reference_omp.npz")
    for p in (1, 2, 4, 8, 16):
        np.testing.assert_array_equal(
            to_host(edpp.gather(to_dev(g["gs_in"]), to_dev(g["gs_loc"]), p)), g["gather_out"])
        np.testing.assert_array_equal(
            to_host(edpp.scatter(to_dev(g["gs_in"]), to_dev(g["gs_loc"]), p)), g["scatter_out"])
    for tag in ("small", "wrap", "signed"):
        x = to_dev(g[f"scan_{tag}_in"])
        for algo in ("lookback", "rts", "ssa"):
            np.testing.assert_array_equal(to_host(edpp.scan(x, algo=algo)), g[f"scan_{tag}_ssa"])
    a = to_dev(g["stream_a"])
    np.testing.assert_array_equal(to_host(edpp.stream("copy", a)), g["stream_copy"])
    np.testing.assert_array_equal(to_host(edpp.stream("scale", a, scalar=3)), g["stream_scale"])


@pytest.mark.gpu
def test_gpu_cuda_vectors(cuda, edpp):
    g = load("reference_cuda.npz")
    for bits in (1, 3, 5, 8):
        ko, _, _ = edpp.split(to_dev(g[f"split_b{bits}_in"]), 1 << bits)
        np.testing.assert_array_equal(to_host(ko), g[f"split_b{bits}_out"])
    np.testing.assert_array_equal(to_host(edpp.gather(to_dev(g["gs_in"]), to_dev(g["gs_loc"]), 4)),
                                  g["gather_out"])
    np.testing.assert_array_equal(
        to_host(edpp.scatter(to_dev(g["gs_in"]), to_dev(g["gs_loc"]), 4)), g["scatter_out"])
    for name in ("copy", "scale", "add", "triad"):
        np.testing.assert_array_equal(
            to_host(edpp.stream(name, to_dev(g["stream_a"]), to_dev(g["stream_b"]), 3)),
            g[f"stream_{name}"])
    np.testing.assert_array_equal(to_host(edpp.scan(to_dev(g["cub_scan_in"]))), g["cub_scan_out"])
