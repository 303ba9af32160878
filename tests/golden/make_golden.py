"""Generate the golden vectors under tests/golden/ from the reference itself.

reference_omp.npz: outputs of the reference's own OpenMP functions
(openmp/test_gather_scatter_CPU.cpp gather/scatter, openmp/test_scan_CPU.cpp
scan_SSA_omp / scan_RTS_omp / scan_tbb, openmp/test_bandwidth_CPU.cpp
copy_omp / scale_omp, openmp/util/utility.cpp average_Hampel), compiled from
the reference tree into oracle/_ref/libref_omp.so by oracle/build.py, on
seeded inputs from the package's generators.  Run here, where the reference
tree exists:   python tests/golden/make_golden.py

reference_cl_wi_split.npz (written by --cl, where the reference tree exists):
outputs of the reference's own WI_split (WI_histogram, exclusive scan,
WI_shuffle of opencl/kernels/split_kernel.cl, compiled as C by
oracle/build.py through oracle/ref_cl_shim.h) for KO, KVS_SOA and KVS_AOS on
several work-group shapes.

reference_cuda.npz (written by --cuda, on a GPU machine): outputs of the
reference's CUDA split (pre_scan / ExclusiveSum / post_scan), gather_kernel,
scatter_kernel and int32 STREAM kernels, launched from the reference's
cubins by oracle/ref_cuda_runner.cu.
"""
import ctypes
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT), str(ROOT / "efficient-dpp_gb300")]

import edpp  # noqa: E402
from oracle import oracle as orc  # noqa: E402


def P(a):
    return ctypes.c_void_p(a.ctypes.data)


def make_omp(out_path: Path):
    orc.build()
    ref = orc.ref_omp()
    if ref is None:
        raise SystemExit("reference OpenMP library not available (needs the reference tree, x86)")
    g = {}
    n = 1031
    loc = edpp.gen_permutation(n, 2)
    inp = edpp.gen_uniform_i32(n, 4, -2**31, 2**31 - 1)
    out = np.zeros(n, np.int32)
    ref.ref_gather(P(inp), P(out), P(loc), n)
    g["gs_loc"], g["gs_in"], g["gather_out"] = loc, inp, out.copy()
    out = np.zeros(n, np.int32)
    ref.ref_scatter(P(inp), P(out), P(loc), n)
    g["scatter_out"] = out.copy()
    for tag, (m, seed, lo, hi) in {"small": (4099, 1, 0, 15), "wrap": (2053, 7, 2**30, 2**31 - 1),
                                   "signed": (1500, 9, -2**31, 2**31 - 1)}.items():
        x = edpp.gen_uniform_i32(m, seed, lo, hi)
        g[f"scan_{tag}_in"] = x
        for name in ("ssa", "rts", "tbb"):
            o = np.zeros(m, np.int32)
            getattr(ref, f"ref_scan_{name}")(P(x), P(o), m)
            g[f"scan_{tag}_{name}"] = o
    a = edpp.gen_uniform_i32(1027, 5, -2**31, 2**31 - 1)
    g["stream_a"] = a
    for name in ("copy", "scale"):
        o = np.zeros(len(a), np.int32)
        getattr(ref, f"ref_{name}")(P(a), P(o), len(a))
        g[f"stream_{name}"] = o
    hs = [np.array(v, np.float64) for v in ([1, 2, 3, 100, 2.5], [5, 5, 5, 5, 9],
                                            [1.0, 1.1, 1.2, 1.3], [3.2, 3.3, 3.1, 3.25, 3.3])]
    for i, h in enumerate(hs):
        g[f"hampel_{i}_in"] = h
        g[f"hampel_{i}_out"] = np.array([ref.ref_average_hampel(P(h), len(h))])
    np.savez_compressed(out_path, **g)
    print(f"wrote {out_path} ({out_path.stat().st_size} bytes, {len(g)} arrays)")


def make_cuda(out_path: Path):
    orc.build()
    rc = orc.ref_cuda()
    if rc is None:
        raise SystemExit("reference CUDA runner not available (needs a GPU and the cubins)")
    g = {}
    for bits in (1, 3, 5, 8):
        n = 4096 + 256 * bits
        k = edpp.gen_uniform_i32(n, 3, 0, (1 << bits) - 1)
        o = np.zeros(n, np.int32)
        assert rc.refcu_split(P(k), P(o), n, bits) == 0
        g[f"split_b{bits}_in"], g[f"split_b{bits}_out"] = k, o
    n = 3001
    loc = edpp.gen_permutation(n, 2)
    inp = edpp.gen_uniform_i32(n, 4, -2**31, 2**31 - 1)
    g["gs_loc"], g["gs_in"] = loc, inp
    for sc, name in ((0, "gather"), (1, "scatter")):
        o = np.zeros(n, np.int32)
        assert rc.refcu_gather_scatter(sc, P(inp), P(o), P(loc), n) == 0
        g[f"{name}_out"] = o
    a = edpp.gen_uniform_i32(2051, 1, -2**31, 2**31 - 1)
    b = edpp.gen_uniform_i32(2051, 2, -2**31, 2**31 - 1)
    g["stream_a"], g["stream_b"] = a, b
    for op, name in enumerate(("copy", "scale", "add", "triad")):
        o = np.zeros(len(a), np.int32)
        assert rc.refcu_stream_i32(op, P(a), P(b), P(o), len(a)) == 0
        g[f"stream_{name}"] = o
    x = edpp.gen_uniform_i32(70001, 1, 0, 15)
    o = np.zeros(len(x), np.int32)
    assert rc.refcu_cub_exclusive_sum_i32(P(x), P(o), len(x)) == 0
    g["cub_scan_in"], g["cub_scan_out"] = x, o
    np.savez_compressed(out_path, **g)
    print(f"wrote {out_path} ({out_path.stat().st_size} bytes, {len(g)} arrays)")


# (n, local_size, grid_size, buckets) of the WI_split fixtures: work-group
# shapes from one work-item per group to 256, grids from 3 to 128 groups,
# inputs shorter than the work-item count, 2 to 1024 buckets
WI_CASES = [(8191, 32, 16, 64), (6007, 64, 7, 2), (5000, 16, 3, 1024), (8191, 256, 8, 256),
            (4099, 256, 128, 16), (3001, 1, 39, 8)]


def make_cl(out_path: Path):
    orc.build()
    g = {}
    for c, (n, local, grid, B) in enumerate(WI_CASES):
        keys = edpp.gen_keys_uniform(n, 30 + c)
        vals = np.arange(n, dtype=np.int32)
        ko = orc.ref_wi_split(keys, B, local_size=local, grid_size=grid)
        so = orc.ref_wi_split(keys, B, vals, local_size=local, grid_size=grid)
        ao = orc.ref_wi_split(np.stack([keys, vals], axis=1), B, aos=True, local_size=local,
                              grid_size=grid)
        if ko is None or so is None or ao is None:
            raise SystemExit("reference OpenCL split not built (needs the reference tree)")
        # The order does not depend on the layout: the SOA values (input
        # index) are the permutation, and every layout's output is the keys
        # (and indices) in that order.  Only the permutation is stored; the
        # keys are regenerated from their seed (generator checked by sum).
        perm = so[1]
        assert np.array_equal(ko[0], keys[perm]) and np.array_equal(so[0], keys[perm])
        assert np.array_equal(ao[0], np.stack([keys[perm], perm], axis=1))
        g[f"wi{c}_params"] = np.array([n, local, grid, B, 30 + c,
                                       int(keys.astype(np.int64).sum())], np.int64)
        g[f"wi{c}_perm"] = perm
    np.savez_compressed(out_path, **g)
    print(f"wrote {out_path} ({out_path.stat().st_size} bytes, {len(g)} arrays)")


if __name__ == "__main__":
    if "--cl" in sys.argv:
        make_cl(HERE / "reference_cl_wi_split.npz")
    elif "--cuda" in sys.argv:
        dst = Path(sys.argv[sys.argv.index("--cuda") + 1]) if len(sys.argv) > 2 else \
            HERE / "reference_cuda.npz"
        make_cuda(dst)
    else:
        make_omp(HERE / "reference_omp.npz")
