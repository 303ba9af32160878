"""The reference's own CUDA kernels (cuda/test_{gather,scatter,split,bandwidth}.cu,
compiled unchanged) and the CUB scan it calls (cuda/test_scan.cu:45-47),
timed on this GPU beside this library's calls on the same data.  Correctness
of both sides is checked elsewhere; here only the reference calls' status is
asserted.  With EDPP_TIMING_JSON set, the table is written there as JSON."""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import to_dev

pytestmark = pytest.mark.gpu


def _ours_ms(cuda, fn, reps=10):
    fn()
    cuda.cuda.synchronize()
    a = cuda.cuda.Event(enable_timing=True)
    b = cuda.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    cuda.cuda.synchronize()
    return a.elapsed_time(b) / reps


def test_reference_kernels_timed_beside_ours(cuda, edpp, orc):
    rc = orc.ref_cuda()
    if rc is None:
        pytest.skip("reference CUDA runner not built on this machine")
    ms = ctypes.c_float(0.0)
    rows = []

    # gather / scatter: 2^26 int32, Fisher-Yates permutation
    n = 1 << 26
    loc = edpp.gen_permutation(n, 2)
    d_loc = to_dev(loc)
    d_in = cuda.arange(n, dtype=cuda.int32, device="cuda")
    out = cuda.empty_like(d_in)
    ws = edpp.workspace(edpp.gs_workspace_bytes("gather", n, 1, "tiled"))
    for kind, scatter in (("gather", 0), ("scatter", 1)):
        assert rc.refcu_time_gather_scatter(scatter, ctypes.c_void_p(loc.ctypes.data), n, 10,
                                            ctypes.byref(ms)) == 0
        f = edpp.gather if kind == "gather" else edpp.scatter
        # "auto": the direct sweep for a gather whose source fits ~2.5x L2, else tiled
        ours = _ours_ms(cuda, lambda: f(d_in, d_loc, 1, out=out, method="auto", ws=ws))
        tiled = _ours_ms(cuda, lambda: f(d_in, d_loc, 1, out=out, method="tiled", ws=ws))
        rows.append({"call": f"{kind} 2^26", "reference_ms": round(ms.value, 4),
                     "ours_ms": round(ours, 4), "ours_tiled_ms": round(tiled, 4)})
    del d_loc, d_in, out, ws

    # exclusive int32 scan: CUB DeviceScan vs look-back and vs the chunked
    # reduce-then-scan (second read from L2), 2^28
    n = 1 << 28
    x = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    y = cuda.empty_like(x)
    assert rc.refcu_time_cub_scan(n, 10, ctypes.byref(ms)) == 0
    for algo in ("lookback", "rts"):
        sws = edpp.workspace(edpp.scan_workspace_bytes(n, "int32", algo))
        ours = _ours_ms(cuda, lambda: edpp.scan(x, algo=algo, out=y, ws=sws))
        rows.append({"call": f"exclusive scan int32 2^28 (CUB) vs {algo}",
                     "reference_ms": round(ms.value, 4), "ours_ms": round(ours, 4)})
        del sws
    del x, y

    # stable key-only split, 256 buckets, 2^24 keys < 256 (the reference's limits)
    n = 1 << 24
    keys = edpp.gen_uniform_i32(n, 3, 0, 255)
    assert rc.refcu_time_split(ctypes.c_void_p(keys.ctypes.data), n, 8, 10, ctypes.byref(ms)) == 0
    d_keys = to_dev(keys)
    ko = cuda.empty_like(d_keys)
    pws = edpp.workspace(edpp.split_workspace_bytes(n, 256, "ko"))
    ours = _ours_ms(cuda, lambda: edpp.split(d_keys, 256, keys_out=ko, ws=pws))
    rows.append({"call": "split KO 2^24, 256 buckets", "reference_ms": round(ms.value, 4),
                 "ours_ms": round(ours, 4)})
    del d_keys, ko, pws

    # STREAM copy / triad, 2^28 int32
    n = 1 << 28
    a = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    b = cuda.zeros(n, dtype=cuda.int32, device="cuda")
    c = cuda.empty_like(a)
    for op, name in ((0, "copy"), (3, "triad")):
        assert rc.refcu_time_stream_i32(op, n, 10, ctypes.byref(ms)) == 0
        ours = _ours_ms(cuda, lambda: edpp.stream(name, a, b, 3, out=c))
        rows.append({"call": f"STREAM {name} int32 2^28", "reference_ms": round(ms.value, 4),
                     "ours_ms": round(ours, 4)})
    for r in rows:
        r["speedup"] = round(r["reference_ms"] / r["ours_ms"], 2)
        print(json.dumps(r))
    path = os.environ.get("EDPP_TIMING_JSON")
    if path:
        with open(path, "w") as f:
            json.dump(rows, f, indent=1)
