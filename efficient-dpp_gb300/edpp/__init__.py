"""edpp — Python host layer over libedpp's C ABI (include/edpp.h).

The primitives run as hand-written sm_103a CUDA kernels inside libedpp.so;
this module only binds the C ABI with ctypes, takes PyTorch CUDA tensors for
device memory and streams, and raises on a non-zero status.  There is no CPU
fallback: without the built library every call raises EdppError.

Device calls (tensors must be on a CUDA device, contiguous):
    gather(inp, loc, passes=1, out=None)        out[i] = inp[loc[i]]
    scatter(inp, loc, passes=1, out=None)       out[loc[i]] = inp[i]
    scan(x, inclusive=False, algo="lookback")   prefix sums (int32/int64/f32)
    split(keys, buckets, values=None, layout=)  stable multi-split
    stream(op, a, b=None, scalar=3)             STREAM copy/scale/add/triad
Host generators (numpy, seeded splitmix64; see csrc/host/datagen.cpp):
    gen_uniform_i32, gen_uniform_i64, gen_uniform_f32, gen_keys_uniform,
    gen_keys_zipf, gen_permutation
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent.parent
LIB_PATH = PKG_DIR / "lib" / "libedpp.so"

EDPP_OK, EDPP_EINVAL, EDPP_ENOMEM, EDPP_ETIMEOUT, EDPP_ECUDA = 0, 1, 2, 3, 4
SCAN_ALGOS = {"lookback": 0, "rts": 1, "ssa": 2}
LAYOUTS = {"ko": 0, "aos": 1, "soa": 2}
DTYPES = {"int32": 0, "int64": 1, "float32": 2}
STREAM_OPS = ("copy", "scale", "add", "triad")

# Every exported C entry point of include/edpp.h, with its ctypes signature.
_VP, _I, _I64, _U64, _SZ, _F = (ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_uint64,
                               ctypes.c_size_t, ctypes.c_float)
SIGNATURES = {
    "edpp_status_string": (ctypes.c_char_p, [_I]),
    "edpp_version": (_I, []),
    "edpp_sync_status": (_I, [_VP, _I]),
    "edpp_device_fault": (_I, [ctypes.POINTER(ctypes.c_uint), _I]),
    "edpp_gather_i32": (_I, [_VP, _VP, _I64, _VP, _I, _VP]),
    "edpp_scatter_i32": (_I, [_VP, _VP, _I64, _VP, _I, _VP]),
    "edpp_gather_workspace_size": (_SZ, [_I64, _I]),
    "edpp_scatter_workspace_size": (_SZ, [_I64, _I]),
    "edpp_gather_i32_ws": (_I, [_VP, _VP, _I64, _VP, _I, _VP, _SZ, _VP]),
    "edpp_scatter_i32_ws": (_I, [_VP, _VP, _I64, _VP, _I, _VP, _SZ, _VP]),
    "edpp_scan_workspace_size": (_SZ, [_I64, _I, _I]),
    "edpp_scan_exclusive_i32": (_I, [_VP, _VP, _I64, _I, _VP, _SZ, _VP]),
    "edpp_scan_inclusive_i32": (_I, [_VP, _VP, _I64, _I, _VP, _SZ, _VP]),
    "edpp_scan_exclusive_i64": (_I, [_VP, _VP, _I64, _I, _VP, _SZ, _VP]),
    "edpp_scan_inclusive_i64": (_I, [_VP, _VP, _I64, _I, _VP, _SZ, _VP]),
    "edpp_scan_exclusive_f32": (_I, [_VP, _VP, _I64, _I, _VP, _SZ, _VP]),
    "edpp_scan_inclusive_f32": (_I, [_VP, _VP, _I64, _I, _VP, _SZ, _VP]),
    "edpp_split_workspace_size": (_SZ, [_I64, _I, _I]),
    "edpp_split_i32": (_I, [_VP, _VP, _VP, _I64, _I, _I, _VP, _VP, _VP, _SZ, _VP]),
    "edpp_split_wi_workspace_size": (_SZ, [_I64, _I, _I]),
    "edpp_split_i32_wi": (_I, [_VP, _VP, _I64, _I, _I, _VP, _VP, _I, _I, _VP, _SZ, _VP]),
    "edpp_radix_sort_workspace_size": (_SZ, [_I64, _I]),
    "edpp_radix_sort_i32": (_I, [_VP, _VP, _VP, _VP, _I64, _I, _I, _VP, _SZ, _VP]),
    "edpp_hash_join_workspace_size": (_SZ, [_I64, _I64, _I]),
    "edpp_hash_join_count": (_I, [_VP, _I64, _VP, _I64, _I, _VP, _VP, _SZ, _VP]),
    "edpp_hash_join_np_workspace_size": (_SZ, [_I64]),
    "edpp_hash_join_np_count": (_I, [_VP, _I64, _VP, _I64, _VP, _VP, _SZ, _VP]),
    "edpp_access_scale_i32": (_I, [_VP, _VP, _I, _I, _I, _I, _VP]),
    "edpp_access_wg_i32": (_I, [_VP, _I64, _VP, _I, _I, _VP, _VP, _VP]),
    "edpp_cache_heat_i32": (_I, [_VP, _I64, _I, _I, _VP]),
    "edpp_local_scan_i32": (_I, [_VP, _VP, _I, _I, _I, _VP]),
    "edpp_gather_prefers_direct": (_I, [_I64]),
    "edpp_gather_tiled_workspace_size": (_SZ, [_I64]),
    "edpp_scatter_tiled_workspace_size": (_SZ, [_I64]),
    "edpp_gather_i32_tiled": (_I, [_VP, _VP, _I64, _VP, _I, _VP, _SZ, _VP]),
    "edpp_scatter_i32_tiled": (_I, [_VP, _VP, _I64, _VP, _I, _VP, _SZ, _VP]),
    "edpp_stream_copy_f32": (_I, [_VP, _VP, _I64, _VP]),
    "edpp_stream_scale_f32": (_I, [_VP, _VP, _F, _I64, _VP]),
    "edpp_stream_add_f32": (_I, [_VP, _VP, _VP, _I64, _VP]),
    "edpp_stream_triad_f32": (_I, [_VP, _VP, _VP, _F, _I64, _VP]),
    "edpp_stream_copy_i32": (_I, [_VP, _VP, _I64, _VP]),
    "edpp_stream_scale_i32": (_I, [_VP, _VP, ctypes.c_int32, _I64, _VP]),
    "edpp_stream_add_i32": (_I, [_VP, _VP, _VP, _I64, _VP]),
    "edpp_stream_triad_i32": (_I, [_VP, _VP, _VP, ctypes.c_int32, _I64, _VP]),
    "edpp_selftest_lookback_timeout": (_I, [_VP, _VP, _I64, _U64, _VP, _SZ, _VP]),
    "edpp_scan_exclusive_i32_noalloc": (_I, [_VP, _VP, _I64, _VP]),
    "edpp_scan_exclusive_i32_noalloc_max_length": (_I64, []),
    # per-size-class tuning of the plain primitives
    "edpp_tune_variants": (_I, [_I]),
    "edpp_tune_set": (_I, [_I, _I, _I, _I, _F]),
    "edpp_tune_get": (_I, [_I, _I, _I64, _VP]),
    "edpp_tune_load": (_I, [ctypes.c_char_p]),
    "edpp_tune_save": (_I, [ctypes.c_char_p]),
    "edpp_tune_clear": (None, []),
    "edpp_autotune_plain": (_I, [_I, _VP, _VP, _VP, _I64, _I, _VP, _SZ, _VP, _I, _VP, _SZ, _VP,
                                 ctypes.POINTER(ctypes.c_float), _VP]),
    # batched segments
    "edpp_batch_plan_create": (_I, [_VP, _I, _VP, ctypes.POINTER(_VP)]),
    "edpp_batch_plan_destroy": (None, [_VP]),
    "edpp_batch_plan_workspace_size": (_SZ, [_VP]),
    "edpp_batch_plan_num_tasks": (_I, [_VP]),
    "edpp_batch_plan_upload": (_I, [_VP, _VP, _SZ, _VP]),
    "edpp_batch_launch": (_I, [_VP, _VP, _VP, _VP, _VP, _VP, _SZ, _VP]),
    "edpp_batch_autotune": (_I, [_VP, _I, _VP, _VP, _VP, _VP, _VP, _SZ, _VP, _I, _VP,
                                 ctypes.POINTER(ctypes.c_float)]),
    "edpp_batch_plain_workspace_size": (_SZ, [_VP, _I]),
    "edpp_batch_run_plain": (_I, [_VP, _I, _VP, _VP, _VP, _VP, _VP, _SZ, _VP]),
    "edpp_gen_batch_inputs": (None, [_VP, _I, _U64, _VP, _VP]),
    # serving (edpp.serve binds these with structure types)
    "edpp_server_create": (_I, [_VP, _VP]),
    "edpp_server_submit": (_I, [_VP, _VP, _VP]),
    "edpp_server_wait": (_I, [_VP, _U64, ctypes.c_double, _VP]),
    "edpp_server_get_stats": (_I, [_VP, _VP]),
    "edpp_server_destroy": (None, [_VP]),
    # host generators
    "edpp_gen_draw": (_U64, [_U64, _U64]),
    "edpp_gen_uniform_i32": (None, [_VP, _I64, _U64, _I64, _I64]),
    "edpp_gen_uniform_i64": (None, [_VP, _I64, _U64, _I64, _I64]),
    "edpp_gen_uniform_f32": (None, [_VP, _I64, _U64, _F, _F]),
    "edpp_gen_keys_uniform": (None, [_VP, _I64, _U64]),
    "edpp_gen_keys_zipf": (None, [_VP, _I64, _U64, _I, ctypes.c_double]),
    "edpp_gen_permutation_i32": (None, [_VP, _I64, _U64]),
}


class EdppError(RuntimeError):
    """A C-ABI call returned a non-zero status, or the library is missing."""

    def __init__(self, status: int, what: str = ""):
        self.status = status
        name = {1: "EINVAL", 2: "ENOMEM", 3: "ETIMEOUT", 4: "ECUDA"}.get(status, str(status))
        super().__init__(f"edpp {what}: {name}")


_lib = None


def lib() -> ctypes.CDLL:
    """The loaded libedpp.so (built by efficient-dpp_gb300/build.py)."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("EDPP_LIB", LIB_PATH))
        if not path.exists():
            raise EdppError(-1, f"library not built: {path} (run __graft_entry__.build())")
        L = ctypes.CDLL(str(path))
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != EDPP_OK:
        raise EdppError(status, what)


# ---------------------------------------------------------------------------
# device helpers
def _torch():
    import torch  # imported lazily: the generators and the ABI load need no torch
    return torch


def _cuda_tensor(t, dtype=None, name="tensor"):
    torch = _torch()
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if dtype is not None and t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    return t


def _p(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr() if t is not None else 0)


def current_stream_handle() -> ctypes.c_void_p:
    return ctypes.c_void_p(_torch().cuda.current_stream().cuda_stream)


def workspace(nbytes: int, device=None):
    torch = _torch()
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device or "cuda")


def sync_status(clear: bool = True) -> int:
    """Wait for the current stream; EDPP_ETIMEOUT if a bounded wait expired."""
    return lib().edpp_sync_status(current_stream_handle(), int(clear))


# ---------------------------------------------------------------------------
# primitives
def _gs(kind, inp, loc, passes, out, method, ws):
    torch = _torch()
    _cuda_tensor(inp, torch.int32, "inp")
    _cuda_tensor(loc, torch.int32, "loc")
    n = loc.numel()
    if kind == "gather" and inp.numel() < n:
        raise ValueError("inp shorter than loc")
    if out is None:
        out = torch.zeros(n, dtype=torch.int32, device=loc.device)
    st = current_stream_handle()
    if method == "auto":  # the faster schedule for this size
        method = ("sweep" if kind == "gather" and lib().edpp_gather_prefers_direct(n)
                  else "tiled")
        passes = 1 if method == "sweep" else passes
    if method == "sweep":
        f = lib().edpp_gather_i32 if kind == "gather" else lib().edpp_scatter_i32
        check(f(_p(inp), _p(out), n, _p(loc), int(passes), st), kind)
    elif method in ("partition", "tiled"):
        need = gs_workspace_bytes(kind, n, passes, method)
        if ws is None:
            ws = workspace(need, loc.device)
        if method == "partition":
            f = lib().edpp_gather_i32_ws if kind == "gather" else lib().edpp_scatter_i32_ws
        else:
            f = lib().edpp_gather_i32_tiled if kind == "gather" else lib().edpp_scatter_i32_tiled
        check(f(_p(inp), _p(out), n, _p(loc), int(passes), _p(ws), ws.numel(), st), kind)
    else:
        raise ValueError(method)
    return out


# ---------------------------------------------------------------------------
# per-size-class tuning (include/edpp.h edpp_tune_*)
TUNE_SCAN_LOOKBACK, TUNE_SCAN_RTS, TUNE_GATHER = 0, 1, 2
TUNE_NAMES = {TUNE_SCAN_LOOKBACK: "scan_lookback", TUNE_SCAN_RTS: "scan_rts",
              TUNE_GATHER: "gather"}


def tune_get(prim: int, elem_bytes: int, n: int):
    """(variant a call of n elements takes now, whether the table has an entry)."""
    v = ctypes.c_int(0)
    st = lib().edpp_tune_get(prim, elem_bytes, int(n), ctypes.byref(v))
    return v.value, st == EDPP_OK


def tune_set(prim: int, elem_bytes: int, log2_n: int, variant: int, ms: float = 0.0):
    check(lib().edpp_tune_set(prim, elem_bytes, log2_n, variant, ms), "tune_set")


def tune_load(path=None) -> int:
    """Replace the table from a file (None: the committed default table)."""
    return lib().edpp_tune_load(None if path is None else str(path).encode())


def tune_save(path):
    check(lib().edpp_tune_save(str(path).encode()), "tune_save")


def autotune_plain(prim: int, x, out, ws, loc=None, reps: int = 5, flush=None):
    """Time every variant of `prim` at x's length on these arrays, record the
    fastest in the table; returns (variant, ms, [ms of every variant]).
    flush: a CUDA tensor larger than L2, overwritten before every timed call
    (cold-L2 timing); None times back to back (warm)."""
    best = ctypes.c_int(-1)
    ms = ctypes.c_float(0.0)
    nv = lib().edpp_tune_variants(prim)
    each = (ctypes.c_float * max(nv, 1))()
    elem = x.element_size()
    check(lib().edpp_autotune_plain(prim, _p(x), _p(out), _p(loc) if loc is not None else None,
                                    x.numel(), elem, _p(ws), ws.numel(), current_stream_handle(),
                                    reps, _p(flush) if flush is not None else None,
                                    flush.numel() * flush.element_size() if flush is not None else 0,
                                    ctypes.byref(best), ctypes.byref(ms), each),
          "autotune_plain")
    return best.value, ms.value, [each[i] for i in range(nv)]


def gs_workspace_bytes(kind: str, n: int, passes: int, method: str = "partition") -> int:
    if method in ("tiled", "auto"):
        f = (lib().edpp_gather_tiled_workspace_size if kind == "gather"
             else lib().edpp_scatter_tiled_workspace_size)
        return f(int(n))
    if method == "sweep":
        return 0
    f = lib().edpp_gather_workspace_size if kind == "gather" else lib().edpp_scatter_workspace_size
    return f(int(n), int(passes))


def gather(inp, loc, passes: int = 1, out=None, method: str = "sweep", ws=None):
    """out[i] = inp[loc[i]].  method "sweep": one launch per pass window, each
    reading all of loc (the reference's schedule); "partition": the windows
    as partitions (passes=0 sizes them to L2); "tiled": shared-memory
    windows; "auto": the faster of the single direct sweep and "tiled" for
    this size (the result does not depend on passes or method)."""
    return _gs("gather", inp, loc, passes, out, method, ws)


def scatter(inp, loc, passes: int = 1, out=None, method: str = "sweep", ws=None):
    """out[loc[i]] = inp[i]; methods as gather."""
    return _gs("scatter", inp, loc, passes, out, method, ws)


_SCAN_FN = {
    ("int32", False): "edpp_scan_exclusive_i32", ("int32", True): "edpp_scan_inclusive_i32",
    ("int64", False): "edpp_scan_exclusive_i64", ("int64", True): "edpp_scan_inclusive_i64",
    ("float32", False): "edpp_scan_exclusive_f32", ("float32", True): "edpp_scan_inclusive_f32",
}


def scan_workspace_bytes(n: int, dtype: str, algo: str = "lookback") -> int:
    return lib().edpp_scan_workspace_size(int(n), DTYPES[dtype], SCAN_ALGOS[algo])


def scan(x, inclusive: bool = False, algo: str = "lookback", out=None, ws=None):
    torch = _torch()
    _cuda_tensor(x, None, "x")
    dt = str(x.dtype).replace("torch.", "")
    if dt not in DTYPES:
        raise TypeError(f"scan supports int32, int64, float32, got {x.dtype}")
    n = x.numel()
    if out is None:
        out = torch.empty_like(x)
    need = scan_workspace_bytes(n, dt, algo)
    if ws is None:
        ws = workspace(need, x.device)
    fn = getattr(lib(), _SCAN_FN[(dt, bool(inclusive))])
    check(fn(_p(x), _p(out), n, SCAN_ALGOS[algo], _p(ws), ws.numel(), current_stream_handle()),
          "scan")
    return out


def split_workspace_bytes(n: int, buckets: int, layout: str = "soa") -> int:
    return lib().edpp_split_workspace_size(int(n), int(buckets), LAYOUTS[layout])


def split(keys, buckets: int, values=None, layout: str | None = None, bucket_start: bool = False,
          keys_out=None, values_out=None, ws=None):
    """Stable multi-split by key & (buckets-1).

    layout "ko": keys only; "soa": keys and values tensors; "aos": keys is an
    (n, 2) int32 tensor of {key, value} pairs.  Returns (keys_out,
    values_out or None, bucket_start or None)."""
    torch = _torch()
    if layout is None:
        layout = "ko" if values is None else "soa"
    _cuda_tensor(keys, torch.int32, "keys")
    if layout == "aos":
        if keys.dim() != 2 or keys.shape[1] != 2:
            raise ValueError("aos keys must have shape (n, 2)")
        n = keys.shape[0]
    else:
        n = keys.numel()
    if layout == "soa":
        _cuda_tensor(values, torch.int32, "values")
    if keys_out is None:
        keys_out = torch.empty_like(keys)
    if layout == "soa" and values_out is None:
        values_out = torch.empty_like(values)
    start = torch.empty(buckets, dtype=torch.int32, device=keys.device) if bucket_start else None
    need = split_workspace_bytes(n, buckets, layout)
    if ws is None:
        ws = workspace(need, keys.device)
    check(lib().edpp_split_i32(_p(keys), _p(keys_out), _p(start), n, int(buckets),
                               LAYOUTS[layout], _p(values if layout == "soa" else None),
                               _p(values_out if layout == "soa" else None), _p(ws), ws.numel(),
                               current_stream_handle()), "split")
    return keys_out, (values_out if layout == "soa" else None), start


def split_wi(keys, buckets, values=None, layout=None, local_size=256, grid_size=32768):
    """The reference WI_split's order (see edpp_split_i32_wi)."""
    torch = _torch()
    if layout is None:
        layout = "ko" if values is None else "soa"
    _cuda_tensor(keys, torch.int32, "keys")
    n = keys.shape[0]
    ko = torch.empty_like(keys)
    vo = torch.empty_like(values) if layout == "soa" else None
    ws = workspace(lib().edpp_split_wi_workspace_size(n, int(buckets), LAYOUTS[layout]),
                   keys.device)
    check(lib().edpp_split_i32_wi(_p(keys), _p(ko), n, int(buckets), LAYOUTS[layout],
                                  _p(values if layout == "soa" else None), _p(vo),
                                  int(local_size), int(grid_size), _p(ws), ws.numel(),
                                  current_stream_handle()), "split_wi")
    return ko, vo


def radix_sort(keys, values=None, begin_bit=0, end_bit=32, keys_out=None, values_out=None,
               ws=None):
    """Stable LSD radix sort by the key's bit pattern (unsigned order)."""
    torch = _torch()
    _cuda_tensor(keys, torch.int32, "keys")
    n = keys.numel()
    if keys_out is None:
        keys_out = torch.empty_like(keys)
    if values is not None:
        _cuda_tensor(values, torch.int32, "values")
        if values_out is None:
            values_out = torch.empty_like(values)
    if ws is None:
        ws = workspace(lib().edpp_radix_sort_workspace_size(n, int(values is not None)),
                       keys.device)
    check(lib().edpp_radix_sort_i32(_p(keys), _p(keys_out), _p(values), _p(values_out), n,
                                    int(begin_bit), int(end_bit), _p(ws), ws.numel(),
                                    current_stream_handle()), "radix_sort")
    return keys_out, values_out


def hash_join_count(r_keys, s_keys, buckets: int = 0, ws=None, partitioned: bool = True,
                    count=None) -> int:
    """Number of equal-key pairs between R and S.  partitioned=True: split
    both sides, one shared-memory table per partition; False: one table in
    device memory built from S and probed with R.  With `count` (a 1-element
    int64 CUDA tensor) the result stays on the device and None is returned."""
    torch = _torch()
    _cuda_tensor(r_keys, torch.int32, "r_keys")
    _cuda_tensor(s_keys, torch.int32, "s_keys")
    cnt = count if count is not None else torch.zeros(1, dtype=torch.int64, device=r_keys.device)
    st = current_stream_handle()
    if partitioned:
        if ws is None:
            ws = workspace(lib().edpp_hash_join_workspace_size(r_keys.numel(), s_keys.numel(),
                                                               int(buckets)), r_keys.device)
        check(lib().edpp_hash_join_count(_p(r_keys), r_keys.numel(), _p(s_keys), s_keys.numel(),
                                         int(buckets), _p(cnt), _p(ws), ws.numel(), st),
              "hash_join_count")
    else:
        if ws is None:
            ws = workspace(lib().edpp_hash_join_np_workspace_size(s_keys.numel()), r_keys.device)
        check(lib().edpp_hash_join_np_count(_p(s_keys), s_keys.numel(), _p(r_keys), r_keys.numel(),
                                            _p(cnt), _p(ws), ws.numel(), st), "hash_join_np_count")
    return None if count is not None else int(cnt.item())


ACCESS_PATTERNS = {"column": 0, "row": 1, "mixed": 2, "vec": 3}
LOCAL_SCAN_SCHEMES = {"lm": 0, "reg": 1, "lm_reg": 2, "warp": 3}


def access_scale(inp, out, repeat: int, pattern: str, local_size: int = 512,
                 grid_size: int = 32768):
    """out[i] = 3*in[i] for i < local_size*grid_size*repeat, with the given
    thread-to-element map."""
    torch = _torch()
    _cuda_tensor(inp, torch.int32, "in")
    _cuda_tensor(out, torch.int32, "out")
    n = local_size * grid_size * repeat
    if inp.numel() < n or out.numel() < n:
        raise ValueError("buffers hold fewer than local_size*grid_size*repeat elements")
    check(lib().edpp_access_scale_i32(_p(inp), _p(out), repeat, ACCESS_PATTERNS[pattern],
                                      local_size, grid_size, current_stream_handle()),
          "access_scale")


def access_wg(inp, order, local_size: int = 1, out=None, ticket=None):
    """Block-order sweep: per-chunk sums of the low bits, chunk visit order
    `order` (int32 CUDA tensor of grid_size chunk ids)."""
    torch = _torch()
    _cuda_tensor(inp, torch.int32, "in")
    _cuda_tensor(order, torch.int32, "order")
    g = order.numel()
    out = out if out is not None else torch.zeros(g, dtype=torch.int64, device=inp.device)
    ticket = ticket if ticket is not None else torch.zeros(1, dtype=torch.int32, device=inp.device)
    check(lib().edpp_access_wg_i32(_p(inp), inp.numel(), _p(order), g, local_size, _p(ticket),
                                   _p(out), current_stream_handle()), "access_wg")
    return out


def cache_heat(data, local_size: int = 512, grid_size: int = 32768):
    torch = _torch()
    _cuda_tensor(data, torch.int32, "data")
    check(lib().edpp_cache_heat_i32(_p(data), data.numel(), local_size, grid_size,
                                    current_stream_handle()), "cache_heat")


def local_scan(inp, tile_size: int, scheme: str, repeat: int = 1, out=None):
    """Exclusive scan of the first 512*tile_size elements by one block."""
    torch = _torch()
    _cuda_tensor(inp, torch.int32, "in")
    n = 512 * tile_size
    if inp.numel() < n:
        raise ValueError("input holds fewer than 512*tile_size elements")
    out = out if out is not None else torch.empty(n, dtype=torch.int32, device=inp.device)
    check(lib().edpp_local_scan_i32(_p(inp), _p(out), tile_size, LOCAL_SCAN_SCHEMES[scheme],
                                    repeat, current_stream_handle()), "local_scan")
    return out


def stream(op: str, a, b=None, scalar=3, out=None):
    torch = _torch()
    if op not in STREAM_OPS:
        raise ValueError(op)
    _cuda_tensor(a, None, "a")
    suffix = {torch.float32: "f32", torch.int32: "i32"}.get(a.dtype)
    if suffix is None:
        raise TypeError("stream supports float32 and int32")
    if out is None:
        out = torch.empty_like(a)
    n = a.numel()
    f = getattr(lib(), f"edpp_stream_{op}_{suffix}")
    s = float(scalar) if suffix == "f32" else int(scalar)
    st = current_stream_handle()
    if op == "copy":
        r = f(_p(a), _p(out), n, st)
    elif op == "scale":
        r = f(_p(a), _p(out), s, n, st)
    elif op == "add":
        r = f(_p(a), _p(b), _p(out), n, st)
    else:
        r = f(_p(a), _p(b), _p(out), s, n, st)
    check(r, f"stream_{op}")
    return out


def selftest_lookback_timeout(n: int, timeout_ns: int, device="cuda") -> int:
    """Run the look-back scan with tile 0 never published; returns the
    status edpp_sync_status reports afterwards (EDPP_ETIMEOUT expected)."""
    torch = _torch()
    x = torch.ones(n, dtype=torch.int32, device=device)
    y = torch.zeros_like(x)
    ws = workspace(scan_workspace_bytes(n, "int32"), device)
    check(lib().edpp_selftest_lookback_timeout(_p(x), _p(y), n, int(timeout_ns), _p(ws), ws.numel(),
                                               current_stream_handle()), "selftest")
    return sync_status(clear=True)


# ---------------------------------------------------------------------------
# seeded host generators (numpy)
def _np_ptr(a: np.ndarray) -> ctypes.c_void_p:
    return ctypes.c_void_p(a.ctypes.data)


def gen_uniform_i32(n: int, seed: int, lo: int, hi: int) -> np.ndarray:
    a = np.empty(n, dtype=np.int32)
    lib().edpp_gen_uniform_i32(_np_ptr(a), n, seed, lo, hi)
    return a


def gen_uniform_i64(n: int, seed: int, lo: int, hi: int) -> np.ndarray:
    a = np.empty(n, dtype=np.int64)
    lib().edpp_gen_uniform_i64(_np_ptr(a), n, seed, lo, hi)
    return a


def gen_uniform_f32(n: int, seed: int, lo: float, hi: float) -> np.ndarray:
    a = np.empty(n, dtype=np.float32)
    lib().edpp_gen_uniform_f32(_np_ptr(a), n, seed, lo, hi)
    return a


def gen_keys_uniform(n: int, seed: int) -> np.ndarray:
    a = np.empty(n, dtype=np.int32)
    lib().edpp_gen_keys_uniform(_np_ptr(a), n, seed)
    return a


def gen_keys_zipf(n: int, seed: int, buckets: int, s: float = 1.0) -> np.ndarray:
    a = np.empty(n, dtype=np.int32)
    lib().edpp_gen_keys_zipf(_np_ptr(a), n, seed, buckets, s)
    return a


def gen_permutation(n: int, seed: int) -> np.ndarray:
    a = np.empty(n, dtype=np.int32)
    lib().edpp_gen_permutation_i32(_np_ptr(a), n, seed)
    return a
