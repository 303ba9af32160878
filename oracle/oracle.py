"""ctypes bindings of the oracle — TEST INFRASTRUCTURE ONLY.

Used as the checker by tests/, __graft_entry__.smoke() and the cpu_baseline
leg of bench.py; never by the product.  Wraps:
  _build/liboracle.so    C restatement of the reference (edpp_oracle.c)
  _ref/libref_omp.so     the reference's own OpenMP functions (x86, built
                         only where the reference tree is present)
  _build/libref_cuda.so  runner of the reference's CUDA kernels (cubins)
  _ref/libref_cl_split_*.so  the reference's OpenCL WI_split kernels compiled
                         as C (ref_cl_shim.h, ref_cl_runner.c)
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
_VP, _I, _I64, _D = ctypes.c_void_p, ctypes.c_int, ctypes.c_int64, ctypes.c_double

_SIG = {
    "orc_gather_i32": (None, [_VP, _VP, _I64, _VP, _I]),
    "orc_scatter_i32": (None, [_VP, _VP, _I64, _VP, _I]),
    "orc_scan_excl_i32": (None, [_VP, _VP, _I64]),
    "orc_scan_incl_i32": (None, [_VP, _VP, _I64]),
    "orc_scan_excl_i64": (None, [_VP, _VP, _I64]),
    "orc_scan_incl_i64": (None, [_VP, _VP, _I64]),
    "orc_scan_f32_in_f64": (None, [_VP, _VP, _I64, _I]),
    "orc_scan_ssa_omp_i32": (_D, [_VP, _VP, _I64, _I]),
    "orc_scan_rts_omp_i32": (_D, [_VP, _VP, _I64, _I]),
    "orc_gather_omp_i32": (_D, [_VP, _VP, _VP, _I64, _I]),
    "orc_scatter_omp_i32": (_D, [_VP, _VP, _VP, _I64, _I]),
    "orc_stream_f32": (_D, [_I, _VP, _VP, _VP, ctypes.c_float, _I64, _I]),
    "orc_stream_i32": (_D, [_I, _VP, _VP, _VP, ctypes.c_int32, _I64, _I]),
    "orc_split_stable": (None, [_VP, _VP, _I64, _I, _I, _VP, _VP, _VP]),
    "orc_split_cuda_ballot": (None, [_VP, _I64, _I, _VP]),
    "orc_split_single": (None, [_VP, _I64, _I, _I, _I, _VP]),
    "orc_split_stable_timed": (_D, [_VP, _VP, _I64, _I, _I, _VP, _VP]),
    "orc_split_wi": (None, [_VP, _VP, _I64, _I, _I, _I, _I, _VP, _VP]),
    "orc_join_count": (ctypes.c_uint64, [_VP, _I64, _VP, _I64]),
    "orc_compute_bandwidth": (_D, [ctypes.c_uint64, _I, _D]),
    "orc_average_hampel": (_D, [_VP, _I]),
    "orc_max_threads": (_I, []),
    "orc_gen_permutation_i32": (None, [_VP, _I64, ctypes.c_uint64]),
}

_lib = None


def build():
    import importlib.util
    spec = importlib.util.spec_from_file_location("edpp_oracle_build", HERE / "build.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.build_all()


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        path = HERE / "_build" / "liboracle.so"
        if not path.exists():
            build()
        L = ctypes.CDLL(str(path))
        for k, (r, a) in _SIG.items():
            f = getattr(L, k)
            f.restype = r
            f.argtypes = a
        _lib = L
    return _lib


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


# ---- restatement ------------------------------------------------------------
def gather(inp, loc, passes=1, out=None):
    inp, loc = _c(inp, np.int32), _c(loc, np.int32)
    out = np.zeros(len(loc), np.int32) if out is None else _c(out, np.int32).copy()
    lib().orc_gather_i32(_p(inp), _p(out), len(loc), _p(loc), passes)
    return out


def scatter(inp, loc, passes=1, out=None):
    inp, loc = _c(inp, np.int32), _c(loc, np.int32)
    out = np.zeros(len(loc), np.int32) if out is None else _c(out, np.int32).copy()
    lib().orc_scatter_i32(_p(inp), _p(out), len(loc), _p(loc), passes)
    return out


def scan(x, inclusive=False):
    """Sequential wrapping scan for int32/int64; f32 -> f64 accumulation."""
    x = np.ascontiguousarray(x)
    if x.dtype == np.int32:
        out = np.empty_like(x)
        (lib().orc_scan_incl_i32 if inclusive else lib().orc_scan_excl_i32)(_p(x), _p(out), len(x))
    elif x.dtype == np.int64:
        out = np.empty_like(x)
        (lib().orc_scan_incl_i64 if inclusive else lib().orc_scan_excl_i64)(_p(x), _p(out), len(x))
    elif x.dtype == np.float32:
        out = np.empty(len(x), np.float64)
        lib().orc_scan_f32_in_f64(_p(x), _p(out), len(x), int(inclusive))
    else:
        raise TypeError(x.dtype)
    return out


def scan_omp(x, scheme="ssa", nthreads=0):
    """OpenMP port of scan_SSA_omp / scan_RTS_omp; returns (out, ms)."""
    x = _c(x, np.int32)
    out = np.empty_like(x)
    f = lib().orc_scan_ssa_omp_i32 if scheme == "ssa" else lib().orc_scan_rts_omp_i32
    ms = f(_p(x), _p(out), len(x), nthreads)
    return out, ms


def gather_omp(inp, idx, nthreads=0, out=None):
    """Timed OpenMP gather; pass `out` to reuse a (touched) buffer."""
    out = np.empty(len(idx), np.int32) if out is None else out
    ms = lib().orc_gather_omp_i32(_p(inp), _p(out), _p(idx), len(idx), nthreads)
    return out, ms


def scatter_omp(inp, idx, nthreads=0, out=None):
    out = np.empty(len(idx), np.int32) if out is None else out
    ms = lib().orc_scatter_omp_i32(_p(inp), _p(out), _p(idx), len(idx), nthreads)
    return out, ms


def stream(op, a, b=None, scalar=3, nthreads=0, out=None):
    ops = {"copy": 0, "scale": 1, "add": 2, "triad": 3}
    a = np.ascontiguousarray(a)
    b = a if b is None else np.ascontiguousarray(b)
    c = np.empty_like(a) if out is None else out
    if a.dtype == np.float32:
        ms = lib().orc_stream_f32(ops[op], _p(a), _p(b), _p(c), float(scalar), len(a), nthreads)
    else:
        ms = lib().orc_stream_i32(ops[op], _p(a), _p(b), _p(c), int(scalar), len(a), nthreads)
    return c, ms


def split(keys, buckets, values=None, layout=None):
    """Stable split.  layout 'ko' | 'soa' | 'aos' (keys shape (n,2))."""
    if layout is None:
        layout = "ko" if values is None else "soa"
    lay = {"ko": 0, "aos": 1, "soa": 2}[layout]
    keys = _c(keys, np.int32)
    n = keys.shape[0]
    ko = np.empty_like(keys)
    vals = _c(values, np.int32) if layout == "soa" else None
    vo = np.empty_like(vals) if vals is not None else None
    start = np.empty(buckets, np.int32)
    lib().orc_split_stable(_p(keys), _p(vals), n, buckets, lay, _p(ko), _p(vo), _p(start))
    return ko, vo, start


def split_timed(keys, buckets, values=None, layout="soa"):
    lay = {"ko": 0, "aos": 1, "soa": 2}[layout]
    keys = _c(keys, np.int32)
    ko = np.empty_like(keys)
    vals = _c(values, np.int32) if values is not None else None
    vo = np.empty_like(vals) if vals is not None else None
    ms = lib().orc_split_stable_timed(_p(keys), _p(vals), keys.shape[0], buckets, lay, _p(ko),
                                      _p(vo))
    return ko, vo, ms


def split_cuda_ballot(keys, bucket_bits):
    keys = _c(keys, np.int32)
    out = np.empty_like(keys)
    lib().orc_split_cuda_ballot(_p(keys), len(keys), bucket_bits, _p(out))
    return out


def split_single(data, buckets, aos=False, groups=39):
    data = _c(data, np.int32)
    out = np.empty_like(data)
    n = data.shape[0]
    lib().orc_split_single(_p(data), n, buckets, int(aos), groups, _p(out))
    return out


def split_wi(keys, buckets, values=None, aos=False, local_size=256, grid_size=32768):
    """The reference WI_split's output order (restated literally)."""
    keys = _c(keys, np.int32)
    out = np.empty_like(keys)
    vals = _c(values, np.int32) if values is not None else None
    vo = np.empty_like(vals) if vals is not None else None
    lib().orc_split_wi(_p(keys), _p(vals), keys.shape[0], buckets, int(aos), local_size, grid_size,
                       _p(out), _p(vo))
    return out, vo


def join_count(r, s):
    r, s = _c(r, np.int32), _c(s, np.int32)
    return int(lib().orc_join_count(_p(r), len(r), _p(s), len(s)))


def average_hampel(x):
    x = _c(x, np.float64)
    return lib().orc_average_hampel(_p(x), len(x))


def compute_bandwidth(num, word_size, ms):
    return lib().orc_compute_bandwidth(num, word_size, ms)


def max_threads():
    return lib().orc_max_threads()


def gen_permutation(n, seed):
    """Seeded Fisher-Yates permutation of [0, n): the same array as the
    library's generator, made without loading the library."""
    a = np.empty(n, np.int32)
    lib().orc_gen_permutation_i32(_p(a), n, seed)
    return a


# ---- the reference itself -------------------------------------------------------
_ref = None


def ref_omp():
    """The reference's OpenMP functions, or None where they were not built."""
    global _ref
    if _ref is None:
        path = HERE / "_ref" / "libref_omp.so"
        if not path.exists():
            return None
        L = ctypes.CDLL(str(path))
        for name in ("ref_gather", "ref_scatter"):
            getattr(L, name).restype = _D
            getattr(L, name).argtypes = [_VP, _VP, _VP, ctypes.c_uint64]
        for name in ("ref_scan_ssa", "ref_scan_rts", "ref_scan_tbb", "ref_copy", "ref_scale"):
            getattr(L, name).restype = _D
            getattr(L, name).argtypes = [_VP, _VP, ctypes.c_uint64]
        L.ref_average_hampel.restype = _D
        L.ref_average_hampel.argtypes = [_VP, _I]
        L.ref_compute_bandwidth.restype = _D
        L.ref_compute_bandwidth.argtypes = [ctypes.c_uint64, _I, _D]
        _ref = L
    return _ref


_refcl = {}


def ref_cl_split(layout):
    """The reference's own WI_split (its OpenCL kernels compiled as C), for
    layout 'ko' | 'soa' | 'aos', or None where it was not built."""
    if layout not in _refcl:
        path = HERE / "_ref" / f"libref_cl_split_{layout}.so"
        if not path.exists():
            return None
        L = ctypes.CDLL(str(path))
        L.ref_wi_split.restype = _I
        L.ref_wi_split.argtypes = [_VP, _VP, _I, _I, _I, _I, _VP, _VP]
        _refcl[layout] = L
    return _refcl[layout]


def ref_wi_split(keys, buckets, values=None, aos=False, local_size=256, grid_size=32768):
    """Run the reference's WI_split (KO, SOA with values, or AOS pairs);
    returns (out, values_out) or None where it is not built."""
    layout = "aos" if aos else ("soa" if values is not None else "ko")
    L = ref_cl_split(layout)
    if L is None:
        return None
    keys = _c(keys, np.int32)
    out = np.zeros_like(keys)
    vals = _c(values, np.int32) if layout == "soa" else None
    vo = np.zeros_like(vals) if vals is not None else None
    rc = L.ref_wi_split(_p(keys), _p(vals), keys.shape[0], buckets, local_size, grid_size, _p(out),
                        _p(vo))
    if rc != 0:
        raise ValueError("the reference cannot run this WI_split configuration")
    return out, vo


_refcu = None


def ref_cuda():
    """Runner of the reference's CUDA kernels (needs a GPU), or None."""
    global _refcu
    if _refcu is None:
        path = HERE / "_build" / "libref_cuda.so"
        if not path.exists():
            return None
        L = ctypes.CDLL(str(path))
        L.refcu_init.argtypes = [ctypes.c_char_p]
        L.refcu_split.argtypes = [_VP, _VP, ctypes.c_longlong, _I]
        L.refcu_gather_scatter.argtypes = [_I, _VP, _VP, _VP, ctypes.c_longlong]
        L.refcu_stream_i32.argtypes = [_I, _VP, _VP, _VP, ctypes.c_longlong]
        L.refcu_cub_exclusive_sum_i32.argtypes = [_VP, _VP, ctypes.c_longlong]
        FP = ctypes.POINTER(ctypes.c_float)
        L.refcu_time_gather_scatter.argtypes = [_I, _VP, ctypes.c_longlong, _I, FP]
        L.refcu_time_cub_scan.argtypes = [ctypes.c_longlong, _I, FP]
        L.refcu_time_split.argtypes = [_VP, ctypes.c_longlong, _I, _I, FP]
        L.refcu_time_stream_i32.argtypes = [_I, ctypes.c_longlong, _I, FP]
        rc = L.refcu_init(str(HERE / "_ref").encode())
        if rc != 0:
            return None
        _refcu = L
    return _refcu
