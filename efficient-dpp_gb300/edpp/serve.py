"""Serving loop: Python harness over edpp_server_* (include/edpp.h).

    srv = Server(pool_bytes=40e9, slots=4)
    rid = srv.submit(op, in0, in1, out0, out1, buckets=64)   # host numpy arrays
    status, timing = srv.wait(rid)
    srv.close()

Host arrays should be pinned (pinned_empty) for asynchronous copies; they must
stay alive until the request has been waited for.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import EdppError, check, lib
from .batch import OP_GATHER, OP_SCAN, OP_SPLIT, Tuning  # noqa: F401


class Request(ctypes.Structure):
    _fields_ = [("op", ctypes.c_int32), ("buckets", ctypes.c_int32), ("length", ctypes.c_int64),
                ("in0", ctypes.c_void_p), ("in1", ctypes.c_void_p), ("out0", ctypes.c_void_p),
                ("out1", ctypes.c_void_p)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("pool_bytes", ctypes.c_size_t), ("slots", ctypes.c_int32),
                ("max_batch_requests", ctypes.c_int32), ("max_batch_elements", ctypes.c_int64),
                ("tuning", Tuning)]


class Timing(ctypes.Structure):
    _fields_ = [("queue_ms", ctypes.c_double), ("latency_ms", ctypes.c_double)]


class Stats(ctypes.Structure):
    _fields_ = [(k, ctypes.c_int64) for k in
                ("submitted", "completed", "batches", "elements_done", "max_requests_per_batch",
                 "max_pool_bytes_used", "max_batches_in_flight")]

    def as_dict(self):
        return {k: int(getattr(self, k)) for k, _ in self._fields_}


_bound = False


def _sigs():
    global _bound
    L = lib()
    if _bound:
        return L
    L.edpp_server_create.argtypes = [ctypes.POINTER(ServerConfig), ctypes.POINTER(ctypes.c_void_p)]
    L.edpp_server_create.restype = ctypes.c_int
    L.edpp_server_submit.argtypes = [ctypes.c_void_p, ctypes.POINTER(Request),
                                     ctypes.POINTER(ctypes.c_uint64)]
    L.edpp_server_submit.restype = ctypes.c_int
    L.edpp_server_wait.argtypes = [ctypes.c_void_p, ctypes.c_uint64, ctypes.c_double,
                                   ctypes.POINTER(Timing)]
    L.edpp_server_wait.restype = ctypes.c_int
    L.edpp_server_get_stats.argtypes = [ctypes.c_void_p, ctypes.POINTER(Stats)]
    L.edpp_server_get_stats.restype = ctypes.c_int
    L.edpp_server_destroy.argtypes = [ctypes.c_void_p]
    L.edpp_server_destroy.restype = None
    _bound = True
    return L


def pinned_empty(n: int, dtype=np.int32) -> np.ndarray:
    """A numpy array in page-locked host memory (via PyTorch)."""
    import torch
    t = torch.empty(int(n), dtype={np.int32: torch.int32}[np.dtype(dtype).type]).pin_memory()
    return t.numpy()  # the view's base keeps the pinned storage alive


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else ctypes.c_void_p(0)


class Server:
    def __init__(self, pool_bytes=1 << 30, slots=4, max_batch_requests=1024,
                 max_batch_elements=0, tuning: Tuning | None = None):
        L = _sigs()
        cfg = ServerConfig(int(pool_bytes), int(slots), int(max_batch_requests),
                           int(max_batch_elements), tuning or Tuning())
        h = ctypes.c_void_p()
        check(L.edpp_server_create(ctypes.byref(cfg), ctypes.byref(h)), "server_create")
        self.h = h
        self._keep = {}

    def submit(self, op, in0, in1=None, out0=None, out1=None, buckets=0) -> int:
        n = len(in0)
        r = Request(int(op), int(buckets), n, _ptr(in0).value, _ptr(in1).value,
                    _ptr(out0).value, _ptr(out1).value)
        rid = ctypes.c_uint64()
        check(_sigs().edpp_server_submit(self.h, ctypes.byref(r), ctypes.byref(rid)), "submit")
        self._keep[rid.value] = (in0, in1, out0, out1)
        return rid.value

    def wait(self, rid, timeout_s=120.0):
        t = Timing()
        st = _sigs().edpp_server_wait(self.h, rid, float(timeout_s), ctypes.byref(t))
        self._keep.pop(rid, None)
        return st, t

    def stats(self) -> dict:
        s = Stats()
        check(_sigs().edpp_server_get_stats(self.h, ctypes.byref(s)), "stats")
        return s.as_dict()

    def close(self):
        if getattr(self, "h", None):
            _sigs().edpp_server_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


__all__ = ["Server", "Request", "ServerConfig", "Timing", "Stats", "pinned_empty", "EdppError",
           "OP_SCAN", "OP_SPLIT", "OP_GATHER"]
