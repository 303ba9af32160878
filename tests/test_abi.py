"""The C ABI library: loads without a GPU, exports every entry point that
include/edpp.h declares, and rejects bad arguments before touching a device.
"""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def declared(header: str):
    text = (ROOT / "include" / header).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(edpp_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = declared("edpp.h")
    assert "edpp_gather_i32" in names and "edpp_split_i32" in names
    assert len(names) >= 20


def test_library_exports_every_declared_symbol(edpp):
    lib = edpp.lib()
    missing = [n for n in declared("edpp.h") if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header(edpp):
    missing = [n for n in declared("edpp.h") if n not in edpp.SIGNATURES]
    assert not missing, missing


def test_status_strings(edpp):
    lib = edpp.lib()
    assert lib.edpp_status_string(0) == b"ok"
    assert b"invalid" in lib.edpp_status_string(1)
    assert b"timeout" in lib.edpp_status_string(3) or b"expired" in lib.edpp_status_string(3)
    assert lib.edpp_version() >= 10000


def test_workspace_queries(edpp):
    lib = edpp.lib()
    assert lib.edpp_scan_workspace_size(0, 0, 0) == 0
    a = lib.edpp_scan_workspace_size(1 << 24, 0, 0)
    b = lib.edpp_scan_workspace_size(1 << 25, 0, 0)
    assert 0 < a < b
    assert lib.edpp_scan_workspace_size(1 << 24, 1, 0) > a  # int64 state is larger
    assert lib.edpp_split_workspace_size(1 << 20, 256, 2) > 0
    assert lib.edpp_split_workspace_size(1 << 20, 3, 2) == 0  # not a power of two
    assert lib.edpp_split_workspace_size(1 << 20, 16384, 2) == 0  # beyond 8192
    # from 2048 buckets the split runs as two passes through a temporary copy
    # of keys and values (8 bytes per element) besides the passes' workspace
    n = 1 << 20
    assert lib.edpp_split_workspace_size(n, 2048, 2) >= 8 * n
    assert lib.edpp_split_workspace_size(n, 4096, 2) >= 8 * n
    assert lib.edpp_split_workspace_size(n, 8192, 2) >= 8 * n
    assert lib.edpp_split_workspace_size(n, 1024, 2) < 8 * n
    # the tiled gather/scatter: one array of 8-byte pairs and one of 6-byte
    # (16-bit window offset + 32-bit value) pairs per element
    assert lib.edpp_gather_tiled_workspace_size(n) >= 14 * n
    assert lib.edpp_scatter_tiled_workspace_size(n) >= 14 * n


def test_argument_errors_before_any_device_work(edpp):
    lib = edpp.lib()
    nul = ctypes.c_void_p(0)
    fake = ctypes.c_void_p(16)  # never dereferenced: validation fails first
    # split: buckets not a power of two; SOA without values (splitImpl.cpp:29-34)
    assert lib.edpp_split_i32(fake, fake, nul, 100, 3, 0, nul, nul, fake, 1 << 20, nul) == 1
    assert lib.edpp_split_i32(fake, fake, nul, 100, 4, 2, nul, nul, fake, 1 << 20, nul) == 1
    assert lib.edpp_split_i32(fake, fake, nul, 100, 4, 7, nul, nul, fake, 1 << 20, nul) == 1
    # workspace too small
    assert lib.edpp_split_i32(fake, fake, nul, 100, 4, 0, nul, nul, fake, 8, nul) == 2
    assert lib.edpp_scan_exclusive_i32(fake, fake, 1000, 0, fake, 8, nul) == 2
    # bad scan algorithm / negative length / gather pass < 1
    assert lib.edpp_scan_exclusive_i32(fake, fake, 1000, 9, fake, 1 << 20, nul) == 1
    assert lib.edpp_scan_exclusive_i32(fake, fake, -1, 0, fake, 1 << 20, nul) == 1
    assert lib.edpp_gather_i32(fake, fake, 100, fake, 0, nul) == 1
    assert lib.edpp_scatter_i32(fake, fake, -5, fake, 1, nul) == 1
    # zero-length calls succeed without work
    assert lib.edpp_gather_i32(nul, nul, 0, nul, 1, nul) == 0
    assert lib.edpp_scan_inclusive_f32(nul, nul, 0, 0, nul, 0, nul) == 0
    assert lib.edpp_split_i32(nul, nul, nul, 0, 16, 0, nul, nul, nul, 0, nul) == 0
    assert lib.edpp_stream_copy_f32(nul, nul, 0, nul) == 0
