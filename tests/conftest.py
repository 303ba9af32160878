"""Test configuration.

Markers:
  gpu   needs a CUDA device (GB300); deselected with -m "not gpu".

The session builds libedpp.so and the oracle if they are missing or stale
(a few seconds with nvcc/gcc), so a fresh checkout tests as-is.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "efficient-dpp_gb300"
for p in (str(ROOT), str(PKG)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300)")


_built = False


def _build_once():
    global _built
    if _built:
        return
    import importlib.util
    spec = importlib.util.spec_from_file_location("edpp_pkg_build", PKG / "build.py")
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    m.build()
    from oracle import oracle as orc
    orc.build()
    _built = True


@pytest.fixture(scope="session")
def edpp():
    _build_once()
    import edpp as e
    e.lib()
    return e


@pytest.fixture(scope="session")
def orc():
    _build_once()
    from oracle import oracle as o
    o.lib()
    return o


@pytest.fixture(scope="session")
def cuda(edpp):
    import torch
    if not torch.cuda.is_available():
        pytest.fail("a gpu-marked test ran without a CUDA device")
    torch.cuda.init()
    return torch


def to_dev(a: np.ndarray):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


def to_host(t) -> np.ndarray:
    return t.cpu().numpy()
