"""The C++ mirror of the reference's primitive API (include/edpp_primitives.hpp),
exercised by tests/cpp/test_primitives.cpp: the reference's test drivers ported
onto it, with the reference's own checks.  Compiled here (CPU) and run on the
GPU."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
SRC = ROOT / "tests" / "cpp" / "test_primitives.cpp"
LIBDIR = ROOT / "efficient-dpp_gb300" / "lib"


def _compile(out: Path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    cmd = [nvcc, "-std=c++17", "-O2", str(SRC), f"-I{ROOT / 'include'}", f"-L{LIBDIR}", "-ledpp",
           f"-Xlinker", f"-rpath={LIBDIR}", "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_mirror_driver_compiles(edpp, tmp_path):
    _compile(tmp_path / "test_primitives")


@pytest.mark.gpu
def test_mirror_driver_passes_on_gpu(cuda, tmp_path):
    exe = tmp_path / "test_primitives"
    _compile(exe)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and "PASSED" in r.stdout, r.stdout + r.stderr
