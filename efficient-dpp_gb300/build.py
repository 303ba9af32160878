"""Build libedpp.so (CUDA kernels + C ABI + C++ host mirror) for sm_103a.

Every .cu under csrc/ and every .cpp under csrc/host/ is compiled to an
object in parallel, then linked into lib/libedpp.so with the CUDA runtime
linked statically, so the library loads on a machine without a GPU.  A
translation unit is rebuilt only when it, a header of the package, or
include/*.h is newer than its object.

Usage:  python efficient-dpp_gb300/build.py [-v] [--force]
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OBJ = PKG / "_build"
LIB = PKG / "lib" / "libedpp.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-Wall", f"-I{INCLUDE}", f"-I{CSRC}"]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-pthread", f"-I{INCLUDE}", f"-I{CSRC}"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libedpp")
    return cand


def _cuda_include() -> Path:
    return Path(_nvcc()).resolve().parent.parent / "include"


def _headers() -> list[Path]:
    return list(CSRC.rglob("*.cuh")) + list(CSRC.rglob("*.h")) + list(CSRC.rglob("*.hpp")) + \
        list(INCLUDE.glob("*.h")) + list(INCLUDE.glob("*.hpp"))


def _stale(src: Path, obj: Path, newest_header: float) -> bool:
    if not obj.exists():
        return True
    m = obj.stat().st_mtime
    return src.stat().st_mtime > m or newest_header > m


def build(verbose: bool = False, force: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    newest_header = max((h.stat().st_mtime for h in _headers()), default=0.0)
    jobs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJ / (src.stem + ".cu.o")
        cmd = [nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)]
        jobs.append((src, obj, cmd))
    for src in sorted((CSRC / "host").glob("*.cpp")):
        obj = OBJ / (src.stem + ".cpp.o")
        cmd = ["g++", *CXX_FLAGS, f"-I{_cuda_include()}", "-c", str(src), "-o", str(obj)]
        jobs.append((src, obj, cmd))

    todo = [j for j in jobs if force or _stale(j[0], j[1], newest_header)]

    def run(job):
        src, obj, cmd = job
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {src.name}\n{r.stdout}\n{r.stderr}")
        return src

    if todo:
        workers = min(len(todo), max(2, os.cpu_count() or 2))
        with cf.ThreadPoolExecutor(max_workers=workers) as ex:
            for f in [ex.submit(run, j) for j in todo]:
                f.result()
    objs = [str(j[1]) for j in jobs]
    if force or todo or not LIB.exists():
        cmd = [nvcc, *ARCH, "-shared", "-o", str(LIB), *objs, "-cudart", "static",
               "-Xcompiler", "-pthread"]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    return LIB


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__)
    ap.add_argument("-v", "--verbose", action="store_true")
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args(argv)
    print(build(verbose=a.verbose, force=a.force))
    return 0


if __name__ == "__main__":
    sys.exit(main())
