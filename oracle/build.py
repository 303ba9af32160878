"""Build the oracle (test infrastructure only).

  oracle/_build/liboracle.so   the C restatement (edpp_oracle.c), gcc -fopenmp
  oracle/_build/libref_cuda.so runner for the reference's CUDA kernels
                               (ref_cuda_runner.cu), built where nvcc and the
                               cubins below exist
  oracle/_ref/libref_omp.so    the reference's own OpenMP functions, compiled
                               from where they lie under the reference tree
                               with main() renamed, plus ref_shim.cpp
  oracle/_ref/libref_cl_split_{ko,soa,aos}.so
                               the reference's OpenCL split kernels
                               (opencl/kernels/split_kernel.cl, included
                               unchanged) compiled as C through ref_cl_shim.h,
                               with ref_cl_runner.c replaying WI_split
  oracle/_ref/*.cubin          the reference's CUDA device code
                               (cuda/test_{split,gather,scatter,bandwidth}.cu)
                               compiled for sm_103a

The oracle/_ref outputs are built only when the reference tree is present:
EDPP_REFERENCE, or else a directory named `reference` beside this
repository's root.  Nothing here is part of the product.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("EDPP_REFERENCE", str(HERE.parent.parent / "reference")))

REF_CUDA_SOURCES = ["test_split", "test_gather", "test_scatter", "test_bandwidth"]


def _run(cmd, cwd=None):
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=cwd)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(map(str, cmd))}\n{r.stdout}\n{r.stderr}")


def _newer(out: Path, *srcs: Path) -> bool:
    return not out.exists() or any(s.stat().st_mtime > out.stat().st_mtime for s in srcs)


def build_oracle() -> Path:
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "liboracle.so"
    src = HERE / "edpp_oracle.c"
    if _newer(out, src, HERE / "edpp_oracle.h"):
        _run(["gcc", "-O2", "-std=c11", "-fopenmp", "-fwrapv", "-fPIC", "-shared", "-Wall",
              str(src), "-o", str(out), "-lm"])
    return out


def _nvcc():
    return shutil.which("nvcc") or ("/usr/local/cuda/bin/nvcc"
                                     if Path("/usr/local/cuda/bin/nvcc").exists() else None)


def build_ref_omp() -> Path | None:
    """The reference's OpenMP CPU functions (x86 only: they use AVX2)."""
    omp = REFERENCE / "openmp"
    if not omp.is_dir() or platform.machine() not in ("x86_64", "AMD64"):
        return None
    REF_OUT.mkdir(exist_ok=True)
    out = REF_OUT / "libref_omp.so"
    units = {
        "gs": omp / "test_gather_scatter_CPU.cpp",
        "scan": omp / "test_scan_CPU.cpp",
        "bw": omp / "test_bandwidth_CPU.cpp",
        "util": omp / "util" / "utility.cpp",
        "log": omp / "util" / "log.cpp",
    }
    shim = HERE / "ref_shim.cpp"
    if not _newer(out, shim, *units.values()):
        return out
    flags = ["-O3", "-std=c++11", "-w", "-mavx2", "-fopenmp", "-fwrapv", "-fPIC",
             "-include", "cstdint", f"-I{omp}", f"-I{omp / 'util'}", f"-I{HERE / 'tbb_stub'}"]
    objs = []

    def cc(name, src):
        obj = REF_OUT / f"{name}.o"
        _run(["g++", *flags, f"-Dmain=edpp_ref_main_{name}", "-c", str(src), "-o", str(obj)])
        return obj

    with cf.ThreadPoolExecutor(max_workers=6) as ex:
        futs = [ex.submit(cc, k, v) for k, v in units.items()]
        futs.append(ex.submit(cc, "shim", shim))
        objs = [f.result() for f in futs]
    _run(["g++", "-shared", "-fopenmp", "-o", str(out), *map(str, objs)])
    for o in objs:
        o.unlink()
    return out


CL_LAYOUTS = {"ko": "KO", "soa": "KVS_SOA", "aos": "KVS_AOS"}


def build_ref_cl_split() -> list[Path]:
    """The reference's OpenCL split kernels, compiled as C for the CPU: one
    library per data layout (the -D flag the reference's host code gives its
    kernel compiler, opencl/primitives/splitImpl.cpp:61-64).  Plain C with
    pthreads, so it builds on any host where the reference tree exists."""
    cl = REFERENCE / "opencl" / "kernels" / "split_kernel.cl"
    if not cl.is_file():
        return []
    REF_OUT.mkdir(exist_ok=True)
    shim, runner = HERE / "ref_cl_shim.h", HERE / "ref_cl_runner.c"
    outs = []
    for name, flag in CL_LAYOUTS.items():
        out = REF_OUT / f"libref_cl_split_{name}.so"
        if _newer(out, shim, runner, cl, REFERENCE / "opencl" / "params.h"):
            _run(["gcc", "-O2", "-std=gnu11", "-w", "-pthread", "-fPIC", "-shared", f"-D{flag}",
                  f'-DREF_SPLIT_CL="{cl}"', "-include", str(shim), str(runner), "-o", str(out)])
        outs.append(out)
    return outs


def build_ref_cubins() -> list[Path]:
    """The reference's CUDA device code for sm_103a (GPU code: it travels to
    the GPU machine with the repository snapshot)."""
    cu = REFERENCE / "cuda"
    nvcc = _nvcc()
    if not cu.is_dir() or nvcc is None:
        return []
    REF_OUT.mkdir(exist_ok=True)
    outs = []

    def one(name):
        src = cu / f"{name}.cu"
        out = REF_OUT / f"{name}.cubin"
        if _newer(out, src):
            _run([nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
                  "-include", "cstdint", f"-I{cu}", f"-I{cu / 'util'}", str(src), "-o", str(out)])
        return out

    with cf.ThreadPoolExecutor(max_workers=4) as ex:
        outs = list(ex.map(one, REF_CUDA_SOURCES))
    return outs


def build_ref_cuda_runner() -> Path | None:
    """Runner that launches the reference's cubin kernels (and the CUB scan
    the reference calls) on seeded host arrays.  Needs nvcc and the cubins."""
    nvcc = _nvcc()
    if nvcc is None or not all((REF_OUT / f"{n}.cubin").exists() for n in REF_CUDA_SOURCES):
        return None
    BUILD.mkdir(exist_ok=True)
    out = BUILD / "libref_cuda.so"
    src = HERE / "ref_cuda_runner.cu"
    if _newer(out, src):
        _run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O2", "-std=c++17",
              "-Xcompiler", "-fPIC", "-shared", str(src), "-o", str(out), "-lcuda"])
    return out


def build_all(verbose: bool = False) -> dict:
    res = {"oracle": build_oracle()}
    try:
        res["ref_omp"] = build_ref_omp()
    except RuntimeError as e:  # the reference failing to build is reported, not fatal
        res["ref_omp"] = None
        if verbose:
            print(e, file=sys.stderr)
    try:
        res["ref_cl_split"] = build_ref_cl_split()
    except RuntimeError as e:
        res["ref_cl_split"] = []
        if verbose:
            print(e, file=sys.stderr)
    try:
        res["ref_cubins"] = build_ref_cubins()
    except RuntimeError as e:
        res["ref_cubins"] = []
        if verbose:
            print(e, file=sys.stderr)
    try:
        res["ref_cuda_runner"] = build_ref_cuda_runner()
    except RuntimeError as e:
        res["ref_cuda_runner"] = None
        if verbose:
            print(e, file=sys.stderr)
    return res


if __name__ == "__main__":
    for k, v in build_all(verbose=True).items():
        print(f"{k}: {v}")
