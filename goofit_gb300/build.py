"""Builds libgfengine.so in-tree (goofit_gb300/lib/) for sm_103a.

The CUDA translation units go through nvcc with
``-gencode arch=compute_103a,code=sm_103a``; host-only C++ (tree analysis,
code generator, NVRTC wrapper, minimiser) through g++.  Kernels generated per
PDF tree are compiled at run time by NVRTC for the same architecture.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
CSRC = HERE / "csrc"
LIBDIR = HERE / "lib"
BUILDDIR = HERE / "_build"
ROOT = HERE.parent
INCLUDE = ROOT / "include"

CUDA_HOME = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
NVCC = str(CUDA_HOME / "bin" / "nvcc")
GENCODE = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["engine.cu", "noalloc.cu", "gram_tc.cu"]
CXX17_SOURCES = ["tree.cpp", "codegen.cpp", "rtc.cpp"]
CXX20_SOURCES = ["migrad.cpp", "fit.cpp"]

LIB_NAME = "libgfengine.so"


def lib_path() -> Path:
    return LIBDIR / LIB_NAME


def _headers() -> list[Path]:
    return list(CSRC.glob("*.h")) + list(INCLUDE.glob("*.h"))


def _stale(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(s.stat().st_mtime > t for s in sources)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _compile(src: str) -> Path:
    s = CSRC / src
    obj = BUILDDIR / (src + ".o")
    deps = [s] + _headers()
    if not _stale(obj, deps):
        return obj
    inc = [f"-I{INCLUDE}", f"-I{CSRC}", f"-I{CUDA_HOME / 'include'}"]
    if src.endswith(".cu"):
        cmd = [NVCC, *GENCODE, "-lineinfo", "-O3", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-c", str(s),
               "-o", str(obj), *inc]
    else:
        std = "-std=c++20" if src in CXX20_SOURCES else "-std=c++17"
        # no floating-point contraction: host arithmetic (analytic norms, bin centres, the kinematic boundary)
        # rounds like the FP64 restatement it is checked against, on x86-64 and on aarch64 alike
        cmd = ["g++", std, "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-variable", "-c", str(s), "-o",
               str(obj), *inc]
    _run(cmd)
    return obj


def build(verbose: bool = False) -> Path:
    """Compiles and links libgfengine.so if any source changed; returns its path."""
    BUILDDIR.mkdir(exist_ok=True)
    LIBDIR.mkdir(exist_ok=True)
    if shutil.which(NVCC) is None and not Path(NVCC).exists():
        raise RuntimeError(f"nvcc not found at {NVCC}")
    srcs = CU_SOURCES + CXX17_SOURCES + CXX20_SOURCES
    with ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    target = lib_path()
    if _stale(target, objs):
        tmp = target.with_suffix(".so.tmp")
        cmd = [NVCC, *GENCODE, "-shared", "-o", str(tmp), *map(str, objs),
               f"-L{CUDA_HOME / 'lib64'}", "-lnvrtc", "-Xlinker", f"-rpath={CUDA_HOME / 'lib64'}"]
        _run(cmd)
        os.replace(tmp, target)
        if verbose:
            print(f"built {target}")
    return target


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
