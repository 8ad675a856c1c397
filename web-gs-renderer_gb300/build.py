"""Build recipe of libwebgs.so (the CUDA kernels + C ABI) and of the CPU oracle library.

Every CUDA translation unit is compiled for sm_103a only, in parallel, with -fmad=false so that
the kernels keep the pinned fp32 semantics (fused multiply-adds only where written explicitly);
the gradient and loss units, whose results are not pinned, contract freely.
Host C++ is built with -ffp-contract=off for the same reason. Outputs stay in the tree:
  web-gs-renderer_gb300/lib/libwebgs.so
  oracle/liboracle.so            (test infrastructure; built beside the product, never linked into it)
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "libwebgs.so"
# the checked build (-DGS_CHECKED): canary-padded buffers and bounds-checked stores, a test-only library
BUILD_CHECKED = PKG / "_build_checked"
LIB_CHECKED = PKG / "lib" / "libwebgs_checked.so"
ORACLE_SRC = ROOT / "oracle" / "gs_oracle.cpp"
ORACLE_INPUTS = ROOT / "oracle" / "gs_inputs.cpp"
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off", "-Xptxas", "-warn-spills",
]
CXX_FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-Wall", "-Wno-unused-function"]
# Translation units whose results are not bit-pinned (gradients, the loss) may contract a*b+c into
# fused multiply-adds and use the approximate division and square root (denormals are kept).
CONTRACTED = {"gs_preprocess_backward.cu", "gs_loss.cu"}


def _nvcc_flags(src: Path) -> list[str]:
    if src.name in CONTRACTED:
        return [{"-fmad=false": "-fmad=true", "-prec-div=true": "-prec-div=false", "-prec-sqrt=true": "-prec-sqrt=false"}.get(f, f) for f in NVCC_FLAGS]
    return NVCC_FLAGS


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    proc = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}")
    if proc.stdout.strip() and os.environ.get("WEBGS_BUILD_VERBOSE"):
        sys.stderr.write(proc.stdout)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False, checked: bool = False) -> Path:
    """Compiles libwebgs.so for sm_103a (nvcc cross-compiles without a GPU); with checked=True the
    checked build libwebgs_checked.so instead."""
    build_dir, lib = (BUILD_CHECKED, LIB_CHECKED) if checked else (BUILD, LIB)
    extra = ["-DGS_CHECKED"] if checked else []
    build_dir.mkdir(exist_ok=True)
    lib.parent.mkdir(exist_ok=True)
    nvcc = _nvcc()
    headers = sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + [ROOT / "include" / "gs.h"]
    jobs, objs = [], []
    for src in sorted(CSRC.glob("*.cu")):
        obj = build_dir / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers + [Path(__file__)]):
            jobs.append([nvcc, *_nvcc_flags(src), *extra, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = build_dir / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src] + headers + [Path(__file__)]):
            jobs.append(["g++", *CXX_FLAGS, *extra, "-I", str(ROOT / "include"), "-c", str(src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _stale(lib, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(lib), *map(str, objs), "-Xcompiler", "-fopenmp", "-lgomp"])
    return lib


def build_oracle(force: bool = False) -> Path:
    """Compiles the CPU restatement used by the tests and the CPU baseline."""
    hdr = ORACLE_SRC.with_suffix(".h")
    if force or _stale(ORACLE_LIB, [ORACLE_SRC, ORACLE_INPUTS, hdr, Path(__file__)]):
        _run(["g++", "-O3", "-shared", "-fPIC", "-std=c++17", "-ffp-contract=off", "-fopenmp", "-Wall",
              str(ORACLE_SRC), str(ORACLE_INPUTS), "-o", str(ORACLE_LIB)])
    return ORACLE_LIB


def build_all(force: bool = False, checked: bool = False) -> None:
    """The product library and the oracle; with checked=True also the checked build."""
    with ThreadPoolExecutor(max_workers=3) as ex:
        jobs = [ex.submit(build_library, force), ex.submit(build_oracle, force)]
        if checked:
            jobs.append(ex.submit(build_library, force, True))
        for j in jobs:
            j.result()


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print(LIB)
