"""Builds the CUDA library (librulinalg_gb300.so, sm_103a only) and the oracle.

The library is compiled in-tree, one nvcc process per translation unit in parallel,
then linked with nvcc into a shared object with the CUDA runtime linked statically.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = PKG / "librulinalg_gb300.so"
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
    "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
    "-I", str(ROOT / "include"),
]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build rulinalg_gb300")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu"))


def build_library(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    OUT_DIR.mkdir(exist_ok=True)
    srcs = sources()
    deps = list(CSRC.glob("*.cuh")) + [ROOT / "include" / "rulinalg_gb300.h"]
    newest_dep = max(p.stat().st_mtime for p in deps)
    objs, jobs = [], []
    for src in srcs:
        obj = OUT_DIR / (src.stem + ".o")
        objs.append(obj)
        if force or not obj.exists() or obj.stat().st_mtime < max(src.stat().st_mtime, newest_dep):
            jobs.append([nvcc, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 1)) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or not LIB.exists():
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs)])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


def build_oracle() -> Path:
    """The oracle is test infrastructure (a CPU restatement of the reference)."""
    oracle_dir = ROOT / "oracle"
    _run(["make", "-s", "-C", str(oracle_dir)])
    return oracle_dir / "liboracle.so"


if __name__ == "__main__":
    build_library(force="--force" in sys.argv, verbose=True)
    build_oracle()
