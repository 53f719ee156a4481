"""Build libgfpdb.so in-tree: CUDA kernels for sm_103a plus the C++ host layer.

Every translation unit is compiled in parallel into ``_build/`` and linked
into ``flexpushdowndb_gb300/libgfpdb.so``. Objects are rebuilt only when a
source or header is newer than the object, so a second build is quick.
"""

from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
OUT_DIR = PKG / "_build"
LIB = PKG / "libgfpdb.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3",
    "-lineinfo",
    "-std=c++17",
    "--expt-relaxed-constexpr",
    "-Xcompiler",
    "-fPIC",
    "-Xcompiler",
    "-Wall",
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgfpdb.so")


def _cuda_include(nvcc: str) -> str:
    return str(Path(nvcc).resolve().parent.parent / "include")


def sources() -> list[Path]:
    return sorted(CSRC.rglob("*.cu")) + sorted(CSRC.rglob("*.cpp"))


def _headers() -> list[Path]:
    return (
        sorted(CSRC.rglob("*.h"))
        + sorted(CSRC.rglob("*.cuh"))
        + sorted(INCLUDE.glob("*.h"))
    )


def _obj_for(src: Path) -> Path:
    rel = src.relative_to(CSRC)
    return OUT_DIR / (str(rel).replace(os.sep, "__") + ".o")


def _compile(src: Path, nvcc: str, newest_header: float, extra: list[str]) -> Path:
    obj = _obj_for(src)
    if obj.exists() and obj.stat().st_mtime >= max(src.stat().st_mtime, newest_header):
        return obj
    if src.suffix == ".cu":
        cmd = [nvcc, *NVCC_FLAGS, *extra, "-c", str(src), "-o", str(obj)]
    else:
        cxx = os.environ.get("CXX", "g++")
        cmd = [cxx, *CXX_FLAGS, f"-I{_cuda_include(nvcc)}", "-c", str(src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def build(verbose: bool = False, extra_nvcc: list[str] | None = None) -> Path:
    nvcc = _nvcc()
    OUT_DIR.mkdir(exist_ok=True)
    newest_header = max(h.stat().st_mtime for h in _headers())
    srcs = sources()
    extra = list(extra_nvcc or [])
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc, newest_header, extra), srcs))
    if not LIB.exists() or LIB.stat().st_mtime < max(o.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        cmd = [nvcc, *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True, extra_nvcc=sys.argv[1:])
