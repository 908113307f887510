"""Build recipe of libtk_heff.so (CUDA kernels + C ABI) for sm_103a.

Each translation unit is compiled in parallel into ``_build/`` beside the
package and linked into ``tk_gb300/libtk_heff.so``.  No cmake, one
``-gencode``; a rebuild is skipped when no source is newer than the library.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
ROOT = PKG_DIR.parent
CSRC = ROOT / "csrc"
BUILD_DIR = ROOT / "_build"
INCLUDE = ROOT.parent / "include"
LIB_PATH = PKG_DIR / "libtk_heff.so"

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "--expt-relaxed-constexpr", "-I", str(CSRC), "-I", str(INCLUDE)]
HOST_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-Wall", "-I", str(CSRC), "-I", str(INCLUDE),
              "-I", "/usr/local/cuda/include"]


def sources() -> list[Path]:
    return sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))


def _stale() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps if p.is_file())


def _compile(src: Path) -> Path:
    obj = BUILD_DIR / (src.name + ".o")
    if src.suffix == ".cu":
        cmd = [NVCC, *ARCH, *CUDA_FLAGS, "-c", str(src), "-o", str(obj)]
    else:
        cmd = ["g++", *HOST_FLAGS, "-c", str(src), "-o", str(obj)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles every CUDA/C++ source and links libtk_heff.so; returns its path."""
    if not force and not _stale():
        return LIB_PATH
    BUILD_DIR.mkdir(parents=True, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(_compile, srcs))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cuda_lib = str(Path(NVCC).resolve().parent.parent / "lib64")
    cmd = [NVCC, *ARCH, "-shared", "-o", str(tmp), *map(str, objs), "-L", cuda_lib, "-lcusolver",
           "-Xlinker", "-rpath=" + cuda_lib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    if verbose:
        print(f"built {LIB_PATH}", file=sys.stderr)
    return LIB_PATH


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
