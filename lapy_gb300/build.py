"""Build recipe for the lapy_gb300 CUDA library (sm_103a only).

Compiles every translation unit under ``lapy_gb300/csrc`` with nvcc in
parallel and links ``lapy_gb300/_lib/liblapy_gb300.so`` in-tree.  The library
exports the C ABI declared in ``include/lapy_gb300.h``; Python binds it with
ctypes (``lapy_gb300/_lib.py``).

Run as ``python -m lapy_gb300.build`` or through ``__graft_entry__.build()``.
``LAPY_NVCC_FLAGS`` adds flags to every compile (tuning experiments); objects
are rebuilt when sources change, so clear ``_build/`` after changing it.
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
INCLUDE = ROOT / "include"
OUT_DIR = PKG / "_lib"
BUILD_DIR = ROOT / "_build"
LIB_NAME = "liblapy_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
          f"-I{INCLUDE}", f"-I{CSRC}", "--expt-relaxed-constexpr"]
# Per-file extra flags.  Assembly must not contract a*b+c into an FMA so that
# element values round exactly like NumPy's separate multiply and add.
EXTRA = {
    "assemble.cu": ["--fmad=false"],
    "geodesic.cu": ["--fmad=false"],
    "ic0.cu": ["--fmad=false"],
    "curvature.cu": ["--fmad=false"],
}


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the lapy_gb300 CUDA library cannot be built")
    return cand


def sources() -> list[Path]:
    return sorted([*CSRC.glob("*.cu"), *CSRC.glob("*.cpp")])


def _compile(src: Path, nvcc: str) -> Path:
    obj = BUILD_DIR / (src.name + ".o")
    deps = [src, *CSRC.glob("*.cuh"), *INCLUDE.glob("*.h")]
    if obj.exists() and obj.stat().st_mtime >= max(d.stat().st_mtime for d in deps):
        return obj
    extra_env = os.environ.get("LAPY_NVCC_FLAGS", "").split()
    cmd = [nvcc, *ARCH, *COMMON, *EXTRA.get(src.name, []), *extra_env, "-c", str(src), "-o", str(obj)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src.name}:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    return obj


def build_library(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile and link the shared library; return its path."""
    nvcc = _nvcc()
    BUILD_DIR.mkdir(exist_ok=True)
    OUT_DIR.mkdir(exist_ok=True)
    srcs = sources()
    jobs = jobs or min(len(srcs), max(1, os.cpu_count() or 1))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, nvcc), srcs))
    lib = OUT_DIR / LIB_NAME
    if lib.exists() and lib.stat().st_mtime >= max(o.stat().st_mtime for o in objs):
        return lib
    tmp = OUT_DIR / (LIB_NAME + ".tmp")
    cmd = [nvcc, *ARCH, "-shared", "-cudart", "shared", "-o", str(tmp), *map(str, objs)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")
    os.replace(tmp, lib)
    if verbose:
        print(f"built {lib}")
    return lib


if __name__ == "__main__":
    build_library(verbose=True)
    sys.exit(0)
