"""Builds the CUDA shared library ``libtorchfem_gb300.so`` for sm_103a.

Plain ``nvcc`` on the translation units in ``csrc/`` (compiled in
parallel), then one link step.  No torch headers are involved: the library is
a C ABI (``include/torchfem_gb300.h``) that Python reaches through ctypes.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG_DIR = Path(__file__).resolve().parent
CSRC = PKG_DIR.parent / "csrc"
INCLUDE = PKG_DIR.parent.parent / "include"
LIB_PATH = PKG_DIR / "libtorchfem_gb300.so"
SOURCES = ("fem_pattern.cu", "fem_element.cu", "fem_solver.cu", "fem_nonlinear.cu", "fem_shell.cu",
           "fem_amg.cu", "fem_heat.cu", "fem_modal.cu", "fem_coupling.cu")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc() -> str:
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cand = Path(cuda_home) / "bin" / "nvcc"
    if cand.exists():
        return str(cand)
    found = shutil.which("nvcc")
    if found is None:
        raise RuntimeError("nvcc not found: set CUDA_HOME")
    return found


def _stale() -> bool:
    if not LIB_PATH.exists():
        return True
    t = LIB_PATH.stat().st_mtime
    deps = [CSRC / s for s in SOURCES] + list(CSRC.glob("*.cuh")) + list(INCLUDE.glob("*.h"))
    return any(d.stat().st_mtime > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> Path:
    """Compiles the library in-tree if it is missing or older than its sources."""
    if not force and not _stale():
        return LIB_PATH
    nvcc = _nvcc()
    obj_dir = PKG_DIR / "_build"
    obj_dir.mkdir(exist_ok=True)

    def compile_one(src: str) -> Path:
        obj = obj_dir / (Path(src).stem + ".o")
        extra = os.environ.get("TORCHFEM_GB300_NVCC_FLAGS", "").split()
        cmd = [nvcc, *FLAGS, *ARCH, *extra, "-I", str(INCLUDE), "-c", str(CSRC / src), "-o", str(obj)]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{res.stderr}")
        if verbose and res.stderr:
            print(res.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=len(SOURCES)) as pool:
        objs = list(pool.map(compile_one, SOURCES))
    tmp = LIB_PATH.with_suffix(".so.tmp")
    cmd = [nvcc, "-shared", *ARCH, "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{res.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    print(build(force=True, verbose=True))
