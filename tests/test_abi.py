"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/torchfem_gb300.h (no GPU needed)."""

import ctypes
import re
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def declared_functions():
    text = (ROOT / "include" / "torchfem_gb300.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(fem_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol():
    from torchfem_gb300 import _build, _lib

    path = _build.build()
    lib = ctypes.CDLL(str(path))
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    # the binding declares exactly the header's entry points
    assert sorted(_lib.symbols()) == names


def test_abi_version_and_error_string():
    from torchfem_gb300 import _lib

    lib = _lib.load()
    assert lib.fem_abi_version() == 1
    assert isinstance(lib.fem_last_error(), bytes)


def test_workspace_queries_need_no_gpu():
    from torchfem_gb300 import _lib

    lib = _lib.load()
    assert lib.fem_pattern_workspace_bytes(1331, 1000, 8) > 1000 * 64 * 8
    m = _lib.FemMatrix(_lib.FEM_FMT_CSR_F64, 1, 3993, 3993, None, None, None, None)
    assert lib.fem_pcg_workspace_bytes(ctypes.byref(m)) >= 4 * 3993 * 8
    bad = _lib.FemMatrix(99, 1, 10, 10, None, None, None, None)
    assert lib.fem_pcg_workspace_bytes(ctypes.byref(bad)) == 0
