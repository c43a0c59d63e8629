"""ctypes binding of the C ABI in ``include/torchfem_gb300.h``.

The library is the only compute path: there is no CPU fallback.  Loading it
fails loudly if it is missing; calling into it needs a CUDA device.
"""

from __future__ import annotations

import ctypes as C
from pathlib import Path

import torch

from ._build import LIB_PATH

FEM_OK = 0
FEM_NOT_CONVERGED = 1
FEM_NONFINITE = 2
FEM_BAD_JACOBIAN = 3
FEM_BOUNDS = 4
FEM_INVALID = 5
FEM_CUDA_ERROR = 6
FEM_BREAKDOWN = 7

FEM_QUAD1, FEM_HEXA1, FEM_TETRA2, FEM_TETRA1, FEM_TRIA1, FEM_QUAD2, FEM_TRIA2, FEM_SHELL3, FEM_HEXA2 = range(1, 10)
FEM_MAT_ISO, FEM_MAT_GENERAL, FEM_MAT_TANGENT_IP = 1, 2, 3
# conductivity tensor [n_elem][dim][dim] of the heat kernels (fem_heat_*)
FEM_MAT_CONDUCTIVITY = 16
FEM_F64, FEM_F32 = 0, 1
FEM_FMT_CSR_F64, FEM_FMT_SELL_F32 = 1, 2

vp = C.c_void_p
i64 = C.c_int64


class FemMesh(C.Structure):
    _fields_ = [
        ("etype", C.c_int),
        ("n_nod", i64),
        ("n_elem", i64),
        ("nodes", vp),
        ("elements", vp),
        ("weights", vp),
        ("bt", vp),
        ("detj", vp),
        ("inc_ptr", vp),
        ("inc", vp),
        ("thickness", vp),
        ("dof_per_node", C.c_int),
    ]


class FemMaterial(C.Structure):
    _fields_ = [("kind", C.c_int), ("data", vp)]


class FemBlocks(C.Structure):
    _fields_ = [
        ("n_e", C.c_int),
        ("dim", C.c_int),
        ("n_nod", i64),
        ("n_blocks", i64),
        ("nbr_ptr", vp),
        ("nbr", vp),
        ("blk_ptr", vp),
        ("contrib", vp),
        ("blk_row", vp),
        ("diag_blk", vp),
        ("inc_ptr", vp),
    ]


class FemMatrix(C.Structure):
    _fields_ = [
        ("format", C.c_int),
        ("block", C.c_int),
        ("n", i64),
        ("n_rows", i64),
        ("row_ptr", vp),
        ("col", vp),
        ("val", vp),
        ("precond", vp),
    ]


class FemSolveInfo(C.Structure):
    _fields_ = [
        ("iterations", i64),
        ("replacements", i64),
        ("rel_residual", C.c_double),
        ("status", C.c_int32),
        ("spmv_ms", C.c_double),
        ("spmv_timed", i64),
    ]


class FemShell(C.Structure):
    _fields_ = [
        ("n_nod", i64),
        ("n_elem", i64),
        ("nodes", vp),
        ("elements", vp),
        ("orientation", vp),
        ("thickness", vp),
        ("n_z", C.c_int),
        ("z", vp),
        ("w", vp),
        ("kappa", C.c_double),
        ("nu_t", C.c_double),
        ("drill", C.c_double),
    ]


class FemOperator64(C.Structure):
    _fields_ = [
        ("mesh", C.POINTER(FemMesh)),
        ("mat", C.POINTER(FemMaterial)),
        ("con_mask", vp),
        ("sell_val64", vp),
    ]


class FemAmgLevel(C.Structure):
    _fields_ = [
        ("n", i64),
        ("block", C.c_int),
        ("a_nnz", i64),
        ("a_ptr", vp),
        ("a_col", vp),
        ("a_val", vp),
        ("n_agg", i64),
        ("agg", vp),
        ("tval", vp),
        ("p_nnz", i64),
        ("p_ptr", vp),
        ("p_col", vp),
        ("p_val", vp),
        ("rho", C.c_double),
        ("coarse_inv", vp),
        ("dropped", i64),
    ]


_P = C.POINTER
_SIGNATURES = {
    "fem_amg_create": (C.c_int, [_P(FemBlocks), vp, vp, _P(vp), vp]),
    "fem_amg_setup": (C.c_int, [vp, _P(FemMatrix), vp]),
    "fem_amg_pcg_workspace_bytes": (C.c_size_t, [vp, _P(FemOperator64)]),
    "fem_amg_pcg": (
        C.c_int,
        [vp, _P(FemMatrix), _P(FemOperator64), vp, vp, C.c_double, C.c_double, i64, vp, C.c_size_t,
         _P(FemSolveInfo), vp],
    ),
    "fem_amg_destroy": (None, [vp]),
    "fem_amg_levels": (C.c_int, [vp]),
    "fem_amg_level_info": (C.c_int, [vp, C.c_int, _P(FemAmgLevel)]),
    "fem_copy_device": (C.c_int, [vp, vp, C.c_size_t, vp]),
    "fem_diag_workspace_bytes": (C.c_size_t, []),
    "fem_diag_barrier_timeout": (C.c_int, [vp, C.c_size_t, C.c_longlong, vp]),
    "fem_minres_workspace_bytes": (C.c_size_t, [_P(FemMatrix)]),
    "fem_minres": (C.c_int, [_P(FemMatrix), vp, vp, C.c_double, i64, vp, C.c_size_t, _P(FemSolveInfo), vp]),
    "fem_shell_stiffness": (C.c_int, [_P(FemShell), vp, vp, vp, vp]),
    "fem_shell_force": (C.c_int, [_P(FemShell), vp, vp, vp, vp, vp, vp]),
    "fem_shell_vjp": (C.c_int, [_P(FemShell), vp, vp, vp, vp, vp, vp, vp, vp]),
    "fem_last_error": (C.c_char_p, []),
    "fem_abi_version": (C.c_int, []),
    "fem_launch_count": (i64, []),
    "fem_pattern_workspace_bytes": (C.c_size_t, [i64, i64, C.c_int]),
    "fem_pattern_graph_count": (
        C.c_int,
        [vp, i64, C.c_int, i64, vp, vp, vp, _P(i64), vp, C.c_size_t, vp, vp],
    ),
    "fem_pattern_graph_fill": (C.c_int, [vp, i64, C.c_int, i64, vp, vp, vp, vp, vp, vp]),
    "fem_pattern_csr_rows": (
        C.c_int,
        [vp, i64, C.c_int, vp, vp, _P(i64), vp, C.c_size_t, vp],
    ),
    "fem_pattern_csr_cols": (C.c_int, [vp, vp, i64, C.c_int, vp, vp, vp, vp, vp]),
    "fem_pattern_kmap": (C.c_int, [vp, i64, C.c_int, C.c_int, vp, vp, vp, vp, vp, vp]),
    "fem_pattern_blocks": (
        C.c_int,
        [vp, i64, C.c_int, i64, vp, vp, vp, vp, i64, vp, vp, vp, vp, vp, C.c_size_t, vp, vp],
    ),
    "fem_geometry": (C.c_int, [_P(FemMesh), vp, vp, vp, vp, vp]),
    "fem_element_stiffness": (C.c_int, [_P(FemMesh), _P(FemMaterial), C.c_int, vp, vp, vp]),
    "fem_element_stiffness_iso64": (C.c_int, [_P(FemMesh), _P(FemMaterial), vp, vp, vp]),
    "fem_element_force": (
        C.c_int,
        [_P(FemMesh), _P(FemMaterial), vp, vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp],
    ),
    "fem_gather_workspace_bytes": (C.c_size_t, [i64]),
    "fem_gather_nodal": (
        C.c_int,
        [_P(FemMesh), vp, vp, vp, C.c_int, vp, vp, vp, vp, C.c_size_t, vp],
    ),
    "fem_element_vjp": (
        C.c_int,
        [_P(FemMesh), _P(FemMaterial), vp, vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp,
         vp, vp],
    ),
    "fem_heat_stiffness": (C.c_int, [_P(FemMesh), vp, C.c_int, vp, vp, vp]),
    "fem_heat_force": (
        C.c_int, [_P(FemMesh), vp, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp]
    ),
    "fem_heat_vjp": (
        C.c_int, [_P(FemMesh), vp, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
    ),
    "fem_heat_mass": (C.c_int, [_P(FemMesh), vp, vp, C.c_int, vp, vp, vp]),
    "fem_heat_mass_vjp": (C.c_int, [_P(FemMesh), vp, vp, vp, vp, vp]),
    "fem_mass_matrices": (C.c_int, [_P(FemMesh), vp, vp, C.c_int, vp, vp]),
    "fem_csr_spmm": (C.c_int, [_P(FemMatrix), C.c_int, vp, vp, vp]),
    "fem_coupled_values": (C.c_int, [i64, vp, vp, vp, vp, vp, vp, vp]),
    "fem_csr_apply": (C.c_int, [i64, vp, vp, vp, vp, vp, vp]),
    "fem_csr_combine": (C.c_int, [i64, C.c_double, vp, C.c_double, vp, vp, vp]),
    "fem_heat_cn_workspace_bytes": (C.c_size_t, [i64]),
    "fem_heat_cn_residual": (
        C.c_int, [_P(FemMatrix), vp, vp, vp, vp, C.c_double, vp, vp, vp, vp, C.c_size_t, vp]
    ),
    "fem_hyper_force": (
        C.c_int, [_P(FemMesh), vp, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp]
    ),
    "fem_hyper_vjp": (
        C.c_int, [_P(FemMesh), vp, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp]
    ),
    "fem_plastic_force": (
        C.c_int,
        [_P(FemMesh), vp, C.c_double, C.c_int, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp,
         vp, vp],
    ),
    "fem_plastic_vjp": (
        C.c_int,
        [_P(FemMesh), vp, C.c_double, C.c_int, vp, vp, vp, C.c_int, vp, vp, vp, vp, vp, vp, vp, vp,
         vp, vp, vp, vp],
    ),
    "fem_assemble_csr": (C.c_int, [_P(FemBlocks), C.c_int, vp, vp, vp, vp, vp]),
    "fem_sell_workspace_bytes": (C.c_size_t, [i64]),
    "fem_sell_layout": (C.c_int, [_P(FemBlocks), vp, _P(i64), vp, C.c_size_t, vp]),
    "fem_sell_columns": (C.c_int, [_P(FemBlocks), vp, vp, vp]),
    "fem_assemble_sell": (C.c_int, [_P(FemBlocks), C.c_int, vp, vp, vp, i64, vp, vp]),
    "fem_assemble_sell_pair": (C.c_int, [_P(FemBlocks), vp, vp, vp, i64, vp, vp, vp]),
    "fem_sell_apply64": (C.c_int, [_P(FemMatrix), vp, vp, vp, vp]),
    "fem_jacobi": (C.c_int, [vp, vp, i64, vp, vp, vp]),
    "fem_block_jacobi": (C.c_int, [_P(FemBlocks), vp, vp, vp, vp, vp]),
    "fem_set_timing": (None, [C.c_int]),
    "fem_amg_set_half_smoother": (None, [C.c_int]),
    "fem_amg_set_fused_cycle": (None, [C.c_int]),
    "fem_amg_set_level0_tma": (None, [C.c_int]),
    "fem_amg_rebind": (C.c_int, [vp, _P(FemMatrix)]),
    "fem_amg_set_pdl": (None, [C.c_int]),
    "fem_set_cg_path": (None, [C.c_int]),
    "fem_get_cg_path": (C.c_int, []),
    "fem_pcg_workspace_bytes": (C.c_size_t, [_P(FemMatrix)]),
    "fem_pcg": (
        C.c_int,
        [_P(FemMatrix), vp, vp, C.c_double, i64, vp, C.c_size_t, _P(FemSolveInfo), vp],
    ),
    "fem_pcg_static_max_unknowns": (i64, []),
    "fem_pcg_static": (
        C.c_int, [_P(FemMatrix), vp, vp, C.c_double, i64, _P(FemSolveInfo), vp]
    ),
    "fem_apply64_workspace_bytes": (C.c_size_t, [_P(FemOperator64)]),
    "fem_apply64": (C.c_int, [_P(FemOperator64), vp, vp, vp, C.c_size_t, vp]),
    "fem_pcg_mixed_workspace_bytes": (C.c_size_t, [_P(FemMatrix), _P(FemOperator64)]),
    "fem_pcg_mixed": (
        C.c_int,
        [_P(FemMatrix), _P(FemOperator64), vp, vp, C.c_double, C.c_double, i64, vp, C.c_size_t,
         _P(FemSolveInfo), vp],
    ),
}

_lib: C.CDLL | None = None


def symbols() -> list[str]:
    """Names of the entry points this binding declares."""
    return list(_SIGNATURES)


def load(path: str | Path | None = None) -> C.CDLL:
    """Loads the shared library (once) and declares every entry point."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"torchfem_gb300 CUDA library not built ({p}); run "
            "torchfem_gb300._build.build() or __graft_entry__.build()"
        )
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


class FemError(RuntimeError):
    """A library call returned a non-OK status."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def check(code: int, what: str) -> None:
    """Maps a FEM_* status to the exception type the reference raises."""
    if code == FEM_OK:
        return
    msg = f"{what}: {load().fem_last_error().decode(errors='replace')} (status {code})"
    if code == FEM_BAD_JACOBIAN:
        raise ValueError("Negative Jacobian. Check element numbering.")
    if code == FEM_INVALID:
        raise ValueError(msg)
    raise FemError(code, msg)


def ptr(t: torch.Tensor | None) -> int | None:
    """Device pointer of a tensor (None for a missing optional argument)."""
    if t is None:
        return None
    return t.data_ptr()


def stream_handle(device: torch.device) -> int:
    """cudaStream_t of torch's current stream on `device`."""
    return torch.cuda.current_stream(device).cuda_stream


def require_cuda() -> torch.device:
    """The compute device.  There is no CPU path: raise if CUDA is absent."""
    if not torch.cuda.is_available():
        raise RuntimeError(
            "torchfem_gb300 runs on a CUDA GPU (sm_103a); no CUDA device is available"
        )
    return torch.device("cuda", torch.cuda.current_device())
