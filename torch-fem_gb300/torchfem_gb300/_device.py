"""Device-resident state of one finite-element mesh and the C-ABI calls on it.

`DeviceMesh` owns everything the kernels need in HBM for a mesh: the
connectivity (int32), the node graph and CSR pattern (FEM.__init__,
src/torchfem/base.py:72-122), the block contributor lists of the
atomic-free assembly, and the geometry cache (shape-function gradients and
Jacobian determinants at every integration point, base.py:293-314), which
the reference recomputes on every integration pass.  All buffers are torch
tensors; the library only borrows their pointers.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch
from torch import Tensor

from . import _lib
from ._lib import check, ptr


def _i(x) -> int:
    return int(x)


@dataclass
class SolveStats:
    """Iteration record of the last linear solve."""

    iterations: int = 0
    replacements: int = 0
    rel_residual: float = 0.0
    spmv_ms: float = 0.0
    spmv_timed: int = 0


class LinearSystem:
    """Assembled, condensed stiffness matrix plus preconditioner on the device.

    precision "fp64": scalar CSR in the reference pattern, FP64 values,
    Jacobi preconditioner (the CuPy branch of sparse.py:406-421).
    precision "mixed": FP32 block-CSR over the node graph, FP32 block-Jacobi
    or smoothed-aggregation multigrid (`amg`), with FP64 residual
    replacement: one FP64 SpMV over an FP64 copy of the same sliced matrix,
    or the matrix-free FP64 element pass (`RESIDUAL_COPY`).
    """

    # The mixed solvers' FP64 residual.  True keeps an FP64 copy of the sliced
    # matrix (8 bytes per stored value more), built from FP64 element
    # matrices, and applies it with one FP64 SpMV: about a sixth of the FP64
    # work of the element pass per replacement.  False recomputes K x from
    # the element geometry on every replacement.  None (the default) takes
    # the copy where FP64 element matrices are cheap: heat conduction (one
    # DOF per node, integrated in FP64 anyway) and isotropic elasticity (the
    # moment form, fem_element_stiffness_iso64).  Other materials keep FP32
    # element matrices and the element pass: integrating their full FP64
    # element matrices costs more FP64 work than a solve's replacements save.
    RESIDUAL_COPY: bool | None = None

    @staticmethod
    def residual_copy(dm: "DeviceMesh", mat) -> bool:
        if LinearSystem.RESIDUAL_COPY is None:
            return dm.heat or mat.kind == _lib.FEM_MAT_ISO
        return bool(LinearSystem.RESIDUAL_COPY)

    _tokens = 0

    def __init__(self, dm: "DeviceMesh", precision: str):
        self.dm = dm
        self.precision = precision
        self.val: Tensor | None = None
        self.bval: Tensor | None = None
        self.bval64: Tensor | None = None
        self.precond: Tensor | None = None
        self.matrix = _lib.FemMatrix()
        self.ws: Tensor | None = None
        self.stats = SolveStats()
        self._op_refs = None
        self.amg: AmgHierarchy | None = None
        self.amg_ws: Tensor | None = None
        self.amg_fresh = True  # False: solved with an earlier matrix's multigrid setup
        LinearSystem._tokens += 1
        self.token = LinearSystem._tokens


class AmgHierarchy:
    """Smoothed-aggregation multigrid hierarchy of one mesh and constraint set
    (the fem_amg handle): the GPU counterpart of the pyamg / AmgX
    preconditioners of the reference (sparse.py:495-507, amgx.py).  The
    symbolic part (aggregation, tentative prolongator from the rigid-body
    modes of FEM.compute_B, every sparsity pattern) is built once; the
    numeric part is redone for each matrix (`setup`)."""

    def __init__(self, dm: "DeviceMesh", con_mask: Tensor):
        self.lib = dm.lib
        self.con_mask = con_mask.clone()
        handle = C.c_void_p()
        check(
            dm.lib.fem_amg_create(C.byref(dm.blocks), ptr(dm.nodes), ptr(self.con_mask), C.byref(handle),
                                  dm.stream),
            "fem_amg_create",
        )
        self.handle = handle
        self.current = 0  # token of the LinearSystem whose matrix is set up

    def setup(self, sysm: LinearSystem, stream: int) -> None:
        check(self.lib.fem_amg_setup(self.handle, C.byref(sysm.matrix), stream), "fem_amg_setup")
        self.current = sysm.token
        sysm.amg_fresh = True

    def rebind(self, sysm: LinearSystem) -> None:
        """Solve sysm's matrix with the preconditioner of the last setup
        (fem_amg_rebind)."""
        check(self.lib.fem_amg_rebind(self.handle, C.byref(sysm.matrix)), "fem_amg_rebind")
        self.current = sysm.token
        sysm.amg_fresh = False

    def levels(self) -> list[_lib.FemAmgLevel]:
        out = []
        for k in range(self.lib.fem_amg_levels(self.handle)):
            info = _lib.FemAmgLevel()
            check(self.lib.fem_amg_level_info(self.handle, k, C.byref(info)), "fem_amg_level_info")
            out.append(info)
        return out

    def close(self) -> None:
        if self.handle:
            self.lib.fem_amg_destroy(self.handle)
            self.handle = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:  # interpreter shutdown: the library may be gone
            pass


class DeviceMesh:
    """Pattern, geometry and kernels for one mesh on one CUDA device."""

    def __init__(self, nodes: Tensor, elements: Tensor, etype, dof_per_node: int, geometry: bool = True):
        self.device = _lib.require_cuda()
        self.lib = _lib.load()
        self.etype = etype
        self.n_e = etype.nodes
        self.dim = nodes.shape[1]
        self.d = dof_per_node
        # heat conduction: one temperature per node, flux [1, dim] per point
        self.heat = geometry and self.d == 1
        if geometry and self.d != self.dim and not self.heat:
            raise NotImplementedError("continua carry one DOF per spatial dimension or one temperature")
        self.flux_shape = (1, self.dim) if self.heat else (self.d, self.d)
        self.flux_n = self.flux_shape[0] * self.flux_shape[1]
        self.n_nod = nodes.shape[0]
        self.n_elem = elements.shape[0]
        self.n_dofs = self.n_nod * self.d
        dev = self.device
        self.nodes = nodes.detach().to(dev, torch.float64).contiguous()
        self.elements = elements.detach().to(dev, torch.int32).contiguous()
        table = etype.gradient_table()
        self.nip = table.shape[0]
        self.dndxi = table.to(dev).contiguous()
        self.weights = etype.iweights().to(dev, torch.float64).contiguous()
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)
        self._build_pattern()
        if geometry:
            self._build_geometry()
        else:  # structural elements (shells) bring their own element kernels
            self.mesh = self.make_mesh(None)

    # ------------------------------------------------------------ plumbing --
    @property
    def stream(self) -> int:
        return _lib.stream_handle(self.device)

    def _empty(self, n, dtype) -> Tensor:
        return torch.empty(int(n), dtype=dtype, device=self.device)

    def _ws(self, nbytes: int) -> Tensor:
        return torch.empty(max(int(nbytes), 256), dtype=torch.uint8, device=self.device)

    def check_status(self, what: str) -> None:
        """Reads the device status word (synchronises) and raises on a flag."""
        s = int(self.status.item())
        if s == 0:
            return
        self.status.zero_()
        if s & (1 << _lib.FEM_BAD_JACOBIAN):
            raise ValueError("Negative Jacobian. Check element numbering.")
        if s & (1 << _lib.FEM_BOUNDS):
            raise _lib.FemError(_lib.FEM_BOUNDS, f"{what}: index or size limit exceeded")
        if s & (1 << _lib.FEM_NONFINITE):
            raise _lib.FemError(_lib.FEM_NONFINITE, f"{what}: non-finite value")
        raise _lib.FemError(s, f"{what}: device status {s:#x}")

    # ------------------------------------------------------------- pattern --
    def _build_pattern(self) -> None:
        L, st = self.lib, self.stream
        n_nod, n_elem, n_e = self.n_nod, self.n_elem, self.n_e
        ws = self._ws(L.fem_pattern_workspace_bytes(n_nod, n_elem, n_e))
        self.inc_ptr = self._empty(n_nod + 1, torch.int64)
        self.inc = self._empty(max(n_elem * n_e, 1), torch.int32)
        self.nbr_ptr = self._empty(n_nod + 1, torch.int64)
        nb = C.c_int64(0)
        check(
            L.fem_pattern_graph_count(
                ptr(self.elements), n_elem, n_e, n_nod, ptr(self.inc_ptr), ptr(self.inc),
                ptr(self.nbr_ptr), C.byref(nb), ptr(ws), ws.numel(), ptr(self.status), st,
            ),
            "fem_pattern_graph_count",
        )
        self.check_status("pattern")
        self.n_blocks = nb.value
        self.nbr = self._empty(self.n_blocks, torch.int32)
        check(
            L.fem_pattern_graph_fill(
                ptr(self.elements), n_elem, n_e, n_nod, ptr(self.inc_ptr), ptr(self.inc),
                ptr(self.nbr_ptr), ptr(self.nbr), ptr(self.status), st,
            ),
            "fem_pattern_graph_fill",
        )
        self.row_ptr = self._empty(self.n_dofs + 1, torch.int64)
        nnz = C.c_int64(0)
        check(
            L.fem_pattern_csr_rows(
                ptr(self.nbr_ptr), n_nod, self.d, ptr(self.inc_ptr), ptr(self.row_ptr),
                C.byref(nnz), ptr(ws), ws.numel(), st,
            ),
            "fem_pattern_csr_rows",
        )
        self.nnz = nnz.value
        self.col = self._empty(self.nnz, torch.int32)
        self.diag_map = self._empty(self.n_dofs, torch.int64)
        check(
            L.fem_pattern_csr_cols(
                ptr(self.nbr_ptr), ptr(self.nbr), n_nod, self.d, ptr(self.inc_ptr),
                ptr(self.row_ptr), ptr(self.col), ptr(self.diag_map), st,
            ),
            "fem_pattern_csr_cols",
        )
        self.blk_ptr = self._empty(self.n_blocks + 1, torch.int64)
        self.contrib = self._empty(max(n_elem * n_e * n_e, 1), torch.int32)
        self.blk_row = self._empty(self.n_blocks, torch.int32)
        self.diag_blk = self._empty(n_nod, torch.int64)
        check(
            L.fem_pattern_blocks(
                ptr(self.elements), n_elem, n_e, n_nod, ptr(self.inc_ptr), ptr(self.inc),
                ptr(self.nbr_ptr), ptr(self.nbr), self.n_blocks, ptr(self.blk_ptr),
                ptr(self.contrib), ptr(self.blk_row), ptr(self.diag_blk), ptr(ws), ws.numel(),
                ptr(self.status), st,
            ),
            "fem_pattern_blocks",
        )
        self.check_status("pattern")
        del ws
        self.blocks = _lib.FemBlocks(
            n_e, self.d, n_nod, self.n_blocks, ptr(self.nbr_ptr), ptr(self.nbr), ptr(self.blk_ptr),
            ptr(self.contrib), ptr(self.blk_row), ptr(self.diag_blk), ptr(self.inc_ptr),
        )
        self._sell = None

    def sell(self):
        """Sliced block layout of the node graph (built on first use)."""
        if self._sell is None:
            L, st = self.lib, self.stream
            n_slices = (self.n_nod + 31) // 32
            base = self._empty(n_slices + 1, torch.int64)
            ws = self._ws(L.fem_sell_workspace_bytes(self.n_nod))
            n_slots = C.c_int64(0)
            check(L.fem_sell_layout(C.byref(self.blocks), ptr(base), C.byref(n_slots), ptr(ws), ws.numel(), st),
                  "fem_sell_layout")
            col = self._empty(max(n_slots.value, 1), torch.int32)
            check(L.fem_sell_columns(C.byref(self.blocks), ptr(base), ptr(col), st), "fem_sell_columns")
            self._sell = (base, col, n_slots.value)
        return self._sell

    def kmap(self) -> Tensor:
        """The reference's k_map (int64 here) for parity checks."""
        out = self._empty(self.n_elem * (self.n_e * self.d) ** 2, torch.int64)
        check(
            self.lib.fem_pattern_kmap(
                ptr(self.elements), self.n_elem, self.n_e, self.d, ptr(self.nbr_ptr), ptr(self.nbr),
                ptr(self.row_ptr), ptr(out), ptr(self.status), self.stream,
            ),
            "fem_pattern_kmap",
        )
        self.check_status("kmap")
        return out

    def glob_idx(self) -> Tensor:
        """[2, nnz] (row, col) of the CSR pattern, int64 (base.py:112-117)."""
        rows = torch.repeat_interleave(
            torch.arange(self.n_dofs, device=self.device), self.row_ptr.diff()
        )
        return torch.stack([rows, self.col.to(torch.int64)])

    # ------------------------------------------------------------ geometry --
    def _build_geometry(self) -> None:
        self.bt = self._empty(self.nip * self.n_elem * self.n_e * self.dim, torch.float64)
        self.detj = self._empty(self.nip * self.n_elem, torch.float64)
        self.mesh = self.make_mesh(None)
        check(
            self.lib.fem_geometry(
                C.byref(self.mesh), ptr(self.dndxi), ptr(self.bt), ptr(self.detj), ptr(self.status),
                self.stream,
            ),
            "fem_geometry",
        )
        self.check_status("geometry")
        self.mesh = self.make_mesh(None)

    def make_mesh(self, thickness: Tensor | None) -> _lib.FemMesh:
        return _lib.FemMesh(
            self.etype.etype_id, self.n_nod, self.n_elem, ptr(self.nodes), ptr(self.elements),
            ptr(self.weights), ptr(getattr(self, "bt", None)), ptr(getattr(self, "detj", None)),
            ptr(self.inc_ptr), ptr(self.inc), ptr(thickness), self.d,
        )

    # ------------------------------------------------------------ elements --
    def element_stiffness(self, mesh, mat, dtype=torch.float64) -> Tensor:
        nd = self.n_e * self.d
        ke = self._empty(self.n_elem * nd * nd, dtype)
        code = _lib.FEM_F64 if dtype == torch.float64 else _lib.FEM_F32
        if self.heat:
            check(self.lib.fem_heat_stiffness(C.byref(mesh), mat.data, code, ptr(ke), ptr(self.status), self.stream),
                  "fem_heat_stiffness")
            return ke.view(self.n_elem, nd, nd)
        check(
            self.lib.fem_element_stiffness(
                C.byref(mesh), C.byref(mat), code, ptr(ke), ptr(self.status), self.stream
            ),
            "fem_element_stiffness",
        )
        return ke.view(self.n_elem, nd, nd)

    def element_stiffness_iso64(self, mesh, mat) -> Tensor:
        """FP64 element matrices of an isotropic material in the moment form
        (fem_element_stiffness_iso64)."""
        nd = self.n_e * self.d
        ke = self._empty(self.n_elem * nd * nd, torch.float64)
        check(self.lib.fem_element_stiffness_iso64(C.byref(mesh), C.byref(mat), ptr(ke), ptr(self.status),
                                                   self.stream),
              "fem_element_stiffness_iso64")
        return ke.view(self.n_elem, nd, nd)

    def element_force(self, mesh, mat, v, con_mask=None, con_values=None, con_mode=0,
                      sigma_prev=None, de0=None, want_flux=False, want_h=False):
        fe = self._empty(self.n_elem * self.n_e * self.d, torch.float64)
        flux = self._empty(self.nip * self.n_elem * self.flux_n, torch.float64) if want_flux else None
        hg = self._empty(self.nip * self.n_elem * self.flux_n, torch.float64) if want_h else None
        if self.heat:
            check(
                self.lib.fem_heat_force(
                    C.byref(mesh), mat.data, ptr(v), ptr(con_mask), ptr(con_values), con_mode, ptr(sigma_prev),
                    ptr(de0), ptr(fe), ptr(flux), ptr(hg), ptr(self.status), self.stream,
                ),
                "fem_heat_force",
            )
            return fe, flux, hg
        check(
            self.lib.fem_element_force(
                C.byref(mesh), C.byref(mat), ptr(v), ptr(con_mask), ptr(con_values), con_mode,
                ptr(sigma_prev), ptr(de0), ptr(fe), ptr(flux), ptr(hg), ptr(self.status), self.stream,
            ),
            "fem_element_force",
        )
        return fe, flux, hg

    def gather(self, fe, sub=None, con_mask=None, con_mode=0, con_src=None, want_norm=False):
        out = self._empty(self.n_dofs, torch.float64)
        sumsq = None
        ws = None
        if want_norm:
            sumsq = self._empty(1, torch.float64)
            ws = self._ws(self.lib.fem_gather_workspace_bytes(self.n_dofs))
        check(
            self.lib.fem_gather_nodal(
                C.byref(self.mesh), ptr(fe), ptr(sub), ptr(con_mask), con_mode, ptr(con_src),
                ptr(out), ptr(sumsq), ptr(ws), 0 if ws is None else ws.numel(), self.stream,
            ),
            "fem_gather_nodal",
        )
        return out, sumsq

    def vjp(self, mesh, mat, v, g, con_mask=None, con_values=None, con_mode=0, sigma_prev=None,
            de0=None, gflux=None, gh=None, want_sig=False, want_mat=False, want_thick=False,
            want_de0=False, want_v=False, mat_numel=0):
        n_ip_e = self.nip * self.n_elem * self.flux_n
        gsig = self._empty(n_ip_e, torch.float64) if want_sig else None
        gmat = self._empty(mat_numel, torch.float64) if want_mat else None
        gthick = self._empty(self.n_elem, torch.float64) if want_thick else None
        gde0 = self._empty(self.n_elem * self.flux_n, torch.float64) if want_de0 else None
        gve = self._empty(self.n_elem * self.n_e * self.d, torch.float64) if want_v else None
        if self.heat:
            check(
                self.lib.fem_heat_vjp(
                    C.byref(mesh), mat.data, ptr(v), ptr(con_mask), ptr(con_values), con_mode, ptr(sigma_prev),
                    ptr(de0), ptr(g), ptr(gflux), ptr(gh), ptr(gsig), ptr(gmat), ptr(gthick), ptr(gde0),
                    ptr(gve), self.stream,
                ),
                "fem_heat_vjp",
            )
        else:
            check(
                self.lib.fem_element_vjp(
                    C.byref(mesh), C.byref(mat), ptr(v), ptr(con_mask), ptr(con_values), con_mode,
                    ptr(sigma_prev), ptr(de0), ptr(g), ptr(gflux), ptr(gh), ptr(gsig), ptr(gmat),
                    ptr(gthick), ptr(gde0), ptr(gve), ptr(self.status), self.stream,
                ),
                "fem_element_vjp",
            )
        gv = None
        if want_v:
            gv, _ = self.gather(gve)
        return gsig, gmat, gthick, gde0, gv

    # ------------------------------------------------------------ assembly --
    def assemble_csr(self, ke: Tensor, con_mask: Tensor) -> Tensor:
        val = self._empty(self.nnz, torch.float64)
        code = _lib.FEM_F64 if ke.dtype == torch.float64 else _lib.FEM_F32
        check(
            self.lib.fem_assemble_csr(
                C.byref(self.blocks), code, ptr(ke), ptr(self.row_ptr), ptr(con_mask), ptr(val),
                self.stream,
            ),
            "fem_assemble_csr",
        )
        return val

    def assemble_sell(self, ke: Tensor, con_mask: Tensor) -> Tensor:
        base, _, n_slots = self.sell()
        sval = self._empty(max(n_slots, 1) * self.d * self.d, torch.float32)
        code = _lib.FEM_F64 if ke.dtype == torch.float64 else _lib.FEM_F32
        check(
            self.lib.fem_assemble_sell(
                C.byref(self.blocks), code, ptr(ke), ptr(con_mask), ptr(base), n_slots, ptr(sval),
                self.stream,
            ),
            "fem_assemble_sell",
        )
        return sval

    def assemble_sell_pair(self, ke: Tensor, con_mask: Tensor) -> tuple[Tensor, Tensor]:
        """FP32 and FP64 copies of the sliced matrix from FP64 element
        matrices, in one pass."""
        base, _, n_slots = self.sell()
        nv = max(n_slots, 1) * self.d * self.d
        sval = self._empty(nv, torch.float32)
        sval64 = self._empty(nv, torch.float64)
        check(
            self.lib.fem_assemble_sell_pair(
                C.byref(self.blocks), ptr(ke), ptr(con_mask), ptr(base), n_slots, ptr(sval), ptr(sval64),
                self.stream,
            ),
            "fem_assemble_sell_pair",
        )
        return sval, sval64

    def amg_hierarchy(self, con_mask: Tensor) -> AmgHierarchy:
        """The multigrid hierarchy of this mesh for the constraint mask (built
        once per mask: it depends on the mesh and the constraints only)."""
        h = getattr(self, "_amg", None)
        if h is None or h.con_mask.shape != con_mask.shape or not torch.equal(h.con_mask, con_mask):
            if h is not None:
                h.close()
            h = AmgHierarchy(self, con_mask)
            self._amg = h
        return h

    def build_system(self, mesh, mat, con_mask: Tensor, precision: str, keep_refs=(),
                     precond: str = "jacobi", amg_reuse: bool = False) -> LinearSystem:
        """Element stiffness, assembly and preconditioner for one tangent.
        precond "amg" adds the multigrid hierarchy to a mixed system;
        amg_reuse keeps the hierarchy's last numeric setup as the
        preconditioner of the new matrix (fem_amg_rebind)."""
        sysm = LinearSystem(self, precision)
        L, st = self.lib, self.stream
        if precision == "fp64":
            ke = self.element_stiffness(mesh, mat, torch.float64)
            val = self.assemble_csr(ke, con_mask)
            del ke
            ws_bytes = self._set_csr(sysm, val)
        elif precision == "mixed":
            if LinearSystem.residual_copy(self, mat):
                if not self.heat and mat.kind == _lib.FEM_MAT_ISO:
                    ke = self.element_stiffness_iso64(mesh, mat)
                else:
                    ke = self.element_stiffness(mesh, mat, torch.float64)
                sysm.bval, sysm.bval64 = self.assemble_sell_pair(ke, con_mask)
            else:
                ke = self.element_stiffness(mesh, mat, torch.float32)
                sysm.bval = self.assemble_sell(ke, con_mask)
            del ke
            base, col, _ = self.sell()
            sysm.precond = self._empty(self.n_nod * self.d * self.d, torch.float32)
            check(
                L.fem_block_jacobi(C.byref(self.blocks), ptr(sysm.bval), ptr(base), ptr(sysm.precond),
                                   ptr(self.status), st),
                "fem_block_jacobi",
            )
            sysm.matrix = _lib.FemMatrix(
                _lib.FEM_FMT_SELL_F32, self.d, self.n_dofs, self.n_nod, ptr(base), ptr(col),
                ptr(sysm.bval), ptr(sysm.precond),
            )
            sysm.op_mesh = mesh
            sysm.op_mat = mat
            sysm.op = _lib.FemOperator64(C.pointer(mesh), C.pointer(mat), ptr(con_mask), ptr(sysm.bval64))
            ws_bytes = L.fem_pcg_mixed_workspace_bytes(C.byref(sysm.matrix), C.byref(sysm.op))
            if precond == "amg":
                sysm.amg = self.amg_hierarchy(con_mask)
                if amg_reuse and sysm.amg.current != 0:
                    sysm.amg.rebind(sysm)
                else:
                    sysm.amg.setup(sysm, st)
                sysm.amg_ws = self._ws(L.fem_amg_pcg_workspace_bytes(sysm.amg.handle, C.byref(sysm.op)))
        else:
            raise ValueError(f"unknown precision {precision!r}")
        sysm.con_mask = con_mask
        sysm._op_refs = keep_refs
        sysm.ws = self._ws(ws_bytes)
        self.check_status("assembly")
        return sysm

    def _set_csr(self, sysm: LinearSystem, val: Tensor) -> int:
        """FP64 CSR values plus their Jacobi preconditioner into sysm; returns
        the CG workspace size."""
        sysm.val = val
        sysm.precond = self._empty(self.n_dofs, torch.float64)
        check(
            self.lib.fem_jacobi(ptr(val), ptr(self.diag_map), self.n_dofs, ptr(sysm.precond), ptr(self.status),
                                self.stream),
            "fem_jacobi",
        )
        sysm.matrix = _lib.FemMatrix(
            _lib.FEM_FMT_CSR_F64, 1, self.n_dofs, self.n_dofs, ptr(self.row_ptr), ptr(self.col), ptr(val),
            ptr(sysm.precond),
        )
        return self.lib.fem_pcg_workspace_bytes(C.byref(sysm.matrix))

    def csr_system(self, val: Tensor, con_mask: Tensor) -> LinearSystem:
        """FP64 system (Jacobi CG) over already assembled CSR values."""
        sysm = LinearSystem(self, "fp64")
        sysm.ws = self._ws(self._set_csr(sysm, val))
        sysm.con_mask = con_mask
        self.check_status("assembly")
        return sysm

    # -------------------------------------------------------- heat transient --
    def heat_mass(self, mesh, rho: Tensor) -> Tensor:
        """Element capacity matrices [n_elem, n_e, n_e] (fem_heat_mass)."""
        nval = self.etype.N(self.etype.ipoints().to(torch.float64)).to(self.device, torch.float64).contiguous()
        me = self._empty(self.n_elem * self.n_e * self.n_e, torch.float64)
        check(
            self.lib.fem_heat_mass(C.byref(mesh), ptr(rho), ptr(nval), _lib.FEM_F64, ptr(me), ptr(self.status),
                                   self.stream),
            "fem_heat_mass",
        )
        return me.view(self.n_elem, self.n_e, self.n_e)

    def csr_combine(self, a: float, x: Tensor, b: float, y: Tensor) -> Tensor:
        out = self._empty(x.numel(), torch.float64)
        check(self.lib.fem_csr_combine(x.numel(), a, ptr(x), b, ptr(y), ptr(out), self.stream), "fem_csr_combine")
        return out

    def cn_residual(self, mass: LinearSystem, du: Tensor, f_old: Tensor | None, f_int: Tensor,
                    f_ext: Tensor | None, half_dt: float, con_mask: Tensor) -> tuple[Tensor, Tensor]:
        """M du + half_dt (f_old + f_int + f_ext), zero on constrained rows,
        and its squared norm (device scalar)."""
        res = self._empty(self.n_dofs, torch.float64)
        sumsq = self._empty(1, torch.float64)
        ws = self._ws(self.lib.fem_heat_cn_workspace_bytes(self.n_dofs))
        check(
            self.lib.fem_heat_cn_residual(
                C.byref(mass.matrix), ptr(du), ptr(f_old), ptr(f_int), ptr(f_ext), half_dt, ptr(con_mask),
                ptr(res), ptr(sumsq), ptr(ws), ws.numel(), self.stream,
            ),
            "fem_heat_cn_residual",
        )
        return res, sumsq

    def solve(self, sysm: LinearSystem, b: Tensor, rtol: float, max_iter: int | None = None,
              delta: float = 0.1, refine: bool = True, linear: str = "cg") -> Tensor:
        """x with A x = b (A the condensed system), from x = 0.  For the mixed
        system, refine=False runs the FP32 CG alone (an inner Newton solve
        whose FP64 refinement is the Newton iteration itself).  linear="minres"
        runs MINRES on the FP64 system."""
        x = self._empty(self.n_dofs, torch.float64)
        info = _lib.FemSolveInfo()
        if max_iter is None:
            max_iter = 10 * self.n_dofs
        b = b.contiguous()
        if linear == "minres":
            if sysm.precision != "fp64":
                raise ValueError("MINRES runs on the FP64 system")
            if getattr(sysm, "mr_ws", None) is None:
                sysm.mr_ws = self._ws(self.lib.fem_minres_workspace_bytes(C.byref(sysm.matrix)))
            rc = self.lib.fem_minres(
                C.byref(sysm.matrix), ptr(b), ptr(x), rtol, max_iter, ptr(sysm.mr_ws), sysm.mr_ws.numel(),
                C.byref(info), self.stream,
            )
            sysm.stats = SolveStats(info.iterations, 0, info.rel_residual, 0.0, 0)
            if rc == _lib.FEM_NOT_CONVERGED:
                raise RuntimeError(f"minres failed with exit code {info.iterations}")
            check(rc, "linear solve")
            return x
        if sysm.amg is not None:
            if sysm.amg.current != sysm.token:
                sysm.amg.setup(sysm, self.stream)
            op = C.byref(sysm.op) if refine else None
            rc = self.lib.fem_amg_pcg(
                sysm.amg.handle, C.byref(sysm.matrix), op, ptr(b), ptr(x), rtol, delta, max_iter,
                ptr(sysm.amg_ws), sysm.amg_ws.numel(), C.byref(info), self.stream,
            )
        elif sysm.precision == "fp64" or not refine:
            rc = self.lib.fem_pcg(
                C.byref(sysm.matrix), ptr(b), ptr(x), rtol, max_iter, ptr(sysm.ws), sysm.ws.numel(),
                C.byref(info), self.stream,
            )
        else:
            rc = self.lib.fem_pcg_mixed(
                C.byref(sysm.matrix), C.byref(sysm.op), ptr(b), ptr(x), rtol, delta, max_iter,
                ptr(sysm.ws), sysm.ws.numel(), C.byref(info), self.stream,
            )
        sysm.stats = SolveStats(info.iterations, info.replacements, info.rel_residual, info.spmv_ms,
                                info.spmv_timed)
        if rc == _lib.FEM_NOT_CONVERGED:
            raise RuntimeError(f"CG failed with exit code {info.iterations}")
        check(rc, "linear solve")
        return x

    # ------------------------------------------------------ nonlinear points --
    def hyper_force(self, mesh, params, v, con_mask=None, con_values=None, con_mode=0, F_prev=None,
                    want_tangent=False, want_flux=False, want_F=False, want_P=False):
        n_ip_e = self.nip * self.n_elem
        fe = self._empty(self.n_elem * self.n_e * 3, torch.float64)
        tangent = self._empty(n_ip_e * 81, torch.float64) if want_tangent else None
        flux = self._empty(n_ip_e * 9, torch.float64) if want_flux else None
        F_out = self._empty(n_ip_e * 9, torch.float64) if want_F else None
        P_out = self._empty(n_ip_e * 9, torch.float64) if want_P else None
        check(
            self.lib.fem_hyper_force(
                C.byref(mesh), ptr(params), ptr(v), ptr(con_mask), ptr(con_values), con_mode, ptr(F_prev),
                ptr(fe), ptr(P_out), ptr(tangent), ptr(flux), ptr(F_out), ptr(self.status), self.stream,
            ),
            "fem_hyper_force",
        )
        return fe, tangent, flux, F_out, P_out

    def hyper_vjp(self, mesh, params, v, g, con_mask=None, con_values=None, con_mode=0, F_prev=None,
                  gflux=None, gF=None, want_Fprev=False, want_params=False, want_v=False):
        n_ip_e = self.nip * self.n_elem
        gFprev = self._empty(n_ip_e * 9, torch.float64) if want_Fprev else None
        gparams = self._empty(self.n_elem * 2, torch.float64) if want_params else None
        gve = self._empty(self.n_elem * self.n_e * 3, torch.float64) if want_v else None
        check(
            self.lib.fem_hyper_vjp(
                C.byref(mesh), ptr(params), ptr(v), ptr(con_mask), ptr(con_values), con_mode, ptr(F_prev),
                ptr(g), ptr(gflux), ptr(gF), ptr(gFprev), ptr(gparams), ptr(gve), self.stream,
            ),
            "fem_hyper_vjp",
        )
        gv = self.gather(gve)[0] if want_v else None
        return gFprev, gparams, gv

    def plastic_force(self, mesh, params, tol, max_iter, v, con_mask=None, con_values=None, con_mode=0,
                      sigma_prev=None, state_prev=None, de0=None, want_tangent=False, want_outputs=False):
        n_ip_e = self.nip * self.n_elem
        fe = self._empty(self.n_elem * self.n_e * 2, torch.float64)
        tangent = self._empty(n_ip_e * 16, torch.float64) if want_tangent else None
        sig = self._empty(n_ip_e * 4, torch.float64) if want_outputs else None
        state = self._empty(n_ip_e * 2, torch.float64) if want_outputs else None
        hg = self._empty(n_ip_e * 4, torch.float64) if want_outputs else None
        check(
            self.lib.fem_plastic_force(
                C.byref(mesh), ptr(params), tol, max_iter, ptr(v), ptr(con_mask), ptr(con_values), con_mode,
                ptr(sigma_prev), ptr(state_prev), ptr(de0), ptr(fe), ptr(sig), ptr(state), ptr(tangent),
                ptr(hg), ptr(self.status), self.stream,
            ),
            "fem_plastic_force",
        )
        return fe, tangent, sig, state, hg

    def plastic_vjp(self, mesh, params, tol, max_iter, v, g, con_mask=None, con_values=None, con_mode=0,
                    sigma_prev=None, state_prev=None, de0=None, gsig=None, gstate=None, gh=None,
                    want_sig=False, want_state=False, want_thick=False, want_v=False):
        n_ip_e = self.nip * self.n_elem
        gsp = self._empty(n_ip_e * 4, torch.float64) if want_sig else None
        gst = self._empty(n_ip_e * 2, torch.float64) if want_state else None
        gth = self._empty(self.n_elem, torch.float64) if want_thick else None
        gve = self._empty(self.n_elem * self.n_e * 2, torch.float64) if want_v else None
        check(
            self.lib.fem_plastic_vjp(
                C.byref(mesh), ptr(params), tol, max_iter, ptr(v), ptr(con_mask), ptr(con_values), con_mode,
                ptr(sigma_prev), ptr(state_prev), ptr(de0), ptr(g), ptr(gsig), ptr(gstate), ptr(gh),
                ptr(gsp), ptr(gst), ptr(gth), ptr(gve), self.stream,
            ),
            "fem_plastic_vjp",
        )
        gv = self.gather(gve)[0] if want_v else None
        return gsp, gst, gth, gv
