"""Parts coupled by kinematic constraints (the reference's
src/torchfem/assembly.py): `Assembly`, `ReferencePoint`, `ReferencePointHeat`.

The host keeps the reference's bookkeeping (parts in DOF order, couplings as
rows of the elimination map T with u = T q, the checks and their messages).
The compute runs on the GPU:

* every part's FP64 matrix comes from the part's own kernels (element
  matrices and the deterministic CSR assembly), unconstrained;
* the reduced matrix K_r = T^T blockdiag(K_parts) T is formed by
  `fem_coupled_values` from per-entry contribution lists that the host builds
  once and keeps while the couplings and parts do not change (the pattern of
  K_r depends on them only), with the Dirichlet condensation of
  Assembly._stiffness;
* u = T q and T^T (F_int - F_ext) are `fem_csr_apply` products;
* the linear solves are the FP64 Jacobi CG (or MINRES) of the single models.

Gradients follow the reference's implicit adjoint (sparse.py:517-700): the
Newton solve of each increment is one autograd node whose backward solves
K_r lambda = g and pulls -lambda back through a differentiable re-evaluation
of the residual, whose parts are the single models' differentiable element
passes.  Parts with a constant tangent (linear materials, the linear shell)
are supported; a state-dependent tangent raises NotImplementedError.
"""

from __future__ import annotations

import ctypes as C
import math
from collections.abc import Iterable, Sequence

import numpy as np
import torch
from torch import Tensor

from . import _lib
from ._lib import check, ptr
from .base import FEM, Heat
from .shell import IntegrateShell, Shell, ShellContext
from .sparse import IntegrateMaterial, SolveContext

EMPTY = torch.empty(0, dtype=torch.int64)
K = 5  # differentiable inputs per part of a Newton node: u_prev, flux_prev, de0, material, thickness


class ReferencePoint:
    """A free node with rigid-body DOFs and no stiffness (assembly.py:39-73):
    three translations and three rotations in 3D, two and one in 2D."""

    n_nod = 1

    def __init__(self, position: Tensor | Sequence[float]):
        self.nodes = torch.as_tensor(position).reshape(1, -1)
        dim = self.nodes.shape[1]
        self.n_dof_per_node = dim + (3 if dim == 3 else 1)
        self.n_dofs = self.n_dof_per_node
        self._neumann = torch.zeros(1, self.n_dofs)
        self._dirichlet = torch.zeros(1, self.n_dofs)
        self._constraints = torch.zeros(1, self.n_dofs, dtype=torch.bool)

    forces = property(lambda self: self._neumann)
    displacements = property(lambda self: self._dirichlet)
    constraints = property(lambda self: self._constraints)

    def __repr__(self) -> str:
        at = ", ".join(f"{x:g}" for x in self.nodes[0].tolist())
        return f"<torch-fem reference point at ({at})>"


class ReferencePointHeat:
    """A free node with one temperature and no capacity (assembly.py:76-106)."""

    n_nod = 1
    n_dof_per_node = 1
    n_dofs = 1

    def __init__(self, position: Tensor | Sequence[float]):
        self.nodes = torch.as_tensor(position).reshape(1, -1)
        self._neumann = torch.zeros(1, 1)
        self._dirichlet = torch.zeros(1, 1)
        self._constraints = torch.zeros(1, 1, dtype=torch.bool)

    heat_flux = property(lambda self: self._neumann)
    temperatures = property(lambda self: self._dirichlet)
    constraints = property(lambda self: self._constraints)

    def __repr__(self) -> str:
        at = ", ".join(f"{x:g}" for x in self.nodes[0].tolist())
        return f"<torch-fem thermal reference point at ({at})>"


Part = FEM | ReferencePoint | ReferencePointHeat


def _csr(rows: np.ndarray, cols: np.ndarray, vals: np.ndarray, n_rows: int):
    """Row-sorted CSR (duplicates summed) of a COO triple, on the host."""
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    if len(rows):
        key = rows * (int(cols.max()) + 1 if len(cols) else 1) + cols
        first = np.r_[True, key[1:] != key[:-1]]
        grp = np.cumsum(first) - 1
        vals = np.bincount(grp, weights=vals, minlength=int(grp[-1]) + 1) if len(grp) else vals
        rows, cols = rows[first], cols[first]
    ptr_ = np.zeros(n_rows + 1, dtype=np.int64)
    np.add.at(ptr_, rows + 1, 1)
    return np.cumsum(ptr_), cols.astype(np.int32), np.asarray(vals, dtype=np.float64)


class _Apply(torch.autograd.Function):
    """y = A x over a device CSR pair (A, A^T): differentiable in x."""

    @staticmethod
    def forward(ctx, pair, x):
        ctx.pair = pair
        return pair.apply(x, transpose=False)

    @staticmethod
    def backward(ctx, g):
        return None, ctx.pair.apply(g.contiguous(), transpose=True)


class _CsrPair:
    """A rectangular FP64 CSR matrix and its transpose on the device."""

    def __init__(self, rows, cols, vals, shape, device):
        n, m = shape
        self.shape = shape
        self.device = device
        self.lib = _lib.load()
        fwd = _csr(rows, cols, vals, n)
        bwd = _csr(cols, rows, vals, m)
        self.fwd = tuple(torch.as_tensor(a).to(device) for a in fwd)
        self.bwd = tuple(torch.as_tensor(a).to(device) for a in bwd)

    def apply(self, x: Tensor, transpose: bool) -> Tensor:
        rp, col, val = self.bwd if transpose else self.fwd
        n = self.shape[1] if transpose else self.shape[0]
        y = torch.empty(n, dtype=torch.float64, device=self.device)
        check(self.lib.fem_csr_apply(n, ptr(rp), ptr(col), ptr(val), ptr(x.contiguous()), ptr(y),
                                     _lib.stream_handle(self.device)), "fem_csr_apply")
        return y

    def __call__(self, x: Tensor) -> Tensor:
        return _Apply.apply(self, x.contiguous())

    def t(self, x: Tensor) -> Tensor:
        return _Apply.apply(_Transposed(self), x.contiguous())


class _Transposed:
    def __init__(self, pair: _CsrPair):
        self.pair = pair

    def apply(self, x: Tensor, transpose: bool) -> Tensor:
        return self.pair.apply(x, transpose=not transpose)


class _PartSlot:
    """Device-side view of one part of a solve: its matrix, forces and
    differentiable inputs."""

    def __init__(self, part: Part, offset: int, device):
        self.part = part
        self.offset = offset
        self.n_dofs = part.n_dofs
        self.kind = "shell" if isinstance(part, Shell) else "fem" if isinstance(part, FEM) else "point"
        self.device = device
        self.ext = None

    def setup(self, track: bool, max_iter: int, rtol: float, atol: float, stol: float):
        part = self.part
        if self.kind == "point":
            return
        dm = part.device_mesh
        self.dm = dm
        zero = torch.zeros(part.n_dofs, dtype=torch.bool, device=dm.device)
        with torch.set_grad_enabled(track):
            if self.kind == "shell":
                self.sc = ShellContext(part, dm, zero, max_iter, rtol, atol, stol, None)
                self.mat = part.kernel_data().to(dm.device, torch.float64).contiguous()
                self.thick = part.thickness.expand(part.n_elem).to(dm.device, torch.float64).contiguous()
            else:
                kind, data = part.material.kernel_data(part.n_elem)
                if isinstance(kind, str):
                    raise NotImplementedError(
                        f"{type(part.material).__name__} has a state-dependent tangent; assemblies take parts "
                        "with a constant tangent"
                    )
                self.sc = SolveContext(dm, zero.to(torch.uint8), kind, "fp64", max_iter, rtol, atol, stol, None)
                self.mat = data.to(dm.device, torch.float64)
                th = part._thickness()
                self.thick = None if th is None else th.to(dm.device, torch.float64).contiguous()
                self.ext = (part._external_gradient.to(dm.device, torch.float64)
                            if getattr(part, "_external_gradient_set", False) else None)

    def matrix_values(self) -> Tensor:
        """The part's unconstrained FP64 CSR values (its pattern: dm.row_ptr, dm.col)."""
        if self.kind == "shell":
            self.sc.prepare(self.mat.detach(), self.thick.detach())
            return self.sc.system.val
        return self.sc.get_system(self.mat.detach(), None if self.thick is None else self.thick.detach()).val

    def forces(self, du: Tensor, u_prev: Tensor | None, sigma_prev: Tensor | None, de0: Tensor | None, mat,
               thick):
        """Internal forces of the part at the increment du (differentiable when
        the inputs track gradients), and the new flux and increment gradient."""
        if self.kind == "shell":
            f, stress = IntegrateShell.apply(self.sc, (u_prev + du).contiguous(), mat, thick)
            return f, stress, None
        self.sc.converged_eval = None
        f, flux, h = IntegrateMaterial.apply(self.sc, du.contiguous(), sigma_prev.contiguous(), de0, mat, thick)
        return f, flux, h


def coupled_pattern(T, patterns, n: int, con: np.ndarray):
    """Symbolic phase of K_r = T^T blockdiag(K_parts) T on the host.

    T: the coupling map as CSR (row_ptr, col, val) over all DOFs; patterns:
    per part (DOF offset, CSR row_ptr, CSR col) of its matrix, whose values
    are concatenated in this order; n: retained DOFs; con: constrained
    retained DOFs (bool [n]).  Returns the CSR pattern of K_r (row_ptr, col),
    with an explicit diagonal for every row as Assembly._stiffness adds it,
    and per entry its contributions (ptr, src value index, coef = product of
    the two T coefficients) sorted by entry then by source, the condensation
    flags (1 zero, 2 unit diagonal) and the diagonal positions.
    """
    tp, tc, tv = T
    n_all = len(tp) - 1
    cnt = np.diff(tp)
    head = tp[:-1]
    # most rows of T are one unit entry (a retained DOF, or a DOF tied to one
    # primary DOF): per DOF, that entry's column and coefficient; a pair of
    # such rows maps one part entry to one entry of K_r directly
    single = cnt == 1
    tgt = np.zeros(n_all, dtype=np.int64)
    cf = np.zeros(n_all)
    tgt[single] = tc[head[single]]
    cf[single] = tv[head[single]]
    key1, c1, s1, ks, ls, qs = [], [], [], [], [], []
    voff = 0
    for offset, rp, cl in patterns:
        m = np.diff(rp)
        d = np.arange(offset, offset + len(m), dtype=np.int64)
        col = cl + offset
        one = np.repeat(single[d], m) & single[col]
        row = np.repeat(d, m)
        io = np.flatnonzero(one)
        ko, lo = row[io], col[io]
        key1.append(tgt[ko] * n + tgt[lo])
        c1.append(cf[ko] * cf[lo])
        s1.append(io + voff)
        # the other pairs touch a row with several entries (a reference
        # point's rigid map): expanded below
        rest = np.flatnonzero(~one)
        kr, lr = row[rest], col[rest]
        keep = (cnt[kr] > 0) & (cnt[lr] > 0)
        ks.append(kr[keep])
        ls.append(lr[keep])
        qs.append(rest[keep] + voff)
        voff += int(rp[-1])

    def cat(xs, dt):
        return np.concatenate(xs) if xs else np.zeros(0, dt)

    key1, c1, s1 = cat(key1, np.int64), cat(c1, np.float64), cat(s1, np.int64)
    k, l_, q = cat(ks, np.int64), cat(ls, np.int64), cat(qs, np.int64)
    tk, tl, cl_ = head[k], head[l_], cnt[l_]
    sizes = cnt[k] * cl_
    total = int(sizes.sum())
    grp = np.repeat(np.arange(len(tk)), sizes)
    start = np.repeat(np.cumsum(sizes) - sizes, sizes)
    pos = np.arange(total, dtype=np.int64) - start
    a_i = tk[grp] + pos // cl_[grp]
    b_i = tl[grp] + pos % cl_[grp]
    diag = np.arange(n, dtype=np.int64)
    key = np.concatenate([key1, tc[a_i].astype(np.int64) * n + tc[b_i], diag * (n + 1)])
    coef = np.concatenate([c1, tv[a_i] * tv[b_i], np.zeros(n)])  # the explicit zero diagonal adds nothing
    src = np.concatenate([s1, q[grp], np.zeros(n, dtype=np.int64)])
    order = np.lexsort((src, key))
    key, coef, src = key[order], coef[order], src[order]
    first = np.empty(len(key), dtype=bool)
    if len(key):
        first[0] = True
        np.not_equal(key[1:], key[:-1], out=first[1:])
    starts = np.flatnonzero(first)
    cptr = np.append(starts, len(key)).astype(np.int64)
    rows, cols = np.divmod(key[starts], n)
    rptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(np.bincount(rows, minlength=n), out=rptr[1:])
    fix = np.zeros(len(starts), dtype=np.uint8)
    if con.any():
        fix[con[rows] | con[cols]] = 1
        fix[(rows == cols) & con[rows]] = 2
    diag_map = np.flatnonzero(rows == cols).astype(np.int64)
    return rptr, cols.astype(np.int32), cptr, src, coef, fix, diag_map


class _CoupledPattern:
    """What a solve needs that depends only on the couplings and the parts'
    patterns: the map T on the device, the pattern of K_r = T^T K T and its
    per-entry contribution lists.  Built once and kept by the Assembly for
    later solves while neither changes; the condensation flags are kept per
    constraint set."""

    def __init__(self, T_rows, T_cols, T_vals, n_all: int, n: int, slots: list[_PartSlot], device):
        self.n_all, self.n = n_all, n
        self.device = device
        self.T = _CsrPair(T_rows, T_cols, T_vals, (n_all, n), device)
        patterns = []
        voff = 0
        self.part_vals: list[tuple[int, int, int]] = []  # (slot index, value offset, values)
        for j, s in enumerate(slots):
            if s.kind == "point":
                continue
            rp = s.dm.row_ptr.cpu().numpy().astype(np.int64)
            cl = s.dm.col.cpu().numpy().astype(np.int64)
            patterns.append((s.offset, rp, cl))
            self.part_vals.append((j, voff, int(rp[-1])))
            voff += int(rp[-1])
        self.n_kval = voff
        T = _csr(T_rows, T_cols, T_vals, n_all)
        rptr, cols, cptr, src, coef, _, diag_map = coupled_pattern(T, patterns, n, np.zeros(n, dtype=bool))
        self.nnz = len(cols)
        self.rows_host = np.repeat(np.arange(n, dtype=np.int32), np.diff(rptr))
        self.cols_host = cols
        self.row_ptr = torch.as_tensor(rptr).to(device)
        self.col = torch.as_tensor(cols.astype(np.int32)).to(device)
        self.cptr = torch.as_tensor(cptr).to(device)
        self.src = torch.as_tensor(src).to(device)
        self.coef = torch.as_tensor(coef).to(device)
        self.diag_map = torch.as_tensor(diag_map).to(device)
        self._fix: dict[bytes, Tensor] = {}

    def fix_for(self, con: np.ndarray) -> Tensor:
        """Condensation flags of K_r for these constrained retained DOFs."""
        key = np.packbits(con).tobytes()
        f = self._fix.get(key)
        if f is None:
            r, c = self.rows_host, self.cols_host
            fix = np.zeros(self.nnz, dtype=np.uint8)
            fix[con[r] | con[c]] = 1
            fix[(r == c) & con[r]] = 2
            f = torch.as_tensor(fix).to(self.device)
            self._fix = {key: f}
        return f


class _AssemblyContext:
    """What one Assembly.solve shares between its Newton steps and backward."""

    def __init__(self, asm: "Assembly", pattern: _CoupledPattern, con: Tensor, device, slots: list[_PartSlot],
                 stol: float, max_iter: int, rtol: float, atol: float, linear: str):
        self.asm = asm
        self.device = device
        self.lib = _lib.load()
        self.slots = slots
        self.pattern = pattern
        self.n_all = asm.n_dofs
        self.n = pattern.n
        self.stol, self.max_iter, self.rtol, self.atol = stol, max_iter, rtol, atol
        self.linear = linear
        self.T = pattern.T
        con_bool = torch.zeros(self.n, dtype=torch.bool)
        con_bool[con] = True
        self.con_bool = con_bool.to(device)
        self.fix = pattern.fix_for(con_bool.numpy())
        self.part_vals = [(slots[j], voff, nnz) for j, voff, nnz in pattern.part_vals]
        self.n_kval = pattern.n_kval
        n, nnz = self.n, pattern.nnz
        self.nnz = nnz
        self.row_ptr, self.col = pattern.row_ptr, pattern.col
        self.cptr, self.src, self.coef, self.diag_map = pattern.cptr, pattern.src, pattern.coef, pattern.diag_map
        self.val = torch.empty(nnz, dtype=torch.float64, device=device)
        self.precond = torch.empty(n, dtype=torch.float64, device=device)
        self.status = torch.zeros(1, dtype=torch.int32, device=device)
        self.matrix = _lib.FemMatrix(_lib.FEM_FMT_CSR_F64, 1, n, n, ptr(self.row_ptr), ptr(self.col),
                                     ptr(self.val), ptr(self.precond))
        self.ws = torch.empty(max(int(self.lib.fem_pcg_workspace_bytes(C.byref(self.matrix))), 256),
                              dtype=torch.uint8, device=device)
        self.mr_ws = None
        self.iterations: list[int] = []
        self.newton_iterations: list[int] = []
        self.spmv_ms = 0.0  # CUDA-event time of the timed CG iterations (fem_set_timing)
        self.spmv_timed = 0
        self.verbose = False
        self.values_ready = False

    # ------------------------------------------------------------- values --
    def assemble(self):
        """Values of K_r and its Jacobi inverse diagonal (constant tangents:
        once per solve)."""
        if self.values_ready:
            return
        st = _lib.stream_handle(self.device)
        kval = torch.zeros(max(self.n_kval, 1), dtype=torch.float64, device=self.device)
        for s, voff, nnz in self.part_vals:
            kval[voff:voff + nnz] = s.matrix_values()
        check(self.lib.fem_coupled_values(self.nnz, ptr(self.cptr), ptr(self.src), ptr(self.coef), ptr(kval),
                                          ptr(self.fix), ptr(self.val), st), "fem_coupled_values")
        check(self.lib.fem_jacobi(ptr(self.val), ptr(self.diag_map), self.n, ptr(self.precond), ptr(self.status),
                                  st), "fem_jacobi")
        if int(self.status.item()) != 0:
            raise RuntimeError("Assembly: a retained DOF has no stiffness (a zero diagonal of the coupled "
                               "matrix); couple or constrain it")
        self.values_ready = True

    def solve(self, b: Tensor) -> Tensor:
        self.assemble()
        x = torch.empty(self.n, dtype=torch.float64, device=self.device)
        info = _lib.FemSolveInfo()
        st = _lib.stream_handle(self.device)
        b = b.contiguous()
        if self.linear == "minres":
            if self.mr_ws is None:
                self.mr_ws = torch.empty(max(int(self.lib.fem_minres_workspace_bytes(C.byref(self.matrix))), 256),
                                         dtype=torch.uint8, device=self.device)
            rc = self.lib.fem_minres(C.byref(self.matrix), ptr(b), ptr(x), self.stol, 10 * self.n, ptr(self.mr_ws),
                                     self.mr_ws.numel(), C.byref(info), st)
        else:
            rc = self.lib.fem_pcg(C.byref(self.matrix), ptr(b), ptr(x), self.stol, 10 * self.n, ptr(self.ws),
                                  self.ws.numel(), C.byref(info), st)
        if rc == _lib.FEM_NOT_CONVERGED:
            raise RuntimeError(f"CG failed with exit code {info.iterations}")
        check(rc, "assembly linear solve")
        self.iterations.append(int(info.iterations))
        self.spmv_ms += float(info.spmv_ms)
        self.spmv_timed += int(info.spmv_timed)
        return x

    # ----------------------------------------------------------- residual --
    def residual(self, q: Tensor, F_ext: Tensor, DU: Tensor, part_in: list) -> Tensor:
        """T^T (F_int(T constrain(q)) - F_ext), zero on constrained rows;
        differentiable when called with grad enabled."""
        qc = torch.where(self.con_bool, DU, q)
        du = self.T(qc)
        F_int = []
        for s, inp in zip(self.slots, part_in):
            if s.kind == "point":
                F_int.append(torch.zeros(s.n_dofs, dtype=torch.float64, device=self.device))
                continue
            u_prev, sigma_prev, de0, mat, thick = inp
            f, _, _ = s.forces(du[s.offset:s.offset + s.n_dofs], u_prev, sigma_prev, de0, mat, thick)
            F_int.append(f)
        res = self.T.t(torch.cat(F_int) - F_ext)
        return torch.where(self.con_bool, torch.zeros_like(res), res)


class _AssemblyNewton(torch.autograd.Function):
    """Newton solve of one increment of an assembly: forward iterates, backward
    is the implicit adjoint (the reference's NewtonRaphsonAdjoint,
    sparse.py:517-700)."""

    @staticmethod
    def forward(ctx, actx: _AssemblyContext, q0, F_ext, DU, *flat):
        part_in = [tuple(flat[K * j:K * j + K]) for j in range(len(actx.slots))]
        q = q0.detach().clone()
        res0 = None
        converged = False
        with torch.no_grad():
            for i in range(actx.max_iter):
                res = actx.residual(q, F_ext, DU, part_in)
                res_norm = float(torch.linalg.norm(res))
                if i == 0:
                    res0 = res_norm
                if actx.verbose:
                    print(f"  newton {i:2d}  |res| = {res_norm:.6e}")
                if res_norm < actx.rtol * res0 or res_norm < actx.atol:
                    converged = True
                    actx.newton_iterations.append(i)
                    break
                if not math.isfinite(res_norm):
                    break
                q = q - actx.solve(res)
        if not converged:
            raise RuntimeError("Newton-Raphson iteration did not converge.")
        ctx.actx = actx
        ctx.n_flat = len(flat)
        ctx.save_for_backward(q, F_ext, DU, *[t if t is not None else torch.empty(0) for t in flat])
        ctx.flat_none = [t is None for t in flat]
        return q

    @staticmethod
    def backward(ctx, grad_q):
        actx: _AssemblyContext = ctx.actx
        q, F_ext, DU, *flat = ctx.saved_tensors
        flat = [None if none else t for t, none in zip(flat, ctx.flat_none)]
        need = ctx.needs_input_grad
        g = torch.where(actx.con_bool, torch.zeros_like(grad_q), grad_q).contiguous()
        lam = actx.solve(g)
        wants = [(2, F_ext), (3, DU)] + [(4 + i, t) for i, t in enumerate(flat)]
        live = [(i, t) for i, t in wants if t is not None and need[i]]
        grads = [None] * (4 + len(flat))
        if live:
            with torch.enable_grad():
                leaves = {i: t.detach().requires_grad_(True) for i, t in live}
                F_d = leaves.get(2, F_ext)
                DU_d = leaves.get(3, DU)
                flat_d = [leaves.get(4 + i, t) for i, t in enumerate(flat)]
                part_in = [tuple(flat_d[K * j:K * j + K]) for j in range(len(actx.slots))]
                res = actx.residual(q.detach(), F_d, DU_d, part_in)
                out = torch.autograd.grad(res, [leaves[i] for i, _ in live], grad_outputs=-lam, allow_unused=True)
            for (i, _), gi in zip(live, out):
                grads[i] = gi
        return tuple(grads)


class Assembly:
    """Several models coupled by kinematic constraints (assembly.py:113-650).

    Parts keep their own nodes, elements, materials and boundary conditions;
    their DOFs are stacked in the order given, and `coupling(...)` ties
    secondary nodes to the nearest primary nodes: translations follow
    u_s = u_p + theta_p x (x_s - x_p), rotations follow theta_s = theta_p.
    Secondary DOFs are eliminated, so the solved system stays symmetric
    positive definite.  The parts share one physics and one dimension.
    """

    def __init__(self, parts: Sequence[Part]):
        if len({id(part) for part in parts}) != len(parts):
            raise ValueError("A part may appear only once in an assembly.")
        dims = {part.nodes.shape[1] for part in parts}
        if len(dims) != 1:
            raise ValueError("All parts of an assembly share one spatial dimension.")
        self.dim = dims.pop()
        thermal = [isinstance(part, (Heat, ReferencePointHeat)) for part in parts]
        if any(thermal) and not all(thermal):
            raise ValueError("An assembly is either mechanical or thermal, not both.")
        self.parts = list(parts)
        sizes = [part.n_dofs for part in self.parts]
        self.offsets = [sum(sizes[:i]) for i in range(len(sizes))]
        self.n_dofs = sum(sizes)
        self._at = {id(part): offset for part, offset in zip(self.parts, self.offsets)}
        self._eliminated: list[Tensor] = [EMPTY]
        self._rows: list[tuple[Tensor, Tensor, Tensor]] = [(EMPTY, EMPTY, torch.empty(0, dtype=torch.float64))]
        self._links: list = []
        self.last_solve: _AssemblyContext | None = None
        self._version = 0  # bumped by every coupling: the cached pattern is then rebuilt
        self._pattern: tuple | None = None  # (key, _CoupledPattern)

    def __repr__(self) -> str:
        return f"<torch-fem assembly ({len(self.parts)} parts, {self.n_dofs} dofs)>"

    def coupling(self, secondary: Part, mask: Tensor, primary: Part, primary_mask: Tensor | None = None,
                 dofs: Iterable[int] | None = None):
        """Couples nodes of `secondary` to the nearest nodes of `primary`
        (assembly.py:180-247)."""
        if id(secondary) not in self._at or id(primary) not in self._at:
            raise ValueError("Both parts must belong to this assembly.")
        n_sec = secondary.n_dof_per_node
        n_pri = primary.n_dof_per_node
        dofs = list(range(n_sec)) if dofs is None else list(dofs)
        if any(dof < 0 or dof >= n_sec for dof in dofs):
            raise ValueError(f"dofs must be indices in [0, {n_sec}) for this part.")
        if any(dof >= self.dim for dof in dofs) and n_pri <= self.dim:
            raise ValueError("Rotational DOFs cannot be coupled to a primary part that has none.")
        mask = torch.as_tensor(mask).cpu()
        secondary_nodes = torch.nonzero(mask).ravel()
        if primary_mask is None:
            primary_nodes = torch.arange(primary.n_nod)
        else:
            primary_nodes = torch.nonzero(torch.as_tensor(primary_mask).cpu()).ravel()
        x_sec = secondary.nodes.detach().cpu().to(torch.float64)[secondary_nodes]
        x_pri_all = primary.nodes.detach().cpu().to(torch.float64)
        distance = torch.cdist(x_sec, x_pri_all[primary_nodes])
        primary_nodes = primary_nodes[distance.argmin(dim=1)]
        self._links.append(((secondary, secondary_nodes), (primary, primary_nodes)))
        self._version += 1
        secondary_base = self._at[id(secondary)] + secondary_nodes * n_sec
        primary_base = self._at[id(primary)] + primary_nodes * n_pri
        ones = torch.ones(len(secondary_nodes), dtype=torch.float64)
        skew = self._skew(x_sec - x_pri_all[primary_nodes])
        axes = (0, 1, 2) if self.dim == 3 else (2,)
        for dof in dofs:
            self._eliminated.append(secondary_base + dof)
            self._rows.append((secondary_base + dof, primary_base + dof, ones))
            if dof < self.dim and n_pri > self.dim:
                for b, axis in enumerate(axes):
                    rot = primary_base + self.dim + b
                    self._rows.append((secondary_base + dof, rot, skew[:, dof, axis]))

    def _skew(self, r: Tensor) -> Tensor:
        """Columns of the theta x r operator (assembly.py:248-257)."""
        r = torch.cat([r, torch.zeros(len(r), 3 - self.dim, dtype=r.dtype)], dim=1)
        eye = torch.eye(3, dtype=r.dtype).expand(len(r), 3, 3)
        cross = torch.linalg.cross(eye, r[:, None, :].expand(-1, 3, -1), dim=-1)
        return cross.transpose(1, 2)

    def _build_T(self):
        """Rows, columns and values of the map u = T q, and the retained DOFs
        (assembly.py:258-294), with the reference's checks."""
        eliminated = torch.cat(self._eliminated)
        if len(torch.unique(eliminated)) != len(eliminated):
            raise ValueError("A DOF is eliminated by more than one constraint.")
        keep = torch.ones(self.n_dofs, dtype=torch.bool)
        keep[eliminated] = False
        retained = torch.nonzero(keep).ravel()
        column = torch.full((self.n_dofs,), -1, dtype=torch.int64)
        column[retained] = torch.arange(len(retained))
        secondary, primary, coeffs = (torch.cat(x) for x in zip(*self._rows))
        if bool((column[primary] < 0).any()):
            raise ValueError(
                "A DOF is both eliminated and used as a primary. Chain the constraints to an independent part instead."
            )
        rows = torch.cat([retained, secondary]).numpy()
        cols = torch.cat([column[retained], column[primary]]).numpy()
        vals = torch.cat([torch.ones(len(retained), dtype=torch.float64), coeffs.to(torch.float64)]).numpy()
        return rows, cols, vals, retained

    def solve(self, increments: Tensor | None = None, max_iter: int = 10, rtol: float = 1e-8, atol: float = 1e-6,
              stol: float = 1e-10, verbose: bool = False, method: str | None = None, device: str | None = None,
              return_intermediate: bool = False, aggregate_integration_points: bool = True,
              differentiable_parameters: Tensor | Iterable[Tensor] | None = None):
        """Quasi-static solve of the coupled parts by load increments
        (assembly.py:378-608).  Same arguments and results as the reference:
        lists with one entry per part of (u, f, flux, grad, state).  The
        linear solves run on the GPU in FP64 ("cg"/None: Jacobi CG,
        "minres": Jacobi MINRES)."""
        if method in ("spsolve", "pardiso", "amgx"):
            raise RuntimeError(
                f"Method '{method}' is a CPU/third-party backend of torch-fem; torchfem_gb300 solves assemblies "
                "with its own GPU Krylov methods ('cg', 'minres')."
            )
        if method not in (None, "cg", "minres", "gb300"):
            raise ValueError(f"Method {method} is not supported for assemblies. Choose 'cg' or 'minres'.")
        if device is not None and torch.device(device).type != "cuda":
            raise RuntimeError("torchfem_gb300 solves on a CUDA device only")
        increments = torch.tensor([0.0, 1.0]) if increments is None else increments
        N = len(increments)
        if differentiable_parameters is None:
            differentiable_parameters = ()
        elif isinstance(differentiable_parameters, Tensor):
            differentiable_parameters = (differentiable_parameters,)
        else:
            differentiable_parameters = tuple(differentiable_parameters)
        track = any(p.requires_grad for p in differentiable_parameters)

        T_rows, T_cols, T_vals, retained = self._build_T()
        constrained = torch.cat([p._constraints.reshape(-1).cpu() for p in self.parts])
        con = torch.nonzero(constrained[retained]).ravel()
        if len(con) != int(constrained.sum()):
            raise ValueError("A constrained DOF is eliminated by a constraint. Constrain the primary part instead.")
        dev = _lib.require_cuda()
        with torch.set_grad_enabled(track):
            neumann = torch.cat([p._neumann.reshape(-1).to(dev, torch.float64) for p in self.parts])
            dirichlet = torch.cat([p._dirichlet.reshape(-1).to(dev, torch.float64) for p in self.parts])

        slots = [_PartSlot(p, off, dev) for p, off in zip(self.parts, self.offsets)]
        for s in slots:
            s.setup(track, max_iter, rtol, atol, stol)
        key = (self._version, tuple(id(s.dm) if s.kind != "point" else None for s in slots))
        if self._pattern is None or self._pattern[0] != key:
            self._pattern = (key, _CoupledPattern(T_rows, T_cols, T_vals, self.n_dofs, len(retained), slots, dev))
        actx = _AssemblyContext(self, self._pattern[1], con, dev, slots, stol, max_iter, rtol, atol,
                                "minres" if method == "minres" else "cg")
        actx.verbose = verbose
        self.last_solve = actx
        retained_d = retained.to(dev)

        # per-part running state: total displacement, flux, gradient, state
        u_all = torch.zeros(self.n_dofs, dtype=torch.float64, device=dev)
        flux_cur, grad_cur, state_cur, shapes = [], [], [], []
        for p in self.parts:
            if not isinstance(p, FEM):
                flux_cur.append(torch.zeros(0, dtype=torch.float64, device=dev))
                grad_cur.append(torch.zeros(0, dtype=torch.float64, device=dev))
                state_cur.append(torch.zeros(0, dtype=torch.float64, device=dev))
                continue
            field = (p.n_int, p.n_elem, *p.n_flux)
            flux_cur.append(torch.zeros(field, dtype=torch.float64, device=dev))
            g0 = torch.zeros(field, dtype=torch.float64, device=dev)
            g0[:] = p.initial_grad.to(dev, torch.float64)
            grad_cur.append(g0)
            state_cur.append(torch.zeros(p.n_int, p.n_elem, p.n_state, dtype=torch.float64, device=dev))
        outs = [[[] for _ in self.parts] for _ in range(5)]

        def record(u_all, f_all):
            for j, p in enumerate(self.parts):
                blk = slice(self.offsets[j], self.offsets[j] + p.n_dofs)
                outs[0][j].append(u_all[blk].reshape(p.n_nod, p.n_dof_per_node))
                outs[1][j].append(f_all[blk].reshape(p.n_nod, p.n_dof_per_node))
                outs[2][j].append(flux_cur[j])
                outs[3][j].append(grad_cur[j])
                outs[4][j].append(state_cur[j])

        record(u_all, torch.zeros_like(u_all))
        dq = torch.zeros(len(retained), dtype=torch.float64, device=dev)
        with torch.set_grad_enabled(track):
            for n in range(1, N):
                level = float(increments[n])
                step = level - float(increments[n - 1])
                if verbose:
                    print(f"increment {n}: load {level:.6g}")
                F_ext = (level * neumann).contiguous()
                DU = (step * dirichlet)[retained_d].contiguous()
                flat = []
                for j, s in enumerate(slots):
                    if s.kind == "point":
                        flat += [None] * K
                    elif s.kind == "shell":
                        u_prev = u_all[s.offset:s.offset + s.n_dofs]
                        u_prev = (u_prev if track else u_prev.detach()).contiguous()
                        flat += [u_prev, None, None, s.mat, s.thick]
                    else:
                        sig = flux_cur[j] if track else flux_cur[j].detach()
                        de0 = None if s.ext is None else (step * s.ext).contiguous()
                        flat += [None, sig.contiguous(), de0, s.mat, s.thick]
                dq = _AssemblyNewton.apply(actx, dq.detach(), F_ext, DU, *flat)
                # the converged state, whose tangent is not needed
                qc = torch.where(actx.con_bool, DU, dq)
                du = actx.T(qc)
                F_int = []
                for j, s in enumerate(slots):
                    if s.kind == "point":
                        F_int.append(torch.zeros(s.n_dofs, dtype=torch.float64, device=dev))
                        continue
                    u_prev, sig, de0, mat, thick = flat[K * j:K * j + K]
                    f, flux_new, h = s.forces(du[s.offset:s.offset + s.n_dofs], u_prev, sig, de0, mat, thick)
                    F_int.append(f)
                    flux_cur[j] = flux_new
                    if h is not None:
                        grad_cur[j] = grad_cur[j] + h
                F_all = torch.cat(F_int)
                # a retained DOF carries what the constraints transmit into it
                f_cur = F_all.index_put((retained_d,), actx.T.t(F_all))
                u_all = u_all + du
                dq = qc
                record(u_all, f_cur)

        result = []
        for q_i, per_part in enumerate(outs):
            vals = [torch.stack(x) for x in per_part]
            result.append(vals)
        u, f, flux, grad, state = result
        if aggregate_integration_points:
            grad = [x.mean(dim=1) if x.dim() > 2 else x for x in grad]
            flux = [x.mean(dim=1) if x.dim() > 2 else x for x in flux]
            state = [x.mean(dim=1) if x.dim() > 2 else x for x in state]
        flux = [x.squeeze((-2, -1)) if x.dim() > 2 else x for x in flux]
        grad = [x.squeeze((-2, -1)) if x.dim() > 2 else x for x in grad]
        out = [u, f, flux, grad, state]
        for q_i in range(5):
            fixed = []
            for j, x in enumerate(out[q_i]):
                if q_i >= 2 and not isinstance(self.parts[j], FEM):
                    x = x.reshape(N, 0)
                x = x if track else x.detach()
                fixed.append(x.to(self.parts[j].nodes.device, self.parts[j].nodes.dtype))
            out[q_i] = fixed
        if not return_intermediate:
            out = [[x[-1] for x in q] for q in out]
        return out[0], out[1], out[2], out[3], out[4]
