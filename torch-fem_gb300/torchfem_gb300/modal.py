"""Modal analysis on the GPU: `FEM.solve_modes` (src/torchfem/base.py:1097-1129)
with the differentiable eigen-solve of src/torchfem/sparse.py:798-1011.

The reference solves K phi = omega^2 M phi on the free DOFs with scipy's (or
CuPy's) shift-invert `eigsh` and differentiates the eigenvalues with the
Rayleigh-quotient sensitivities d(omega^2)/dK_ij = phi_i phi_j,
d(omega^2)/dM_ij = -omega^2 phi_i phi_j (phi^T M phi = 1).

Here:
  - K and M are assembled in FP64 by the library's atomic-free assembly (the
    element stiffness matrices, and the element mass matrices of
    fem_mass_matrices), condensed as the reference's assemble_matrix does;
  - the lowest eigenpairs come from LOBPCG (Knyazev, SIAM J. Sci. Comput. 23
    (2001) 517-541) in the M inner product, with the iterates kept zero on
    the constrained DOFs (the reference's free-DOF restriction), operator
    applications by the FP64 CSR block product fem_csr_spmm, and a
    preconditioner that approximates K^-1: the mixed-precision multigrid CG
    of the static solves, stopped at a loose tolerance.  Every basis block is
    M-orthogonalised against the previous ones before the Rayleigh-Ritz
    step, as in the variant of Hetmaniuk & Lehoucq (J. Comput. Phys. 218
    (2006) 324-332), so the small generalized eigenproblems stay well
    conditioned near convergence;
  - the eigenvalue gradients are the same sensitivities contracted per
    element, without forming dK or dM: phi^T (dK/d theta) phi by the element
    vector-Jacobian product (fem_element_vjp) and phi^T (dM/d theta) phi by
    the capacity vector-Jacobian product (fem_heat_mass_vjp), one pass per
    mode and component.
The small dense algebra of the Rayleigh-Ritz step (Gram matrices of a few
dozen columns and their eigendecomposition) runs through torch on the device.
"""

from __future__ import annotations

import ctypes as C

import torch
from torch import Tensor

from . import _lib
from ._lib import check, ptr


def _mass_values(dm, mesh, rho: Tensor, con_mask: Tensor):
    """Condensed FP64 CSR values of the mass matrix, and the shape-function
    values at the integration points."""
    nval = dm.etype.N(dm.etype.ipoints().to(torch.float64)).to(dm.device, torch.float64).contiguous()
    nd = dm.n_e * dm.d
    me = torch.empty(dm.n_elem * nd * nd, dtype=torch.float64, device=dm.device)
    check(dm.lib.fem_mass_matrices(C.byref(mesh), ptr(rho), ptr(nval), dm.d, ptr(me), dm.stream),
          "fem_mass_matrices")
    return dm.assemble_csr(me.view(dm.n_elem, nd, nd), con_mask), nval


class _Operator:
    """Y = A X for an assembled FP64 CSR matrix and a block X [n, m]."""

    def __init__(self, dm, val: Tensor):
        self.dm = dm
        self.val = val
        self.matrix = _lib.FemMatrix(_lib.FEM_FMT_CSR_F64, 1, dm.n_dofs, dm.n_dofs, ptr(dm.row_ptr), ptr(dm.col),
                                     ptr(val), None)

    def __call__(self, X: Tensor) -> Tensor:
        X = X.contiguous()
        Y = torch.empty_like(X)
        check(self.dm.lib.fem_csr_spmm(C.byref(self.matrix), X.shape[1], ptr(X), ptr(Y), self.dm.stream),
              "fem_csr_spmm")
        return Y


def _m_orthonormal(V: Tensor, MV: Tensor, KV: Tensor, drop: float = 1e-10):
    """Columns spanning V, M-orthonormal (eigen-whitening of the M Gram
    matrix after column scaling; directions below `drop` are dropped), with
    their M and K images."""
    scale = (V * MV).sum(0).clamp_min(0.0).sqrt()
    keep = scale > 0
    V, MV, KV, scale = V[:, keep], MV[:, keep], KV[:, keep], scale[keep]
    if V.shape[1] == 0:
        return V, MV, KV
    V, MV, KV = V / scale, MV / scale, KV / scale
    G = V.T @ MV
    G = 0.5 * (G + G.T)
    w, Q = torch.linalg.eigh(G)
    sel = w > drop * w.max()
    T = Q[:, sel] / w[sel].sqrt()
    return V @ T, MV @ T, KV @ T


def lobpcg(apply_k, apply_m, apply_t, X: Tensor, n_ev: int, tol: float, max_iter: int):
    """Lowest n_ev eigenpairs of K x = lambda M x from the start block X
    (zero on constrained DOFs, kept so by apply_t).  Returns (lambda, X, its)
    with X M-orthonormal."""
    X, MX, KX = _m_orthonormal(X, apply_m(X), apply_k(X))
    nb = X.shape[1]
    A = X.T @ KX
    lam, Y = torch.linalg.eigh(0.5 * (A + A.T))
    X, MX, KX = X @ Y, MX @ Y, KX @ Y
    P = MP = KP = None
    it = 0
    for it in range(1, max_iter + 1):
        R = KX - MX * lam
        rel = R.norm(dim=0) / KX.norm(dim=0).clamp_min(1e-300)
        if bool((rel[:n_ev] <= tol).all()):
            break
        W = apply_t(R[:, rel > 0.1 * tol])
        blocks = [(X, MX, KX)]
        for V, MV, KV in ((W, apply_m(W), apply_k(W)), (P, MP, KP)):
            if V is None or V.shape[1] == 0:
                continue
            for _ in range(2):  # twice is enough
                for B, MB, KB in blocks:
                    H = MB.T @ V
                    V, MV, KV = V - B @ H, MV - MB @ H, KV - KB @ H
            V, MV, KV = _m_orthonormal(V, MV, KV)
            if V.shape[1]:
                blocks.append((V, MV, KV))
        S = torch.cat([b[0] for b in blocks], 1)
        MS = torch.cat([b[1] for b in blocks], 1)
        KS = torch.cat([b[2] for b in blocks], 1)
        A = S.T @ KS
        lam_all, Y = torch.linalg.eigh(0.5 * (A + A.T))  # S is M-orthonormal
        Y = Y[:, :nb]
        lam = lam_all[:nb]
        Yp = Y[nb:]  # the update's part outside the old X block: the new direction
        if Yp.shape[0]:
            P, MP, KP = S[:, nb:] @ Yp, MS[:, nb:] @ Yp, KS[:, nb:] @ Yp
        X, MX, KX = S @ Y, MS @ Y, KS @ Y
    return lam, X, it


class ModalSolve(torch.autograd.Function):
    """(omega^2 [n_modes], phi [n_dofs, n_modes]) of K phi = omega^2 M phi on
    the free DOFs; gradients of omega^2 w.r.t. the material data, the
    thickness and the density (sparse.py:930-983)."""

    @staticmethod
    def forward(ctx, model, n_modes: int, mat_data: Tensor, thickness, rho: Tensor, tol: float, max_iter: int):
        from .sparse import SolveContext

        dm = model.device_mesh
        dev = dm.device
        con_bool = model.constraints.reshape(-1).to(dev).clone()
        con_mask = con_bool.to(torch.uint8).contiguous()
        n_free = int((~con_bool).sum())
        if n_modes < 1 or n_modes > n_free:
            raise ValueError(f"n_modes must lie in [1, {n_free}] (the free DOFs)")
        mat_kind, _ = model.material.kernel_data(model.n_elem)
        mixed = dm.d >= 2
        sc = SolveContext(dm, con_mask, mat_kind, "mixed" if mixed else "fp64", 1, 0.0, 0.0, 1e-2, None)
        sc.precond = "amg" if mixed else "jacobi"
        mesh, mat = sc.structs(mat_data, thickness)
        kval = dm.assemble_csr(dm.element_stiffness(mesh, mat, torch.float64), con_mask)
        mval, nval = _mass_values(dm, mesh, rho, con_mask)
        apply_k, apply_m = _Operator(dm, kval), _Operator(dm, mval)
        sysm = sc.get_system(mat_data, thickness)
        free = (~con_bool).to(torch.float64)

        def apply_t(R: Tensor) -> Tensor:
            cols = []
            for j in range(R.shape[1]):
                b = (R[:, j] * free).contiguous()
                if sysm.precision == "mixed":
                    cols.append(dm.solve(sysm, b, 1e-2, refine=False))
                else:
                    cols.append(dm.solve(sysm, b, 1e-2))
            return torch.stack(cols, 1) * free[:, None]

        nb = min(n_free, n_modes + max(2, n_modes // 2))
        gen = torch.Generator(device="cpu").manual_seed(0)
        X0 = torch.rand(dm.n_dofs, nb, generator=gen, dtype=torch.float64).to(dev) * free[:, None]
        lam, X, its = lobpcg(apply_k, apply_m, apply_t, X0, n_modes, tol, max_iter)
        R = apply_k(X[:, :n_modes]) - apply_m(X[:, :n_modes]) * lam[:n_modes]
        if its >= max_iter and not bool((R.norm(dim=0) <= tol * apply_k(X[:, :n_modes]).norm(dim=0)).all()):
            raise RuntimeError(f"LOBPCG did not converge in {max_iter} iterations")
        lam, X = lam[:n_modes].contiguous(), X[:, :n_modes].contiguous()
        model.last_modal_iterations = its
        ctx.model = model
        ctx.mesh_mat = (mesh, mat)
        ctx.nval = nval
        ctx.save_for_backward(mat_data, thickness, rho, lam, X)
        ctx.mark_non_differentiable(X)
        return lam, X

    @staticmethod
    def backward(ctx, g_lam, g_x):
        mat_data, thickness, rho, lam, X = ctx.saved_tensors
        dm = ctx.model.device_mesh
        mesh, mat = ctx.mesh_mat
        need = ctx.needs_input_grad
        want_thick = need[3] and thickness is not None
        gmat = torch.zeros_like(mat_data) if need[2] else None
        gthick = torch.zeros_like(thickness) if want_thick else None
        grho = torch.zeros(dm.n_elem, dtype=torch.float64, device=dm.device)
        if g_lam is not None:
            for k in range(lam.numel()):
                gk = float(g_lam[k])
                if gk == 0.0:
                    continue
                phi = X[:, k].contiguous()
                if need[2] or want_thick:
                    _, gm, gt, _, _ = dm.vjp(mesh, mat, phi, (gk * phi).contiguous(), want_mat=need[2],
                                             want_thick=want_thick, mat_numel=mat_data.numel())
                    if gm is not None:
                        gmat += gm.view_as(mat_data)
                    if gt is not None:
                        gthick += gt
                if need[4] or want_thick:
                    s = torch.zeros(dm.n_elem, dtype=torch.float64, device=dm.device)
                    p = torch.empty_like(s)
                    comp = phi.view(dm.n_nod, dm.d)
                    for c in range(dm.d):
                        a = comp[:, c].contiguous()
                        check(dm.lib.fem_heat_mass_vjp(C.byref(mesh), ptr(ctx.nval), ptr(a), ptr(a), ptr(p),
                                                       dm.stream), "fem_heat_mass_vjp")
                        s += p
                    grho += -gk * float(lam[k]) * s
        g_rho_out = None
        if need[4]:
            g_rho_out = grho * thickness if thickness is not None else grho
        if want_thick:
            gthick = gthick + grho * rho
        return None, None, gmat, gthick, g_rho_out, None, None
