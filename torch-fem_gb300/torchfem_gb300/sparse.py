"""Newton solve with a hand-written adjoint, on the GPU kernels.

Mirrors `newton_solve` / `NewtonRaphsonAdjoint` (src/torchfem/sparse.py:517-795)
for small-strain materials with a constant tangent (linear elasticity):

forward   Newton iterations on res(du) = F_int(du_bc; sigma_prev, de0, C, t) - F_ext,
          res[con] = 0 (base.py:704-743), each linear step solved by the GPU CG.
backward  the adjoint solve K lambda = grad_du on the same CG and
          preconditioner (sparse.py:671-680), then the residual's
          vector-Jacobian product with cotangent -lambda computed by one element
          kernel (fem_element_vjp) instead of an autograd replay of the
          assembly (sparse.py:690-705).

`IntegrateMaterial` is the converged-state evaluation (base.py:843-857):
nodal internal forces, stress and increment gradient of a displacement
increment, with its own kernel-based backward.
"""

from __future__ import annotations

import ctypes as C
import math
import warnings

import torch
from torch import Tensor

from ._device import DeviceMesh, LinearSystem
from ._lib import check, ptr


class SolveContext:
    """What one solve() call shares between its Newton steps and backward."""

    AMG_DELTA = 1e-4  # default FP64 replacement threshold of the multigrid CG

    def __init__(self, dm: DeviceMesh, con_mask: Tensor, mat_kind: int, precision: str,
                 max_iter: int, rtol: float, atol: float, stol: float, cg_max_iter: int | None,
                 delta: float = 0.1):
        self.dm = dm
        self.con_mask = con_mask  # uint8 [n_dofs] on the device
        self.con_bool = con_mask.bool()
        self.mat_kind = mat_kind
        self.precision = precision
        self.max_iter = max_iter
        self.rtol = rtol
        self.atol = atol
        self.stol = stol
        self.cg_max_iter = cg_max_iter
        self.delta = delta
        self.system: LinearSystem | None = None
        self.system_key = None
        self.iterations: list[int] = []
        self.newton_iterations: list[int] = []
        self.verbose = False
        self.inner_rtol = 1e-6
        self.linear = "cg"  # or "minres" (FP64 path)
        self.precond = "jacobi"  # or "amg" (mixed precision)
        self.precond_explicit = False  # the caller asked for this preconditioner by name
        # FP64 replacement threshold of the multigrid CG: each V-cycle cuts the
        # residual severalfold, so replacements are spaced by a deeper drop
        self.amg_delta = SolveContext.AMG_DELTA
        # set by the caller when the Newton start is known to give zero internal
        # forces (zero increment, zero previous stress, zero prescribed values)
        self.zero_start = False
        # (f_e, flux, H) of the residual evaluation at which Newton converged,
        # taken by the converged-state evaluation of the same increment
        self.converged_eval = None

    def structs(self, mat_data: Tensor, thickness: Tensor | None):
        from . import _lib

        mesh = self.dm.make_mesh(thickness)
        mat = _lib.FemMaterial(self.mat_kind, mat_data.data_ptr())
        return mesh, mat

    def build_system(self, mesh, mat, keep_refs, amg_reuse: bool = False) -> LinearSystem:
        """The device system of one tangent with this context's preconditioner.
        A multigrid hierarchy that cannot be built for this mesh (a row over its
        size caps, a coarsening that stalls, a singular coarse block) falls back
        to block Jacobi with a warning when the preconditioner was the default;
        a preconditioner asked for by name raises instead."""
        from . import _lib

        precond = self.precond if self.precision == "mixed" else "jacobi"
        try:
            return self.dm.build_system(mesh, mat, self.con_mask, self.precision, keep_refs=keep_refs,
                                        precond=precond, amg_reuse=amg_reuse and precond == "amg")
        except (_lib.FemError, ValueError) as err:
            if precond != "amg" or self.precond_explicit:
                raise
            # one DOF per node has no FP32 block-Jacobi CG: fall back to FP64
            scalar = self.dm.d == 1
            warnings.warn(f"multigrid preconditioner unavailable for this mesh ({err}); using "
                          f"{'the FP64 Jacobi CG' if scalar else 'block Jacobi'}", RuntimeWarning, stacklevel=2)
            self.precond = "jacobi"
            return self.dm.build_system(mesh, mat, self.con_mask, "fp64" if scalar else self.precision,
                                        keep_refs=keep_refs, precond="jacobi")

    def get_system(self, mat_data: Tensor, thickness: Tensor | None) -> LinearSystem:
        """The condensed tangent for these material data (built once per solve,
        as the reference keeps self.K for a constant-tangent material)."""
        key = (mat_data.data_ptr(), None if thickness is None else thickness.data_ptr())
        if self.system is None or self.system_key != key:
            mesh, mat = self.structs(mat_data, thickness)
            self.system = self.build_system(mesh, mat, keep_refs=(mat_data, thickness, mesh, mat))
            self.system_key = key
        return self.system

    def solve(self, b: Tensor, inner: bool = False) -> Tensor:
        """Linear solve on the current system.  inner=True marks a Newton
        correction of a nonlinear material, solved to max(stol, inner_rtol)
        (inexact Newton: the FP64 Newton residual, checked against rtol and
        atol, decides convergence, so the converged state is unchanged); in
        mixed precision the FP32 CG runs alone, the Newton iteration being its
        refinement.  Adjoint and linear-material solves use stol."""
        assert self.system is not None
        delta = self.amg_delta if self.system.amg is not None else self.delta
        if inner and self.precision == "mixed":
            x = self.dm.solve(self.system, b, max(self.stol, self.inner_rtol), self.cg_max_iter, refine=False)
        elif inner:
            x = self.dm.solve(self.system, b, max(self.stol, self.inner_rtol), self.cg_max_iter, delta,
                              linear=self.linear)
        else:
            x = self.dm.solve(self.system, b, self.stol, self.cg_max_iter, delta, linear=self.linear)
        self.iterations.append(self.system.stats.iterations)
        return x


def _residual(sc: SolveContext, du, F_ext, DU, sigma_prev, de0, mat_data, thickness, zero=False):
    """res = F_int(du_bc) - F_ext with res[con] = 0, and ||res||^2 (device);
    also the element forces, fluxes and increment gradients of du_bc, which
    the converged-state evaluation reuses.  zero=True: F_int is known to be
    zero (zero increment, prescribed values and previous stress, no initial
    strain), so no element pass runs."""
    if zero:
        res = torch.where(sc.con_bool, torch.zeros_like(F_ext), -F_ext).contiguous()
        return res, (res * res).sum().reshape(1), None
    mesh, mat = sc.structs(mat_data, thickness)
    fe, flux, hg = sc.dm.element_force(
        mesh, mat, du, sc.con_mask, DU, 1, sigma_prev, de0, want_flux=True, want_h=True
    )
    res, sumsq = sc.dm.gather(fe, sub=F_ext, con_mask=sc.con_mask, con_mode=1, want_norm=True)
    return res, sumsq, (fe, flux, hg)


class NewtonLinear(torch.autograd.Function):
    """Newton solve of one load (sub)step for a constant-tangent material."""

    @staticmethod
    def forward(ctx, sc: SolveContext, du, F_ext, DU, sigma_prev, de0, mat_data, thickness):
        du = du.detach().clone()
        res0 = None
        converged = False
        sc.converged_eval = None
        for i in range(sc.max_iter):
            res, sumsq, ev = _residual(sc, du, F_ext, DU, sigma_prev, de0, mat_data, thickness,
                                       zero=(i == 0 and sc.zero_start and de0 is None))
            res_norm = float(sumsq.sqrt().item())
            if i == 0:
                res0 = res_norm
            if sc.verbose:
                last = sc.system.stats if sc.system is not None else None
                cg = f" | CG {last.iterations} it, rel {last.rel_residual:.2e}" if (last and i) else ""
                print(f"  newton {i:2d}  |res| = {res_norm:.6e}{cg}")
            if res_norm < sc.rtol * res0 or res_norm < sc.atol:
                converged = True
                sc.newton_iterations.append(i)
                sc.converged_eval = ev
                break
            if res_norm != res_norm or res_norm in (float("inf"), float("-inf")):
                break
            sc.get_system(mat_data, thickness)
            du = du - sc.solve(res)
        if not converged:
            raise RuntimeError("Newton-Raphson iteration did not converge.")
        ctx.sc = sc
        ctx.save_for_backward(du, DU, sigma_prev, de0, mat_data, thickness)
        return du

    @staticmethod
    def backward(ctx, grad_du):
        sc: SolveContext = ctx.sc
        du, DU, sigma_prev, de0, mat_data, thickness = ctx.saved_tensors
        need = ctx.needs_input_grad
        g = torch.where(sc.con_bool, torch.zeros_like(grad_du), grad_du).contiguous()
        sc.get_system(mat_data, thickness)
        lam = sc.solve(g)
        gsig = gmat = gthick = gde0 = gv = None
        want_thick = need[7] and thickness is not None
        want_de0 = need[5] and de0 is not None
        if need[3] or need[4] or need[6] or want_thick or want_de0:
            # the residual's parameter pull-back (a gradient w.r.t. the loads
            # alone is lambda itself and needs no element pass)
            mesh, mat = sc.structs(mat_data, thickness)
            neg = (-lam).contiguous()
            gsig, gmat, gthick, gde0, gv = sc.dm.vjp(
                mesh, mat, du, neg, sc.con_mask, DU, 1, sigma_prev, de0,
                want_sig=need[4], want_mat=need[6], want_thick=want_thick,
                want_de0=want_de0, want_v=need[3], mat_numel=mat_data.numel(),
            )
        g_F = lam if need[2] else None
        g_DU = torch.where(sc.con_bool, gv, torch.zeros_like(gv)) if need[3] else None
        return (
            None,
            None,
            g_F,
            g_DU,
            None if gsig is None else gsig.view_as(sigma_prev),
            None if gde0 is None else gde0.view_as(de0),
            None if gmat is None else gmat.view_as(mat_data),
            gthick,
        )


class IntegrateMaterial(torch.autograd.Function):
    """Converged-state evaluation: (F_int, flux, H_inc) of an increment."""

    @staticmethod
    def forward(ctx, sc: SolveContext, du_eval, sigma_prev, de0, mat_data, thickness):
        mesh, mat = sc.structs(mat_data, thickness)
        dm = sc.dm
        cached, sc.converged_eval = sc.converged_eval, None
        if cached is not None:
            # the Newton iteration's last residual was evaluated at this same
            # displacement (du with the prescribed values on constrained DOFs)
            fe, flux, hg = cached
        else:
            fe, flux, hg = dm.element_force(
                mesh, mat, du_eval, None, None, 0, sigma_prev, de0, want_flux=True, want_h=True
            )
        f_int, _ = dm.gather(fe)
        shape = (dm.nip, dm.n_elem, *dm.flux_shape)
        ctx.sc = sc
        ctx.save_for_backward(du_eval, sigma_prev, de0, mat_data, thickness)
        return f_int, flux.view(shape), hg.view(shape)

    @staticmethod
    def backward(ctx, g_f, g_flux, g_h):
        sc: SolveContext = ctx.sc
        du_eval, sigma_prev, de0, mat_data, thickness = ctx.saved_tensors
        need = ctx.needs_input_grad
        mesh, mat = sc.structs(mat_data, thickness)
        gsig, gmat, gthick, gde0, gv = sc.dm.vjp(
            mesh, mat, du_eval, None if g_f is None else g_f.contiguous(), None, None, 0,
            sigma_prev, de0,
            gflux=None if g_flux is None else g_flux.contiguous(),
            gh=None if g_h is None else g_h.contiguous(),
            want_sig=need[2], want_mat=need[4], want_thick=need[5] and thickness is not None,
            want_de0=need[3] and de0 is not None, want_v=need[1], mat_numel=mat_data.numel(),
        )
        return (
            None,
            gv,
            None if gsig is None else gsig.view_as(sigma_prev),
            None if gde0 is None else gde0.view_as(de0),
            None if gmat is None else gmat.view_as(mat_data),
            gthick,
        )


class TransientContext:
    """What one time_integration() call shares between its Crank-Nicolson
    steps and their backward: the assembled capacity and conductivity values,
    the step systems M + dt/2 K (one per distinct dt, FP64 Jacobi CG) and the
    Newton controls."""

    def __init__(self, dm: DeviceMesh, con_mask: Tensor, mat_kind: int, mval: Tensor, kval: Tensor,
                 max_iter: int, rtol: float, atol: float, stol: float, verbose: bool):
        self.dm = dm
        self.con_mask = con_mask
        self.con_bool = con_mask.bool()
        self.mat_kind = mat_kind
        self.mval = mval
        self.kval = kval
        self.mass = dm.csr_system(mval, con_mask)
        self.systems: dict[float, LinearSystem] = {}
        self.max_iter = max_iter
        self.rtol = rtol
        self.atol = atol
        self.stol = stol
        self.verbose = verbose
        self.iterations: list[int] = []
        self.nval = dm.etype.N(dm.etype.ipoints().to(torch.float64)).to(dm.device, torch.float64).contiguous()

    def system(self, dt: float) -> LinearSystem:
        sysm = self.systems.get(dt)
        if sysm is None:
            sysm = self.dm.csr_system(self.dm.csr_combine(1.0, self.mval, 0.5 * dt, self.kval), self.con_mask)
            self.systems[dt] = sysm
        return sysm

    def structs(self, mat_data: Tensor, thickness: Tensor | None):
        from . import _lib

        mesh = self.dm.make_mesh(thickness)
        return mesh, _lib.FemMaterial(self.mat_kind, mat_data.data_ptr())


class CrankNicolsonStep(torch.autograd.Function):
    """One Crank-Nicolson time step of Heat.time_integration
    (src/torchfem/base.py:1420-1530): Newton iterations on

        r(du) = M du + dt/2 (f_old + f_int(du; flux_prev, kappa, t) + f_ext),
        r = 0 on constrained DOFs,

    each correction (M + dt/2 K) x = -r solved by the FP64 CG; returns du.

    backward is the reference's NewtonRaphsonAdjoint at the converged step
    (sparse.py:641-724) written out for this residual: the adjoint solve
    (M + dt/2 K) lambda = grad_du on the free DOFs on the same CG, then the
    residual's vector-Jacobian product with cotangent c = -lambda:
    dt/2 c to f_old and f_ext, the heat-force vjp kernel with cotangent
    dt/2 c to flux_prev, the conductivity and the thickness, and the capacity
    vjp kernel (fem_heat_mass_vjp) c^T (dM/d theta) du to the density and the
    thickness."""

    @staticmethod
    def forward(ctx, tc: TransientContext, dt: float, f_old, flux_prev, f_ext, mat_data, thickness, rho):
        dm = tc.dm
        mesh, mat = tc.structs(mat_data, thickness)
        half = 0.5 * dt
        du = torch.zeros(dm.n_dofs, dtype=torch.float64, device=dm.device)
        res0 = None
        converged = False
        for it in range(tc.max_iter):
            fe, _, _ = dm.element_force(mesh, mat, du, None, None, 0, flux_prev, None)
            f_int, _ = dm.gather(fe)
            res, sumsq = dm.cn_residual(tc.mass, du, f_old, f_int, f_ext, half, tc.con_mask)
            res_norm = math.sqrt(float(sumsq.item()))
            if it == 0:
                res0 = res_norm
            if tc.verbose:
                print(f"  newton {it:2d}  |res| = {res_norm:.6e}")
            if res_norm < tc.rtol * res0 or res_norm < tc.atol:
                converged = True
                break
            sysm = tc.system(dt)
            du = du + dm.solve(sysm, (-res).contiguous(), tc.stol)
            tc.iterations.append(sysm.stats.iterations)
        if not converged:
            raise RuntimeError("Newton-Raphson iteration did not converge.")
        ctx.tc = tc
        ctx.dt = dt
        ctx.save_for_backward(du, flux_prev, mat_data, thickness, rho)
        return du

    @staticmethod
    def backward(ctx, grad_du):
        tc: TransientContext = ctx.tc
        dm = tc.dm
        du, flux_prev, mat_data, thickness, rho = ctx.saved_tensors
        need = ctx.needs_input_grad
        half = 0.5 * ctx.dt
        g = torch.where(tc.con_bool, torch.zeros_like(grad_du), grad_du).contiguous()
        sysm = tc.system(ctx.dt)
        lam = dm.solve(sysm, g, tc.stol)
        tc.iterations.append(sysm.stats.iterations)
        c = (-lam).contiguous()
        ch = (half * c).contiguous()
        mesh, mat = tc.structs(mat_data, thickness)
        want_thick = need[6] and thickness is not None
        gsig = gmat = gthick = None
        if need[3] or need[5] or want_thick:
            gsig, gmat, gthick, _, _ = dm.vjp(
                mesh, mat, du, ch, None, None, 0, flux_prev, None,
                want_sig=need[3], want_mat=need[5], want_thick=want_thick, mat_numel=mat_data.numel(),
            )
        g_rho = None
        if need[7] or want_thick:
            p = torch.empty(dm.n_elem, dtype=torch.float64, device=dm.device)
            check(dm.lib.fem_heat_mass_vjp(C.byref(mesh), ptr(tc.nval), ptr(c), ptr(du), ptr(p), dm.stream),
                  "fem_heat_mass_vjp")
            if need[7]:
                g_rho = p * thickness if thickness is not None else p
            if want_thick:
                gthick = gthick + p * rho
        return (
            None,
            None,
            ch if need[2] else None,
            None if gsig is None else gsig.view_as(flux_prev),
            ch if need[4] else None,
            None if gmat is None else gmat.view_as(mat_data),
            gthick,
            g_rho,
        )
