"""Flat-facet triangular shell (src/torchfem/shell.py) on the GPU kernels.

`Shell(nodes, elements, material, thickness, transverse_nu, transverse_kappa,
transverse_G, drill_penalty, n_simpson, orientation)` keeps the reference's
constructor (shell.py:48-177) for a homogeneous plane-stress section, and
`solve(...)` its signature and results: u and f with six components per node,
the station stresses (n_simpson per element, mean over them unless
`aggregate_integration_points=False`), the unchanged in-plane identity as the
deformation gradient, and an empty state.

The element matrices, forces, station stresses and the parameter
vector-Jacobian product are CUDA kernels (`fem_shell_*` in the C ABI); the
assembled FP64 matrix and the Jacobi CG are the solid path's.  The Newton loop
per load increment and the adjoint mirror `NewtonRaphsonAdjoint`
(sparse.py:517-795): forward Newton on res = f(u_prev + du) - F_ext with
res[con] = 0; backward K lambda = dL/ddu, then the residual's vjp with -lambda.
Layered (`Laminate`) sections, geometric nonlinearity and inelastic materials
are not part of this path.
"""

from __future__ import annotations

import ctypes as C
import math
from collections.abc import Iterable

import torch
from torch import Tensor

from . import _lib
from ._device import DeviceMesh
from ._lib import check, ptr
from .base import Mechanics, resolve_precision
from .elements import Tria1
from .materials import Material


class ShellTria1(Tria1):
    """Tria1 carrying six DOFs per node (the gather uses FEM_SHELL3)."""

    etype_id = _lib.FEM_SHELL3


def _voigt(C4: Tensor) -> Tensor:
    """[..., 3, 3] Voigt form of a 2D tangent, pairs (00, 11, 01) (utils.py:47-50)."""
    pairs = ((0, 0), (1, 1), (0, 1))
    return torch.stack([torch.stack([C4[..., i, j, k, l] for (k, l) in pairs], -1) for (i, j) in pairs], -2)


class Shell(Mechanics):
    """Tria1 flat-facet shell with a homogeneous plane-stress section."""

    def __init__(self, nodes: Tensor, elements: Tensor, material, thickness: Tensor | float = 1.0,
                 transverse_nu: float = 0.5, transverse_kappa: float = 5.0 / 6.0,
                 transverse_G=None, drill_penalty: float = 1.0, n_simpson: int = 3,
                 orientation: Tensor | None = None):
        if not isinstance(material, Material):
            raise NotImplementedError("layered (Laminate) shell sections are not implemented on the GPU path")
        super().__init__(nodes, elements, material)
        if orientation is None:
            orientation = torch.tensor([1.0, 0.0, 0.0])
        orientation = torch.as_tensor(orientation, dtype=self.nodes.dtype)
        if orientation.dim() == 1:
            orientation = orientation.unsqueeze(0).expand(self.n_elem, 3)
        self.orientation = orientation
        self.drill_penalty = drill_penalty
        self.transverse_nu = transverse_nu
        self.transverse_kappa = transverse_kappa
        if isinstance(thickness, float):
            self.thickness = torch.full((self.n_elem,), thickness)
        else:
            self.thickness = torch.as_tensor(thickness)
        if n_simpson % 2 == 0:
            raise ValueError("n_simpson must be an odd integer.")
        self.n_simpson = n_simpson
        self.n_z = n_simpson
        self.z_simpson = torch.linspace(-0.5, 0.5, n_simpson)
        self.w_simpson = torch.ones(n_simpson)
        self.w_simpson[1:-1:2] = 4.0
        self.w_simpson[2:-2:2] = 2.0
        self.w_simpson *= 1.0 / (n_simpson - 1) / 3.0
        if transverse_G is None:
            if hasattr(self.material, "G"):
                G = 2 * [self.material.G]
            elif hasattr(self.material, "G_13") and hasattr(self.material, "G_23"):
                G = [self.material.G_13, self.material.G_23]
            else:
                raise ValueError("Material must have shear modulus 'G' defined or transverse_G must be provided.")
            G = [torch.as_tensor(g).expand(self.n_elem) if torch.as_tensor(g).dim() == 0 else torch.as_tensor(g)
                 for g in G]
        else:
            G = [torch.as_tensor(transverse_G[0]).repeat(self.n_elem),
                 torch.as_tensor(transverse_G[1]).repeat(self.n_elem)]
        self._shear_G = G
        z = torch.zeros(self.n_elem)
        Cs = torch.stack([torch.stack([G[0], z], dim=-1), torch.stack([z, G[1]], dim=-1)], dim=-1)
        self.As = self.thickness[:, None, None] * Cs
        self.n_int = self.n_int * self.n_z

    def __repr__(self) -> str:
        return f"<torch-fem shell ({self.n_nod} nodes, {self.n_elem} Tria1 elements)>"

    @property
    def n_dof_per_node(self) -> int:
        return 6

    @property
    def n_flux(self) -> list[int]:
        return [2, 2]

    @property
    def etype(self):
        return ShellTria1

    @property
    def volume_scale(self) -> Tensor:
        return self.thickness

    @property
    def device_mesh(self) -> DeviceMesh:
        if self._dm is None:
            self._dm = DeviceMesh(self.nodes, self.elements, ShellTria1, 6, geometry=False)
        return self._dm

    def kernel_data(self) -> Tensor:
        """[n_elem, 11]: Voigt plane-stress tangent (row-major) and the two
        transverse shear moduli, differentiable in the material's tensors."""
        assert self.material is not None
        if self.material.n_state != 0:
            raise NotImplementedError("shells with inelastic materials are not implemented on the GPU path")
        Cv = _voigt(self.material.C).reshape(-1, 9)
        if Cv.shape[0] != self.n_elem:
            Cv = Cv.expand(self.n_elem, 9)
        G = torch.stack([g.to(Cv.dtype) for g in self._shear_G], dim=-1)
        return torch.cat([Cv, G], dim=-1)

    # -------------------------------------------------------------- solve --
    def solve(self, increments: Tensor | None = None, max_iter: int = 10, rtol: float = 1e-8,
              atol: float = 1e-6, stol: float = 1e-10, cutback_factor: float = 0.5,
              growth_factor: float = 1.1, max_cutbacks: int = 10, verbose: bool = False,
              method: str | None = None, device: str | None = None, return_intermediate: bool = False,
              aggregate_integration_points: bool = True, use_cached_solve: bool = False,
              nlgeom: bool = False, alpha: float = 0.0,
              differentiable_parameters: Tensor | Iterable[Tensor] | None = None,
              precision: str | None = None, cg_max_iter: int | None = None):
        """Quasi-static solve by load increments (base.py:597-923 with the
        shell's integrate_material, shell.py:416-603)."""
        prec = resolve_precision(method, precision)
        if prec != "fp64":
            raise NotImplementedError("shells solve in FP64 (no 6 x 6 block layout on the mixed path)")
        if nlgeom:
            raise NotImplementedError("Geometric nonlinearity is not yet implemented for shells.")
        if alpha > 0.0:
            raise NotImplementedError("viscous stabilization (alpha > 0) is not implemented")
        if device is not None and torch.device(device).type != "cuda":
            raise RuntimeError("torchfem_gb300 solves on a CUDA device only")
        increments = torch.tensor([0.0, 1.0]) if increments is None else increments
        N = len(increments)
        if differentiable_parameters is None:
            differentiable_parameters = ()
        elif isinstance(differentiable_parameters, torch.Tensor):
            differentiable_parameters = (differentiable_parameters,)
        else:
            differentiable_parameters = tuple(differentiable_parameters)
        track = any(p.requires_grad for p in differentiable_parameters)

        dm = self.device_mesh
        dev = dm.device
        con_bool = self._constraints.reshape(-1).to(dev)
        sc = ShellContext(self, dm, con_bool, max_iter, rtol, atol, stol, cg_max_iter)
        sc.verbose = verbose
        sc.linear = "minres" if method == "minres" else "cg"
        self.last_solve = sc
        with torch.set_grad_enabled(track):
            mat = self.kernel_data().to(dev, torch.float64).contiguous()
            thick = self.thickness.expand(self.n_elem).to(dev, torch.float64).contiguous()
            F_neu = self._neumann.reshape(-1).to(dev, torch.float64)
            DU_dir = self._dirichlet.reshape(-1).to(dev, torch.float64)

        n_ip = self.n_int
        u_cur = torch.zeros(self.n_dofs, dtype=torch.float64, device=dev)
        f_cur = torch.zeros(self.n_dofs, dtype=torch.float64, device=dev)
        flux_cur = torch.zeros(n_ip, self.n_elem, 2, 2, dtype=torch.float64, device=dev)
        grad_cur = torch.eye(2, dtype=torch.float64, device=dev).expand(n_ip, self.n_elem, 2, 2).clone()
        state_cur = torch.zeros(n_ip, self.n_elem, self.n_state, dtype=torch.float64, device=dev)
        outs = [(u_cur, f_cur, flux_cur, grad_cur, state_cur)]
        lam = float(increments[0])
        step_frac = 1.0
        with torch.set_grad_enabled(track):
            for n in range(1, N):
                target = float(increments[n])
                span = target - lam
                direction = math.copysign(1.0, span)
                step_size = step_frac * abs(span)
                min_step = abs(span) * cutback_factor**max_cutbacks
                while abs(target - lam) > 1e-12 * max(1.0, abs(target)):
                    step = direction * min(step_size, abs(target - lam))
                    if verbose:
                        print(f"increment {n}: load {lam + step:.6g}")
                    F_ext = ((lam + step) * F_neu).contiguous()
                    DU = (step * DU_dir).contiguous()
                    u_prev = u_cur if track else u_cur.detach()
                    try:
                        du = NewtonShell.apply(sc, u_prev.contiguous(), F_ext, DU, mat, thick)
                    except RuntimeError as err:
                        if verbose:
                            print(f"  cutback: {err}")
                        if isinstance(err, _lib.FemError) and err.code not in (
                            _lib.FEM_NOT_CONVERGED, _lib.FEM_NONFINITE, _lib.FEM_BREAKDOWN
                        ):
                            raise
                        step_size = cutback_factor * abs(step)
                        if step_size < min_step:
                            raise RuntimeError(
                                f"Newton-Raphson did not converge in increment {n} after {max_cutbacks} cutbacks."
                            ) from err
                        continue
                    du_eval = torch.where(con_bool, DU, du)
                    u_cur = u_prev + du_eval
                    f_cur, flux_cur = IntegrateShell.apply(sc, u_cur.contiguous(), mat, thick)
                    lam += step
                    step_size = min(growth_factor * step_size, abs(span))
                step_frac = min(step_size / abs(span), 1.0) if span != 0.0 else 1.0
                outs.append((u_cur, f_cur, flux_cur, grad_cur, state_cur))

            u = torch.stack([o[0] for o in outs]).reshape(N, self.n_nod, 6)
            f = torch.stack([o[1] for o in outs]).reshape(N, self.n_nod, 6)
            flux = torch.stack([o[2] for o in outs])
            grad = torch.stack([o[3] for o in outs])
            state = torch.stack([o[4] for o in outs])
            if aggregate_integration_points:
                flux, grad, state = flux.mean(dim=1), grad.mean(dim=1), state.mean(dim=1)
            if not track:
                u, f, flux, grad, state = (t.detach() for t in (u, f, flux, grad, state))
            out_dev, dt = self.nodes.device, self.nodes.dtype
            u, f, flux, grad, state = (t.to(out_dev, dt) for t in (u, f, flux, grad, state))
        if return_intermediate:
            return u, f, flux, grad, state
        return u[-1], f[-1], flux[-1], grad[-1], state[-1]


class ShellContext:
    """Device descriptors, element matrices and the assembled system of one
    shell solve (built once per material / thickness tensors)."""

    def __init__(self, model: Shell, dm: DeviceMesh, con_bool: Tensor, max_iter: int, rtol: float,
                 atol: float, stol: float, cg_max_iter: int | None):
        self.dm = dm
        dev = dm.device
        self.con_bool = con_bool
        self.con_mask = con_bool.to(torch.uint8).contiguous()
        self.max_iter, self.rtol, self.atol, self.stol = max_iter, rtol, atol, stol
        self.cg_max_iter = cg_max_iter
        self.verbose = False
        self.linear = "cg"
        self.n_z = model.n_z
        self.z = model.z_simpson.to(dev, torch.float64).contiguous()
        self.w = model.w_simpson.to(dev, torch.float64).contiguous()
        self.orientation = model.orientation.to(dev, torch.float64).contiguous()
        self.kappa = float(model.transverse_kappa)
        self.nu_t = float(model.transverse_nu)
        self.drill = float(model.drill_penalty)
        self.key = None
        self.ke: Tensor | None = None
        self.system = None
        self.iterations: list[int] = []
        self.newton_iterations: list[int] = []

    def desc(self, thickness: Tensor) -> _lib.FemShell:
        dm = self.dm
        return _lib.FemShell(
            dm.n_nod, dm.n_elem, ptr(dm.nodes), ptr(dm.elements), ptr(self.orientation), ptr(thickness),
            self.n_z, ptr(self.z), ptr(self.w), self.kappa, self.nu_t, self.drill,
        )

    def prepare(self, mat: Tensor, thickness: Tensor) -> None:
        """Element matrices and the condensed FP64 system for these data."""
        key = (mat.data_ptr(), mat._version, thickness.data_ptr(), thickness._version)
        if self.key == key:
            return
        dm, L = self.dm, self.dm.lib
        self.ke = dm._empty(dm.n_elem * 324, torch.float64)
        check(L.fem_shell_stiffness(C.byref(self.desc(thickness)), ptr(mat), ptr(self.ke), ptr(dm.status),
                                    dm.stream), "fem_shell_stiffness")
        dm.check_status("shell stiffness")
        from ._device import LinearSystem

        sysm = LinearSystem(dm, "fp64")
        sysm.val = dm.assemble_csr(self.ke.view(dm.n_elem, 18, 18), self.con_mask)
        sysm.precond = dm._empty(dm.n_dofs, torch.float64)
        check(L.fem_jacobi(ptr(sysm.val), ptr(dm.diag_map), dm.n_dofs, ptr(sysm.precond), ptr(dm.status),
                           dm.stream), "fem_jacobi")
        sysm.matrix = _lib.FemMatrix(_lib.FEM_FMT_CSR_F64, 1, dm.n_dofs, dm.n_dofs, ptr(dm.row_ptr), ptr(dm.col),
                                     ptr(sysm.val), ptr(sysm.precond))
        sysm.con_mask = self.con_mask
        sysm.ws = dm._ws(L.fem_pcg_workspace_bytes(C.byref(sysm.matrix)))
        dm.check_status("shell assembly")
        self.system = sysm
        self.key = key
        self._refs = (mat, thickness)

    def forces(self, u: Tensor, mat: Tensor, thickness: Tensor, want_stress: bool = False):
        """Assembled element forces K_e u_e (all DOFs) and the station stresses."""
        dm = self.dm
        fe = dm._empty(dm.n_elem * 18, torch.float64)
        stress = dm._empty(self.n_z * dm.n_elem * 4, torch.float64) if want_stress else None
        check(dm.lib.fem_shell_force(C.byref(self.desc(thickness)), ptr(mat), ptr(self.ke), ptr(u), ptr(fe),
                                     ptr(stress), dm.stream), "fem_shell_force")
        f, _ = dm.gather(fe)
        return f, (None if stress is None else stress.view(self.n_z, dm.n_elem, 2, 2))

    def vjp(self, u: Tensor, a: Tensor | None, gstress: Tensor | None, mat: Tensor, thickness: Tensor,
            want_mat: bool, want_thick: bool, want_u: bool):
        dm = self.dm
        gmat = dm._empty(dm.n_elem * 11, torch.float64) if want_mat else None
        gthick = dm._empty(dm.n_elem, torch.float64) if want_thick else None
        gue = dm._empty(dm.n_elem * 18, torch.float64) if (want_u and gstress is not None) else None
        check(dm.lib.fem_shell_vjp(C.byref(self.desc(thickness)), ptr(mat), ptr(u), ptr(a), ptr(gstress),
                                   ptr(gmat), ptr(gthick), ptr(gue), dm.stream), "fem_shell_vjp")
        gu = None
        if want_u:
            gu = torch.zeros(dm.n_dofs, dtype=torch.float64, device=dm.device)
            if a is not None:
                gu = gu + self.forces(a, mat, thickness)[0]
            if gue is not None:
                gu = gu + dm.gather(gue)[0]
        return (None if gmat is None else gmat.view(dm.n_elem, 11)), gthick, gu

    def solve(self, b: Tensor) -> Tensor:
        x = self.dm.solve(self.system, b, self.stol, self.cg_max_iter, linear=self.linear)
        self.iterations.append(self.system.stats.iterations)
        return x


class NewtonShell(torch.autograd.Function):
    """Newton solve of one load (sub)step of the linear-elastic shell."""

    @staticmethod
    def forward(ctx, sc: ShellContext, u_prev, F_ext, DU, mat, thickness):
        sc.prepare(mat, thickness)
        du = torch.zeros_like(u_prev)
        res0 = None
        converged = False
        for i in range(sc.max_iter):
            u_trial = u_prev + torch.where(sc.con_bool, DU, du)
            f_int, _ = sc.forces(u_trial.contiguous(), mat, thickness)
            res = torch.where(sc.con_bool, torch.zeros_like(f_int), f_int - F_ext)
            res_norm = float(res.norm())
            if i == 0:
                res0 = res_norm
            if sc.verbose:
                print(f"  newton {i:2d}  |res| = {res_norm:.6e}")
            if res_norm < sc.rtol * res0 or res_norm < sc.atol:
                converged = True
                sc.newton_iterations.append(i)
                break
            if not math.isfinite(res_norm):
                break
            du = du - sc.solve(res.contiguous())
        if not converged:
            raise RuntimeError("Newton-Raphson iteration did not converge.")
        ctx.sc = sc
        ctx.save_for_backward(u_prev, du, DU, mat, thickness)
        return du

    @staticmethod
    def backward(ctx, grad_du):
        sc: ShellContext = ctx.sc
        u_prev, du, DU, mat, thickness = ctx.saved_tensors
        need = ctx.needs_input_grad
        sc.prepare(mat, thickness)
        g = torch.where(sc.con_bool, torch.zeros_like(grad_du), grad_du).contiguous()
        lam = sc.solve(g)
        u_trial = (u_prev + torch.where(sc.con_bool, DU, du)).contiguous()
        neg = (-lam).contiguous()
        gmat, gthick, gu = sc.vjp(u_trial, neg, None, mat, thickness, want_mat=need[4], want_thick=need[5],
                                  want_u=need[1] or need[3])
        g_DU = torch.where(sc.con_bool, gu, torch.zeros_like(gu)) if need[3] else None
        return None, (gu if need[1] else None), (lam if need[2] else None), g_DU, gmat, gthick


class IntegrateShell(torch.autograd.Function):
    """Converged-state evaluation: assembled forces and station stresses."""

    @staticmethod
    def forward(ctx, sc: ShellContext, u, mat, thickness):
        sc.prepare(mat, thickness)
        f, stress = sc.forces(u, mat, thickness, want_stress=True)
        ctx.sc = sc
        ctx.save_for_backward(u, mat, thickness)
        return f, stress

    @staticmethod
    def backward(ctx, g_f, g_stress):
        sc: ShellContext = ctx.sc
        u, mat, thickness = ctx.saved_tensors
        need = ctx.needs_input_grad
        sc.prepare(mat, thickness)
        gmat, gthick, gu = sc.vjp(
            u, None if g_f is None else g_f.contiguous(), None if g_stress is None else g_stress.contiguous(),
            mat, thickness, want_mat=need[2], want_thick=need[3], want_u=need[1],
        )
        return None, gu, gmat, gthick
