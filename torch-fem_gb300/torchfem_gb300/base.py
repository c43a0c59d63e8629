"""Finite-element model base classes with the reference's API
(src/torchfem/base.py:23-1092): constructor, load/BC attributes with the same
validation, and `solve(...)` with the reference signature.  The compute
behind `solve` runs on the GPU through the C ABI; there is no CPU path.
"""

from __future__ import annotations

import math
from collections.abc import Iterable

import torch
from torch import Tensor

from . import _lib
from ._device import DeviceMesh
from .elements import Element
from .materials import Material
from ._nonlinear import IntegrateNonlinear, NewtonNonlinear, NLContext
from .sparse import CrankNicolsonStep, IntegrateMaterial, NewtonLinear, SolveContext, TransientContext

_REFERENCE_METHODS = ("spsolve", "minres", "cg", "pardiso", "amgx")
_GPU_METHODS = {None: "fp64", "cg": "fp64", "gb300": "fp64", "gb300-mixed": "mixed"}
_PRECONDITIONERS = ("jacobi", "amg")


def resolve_preconditioner(preconditioner: str | None, precision: str, n_dof_per_node: int) -> str:
    """'jacobi' (block Jacobi in mixed precision, Jacobi in FP64) or 'amg'
    (smoothed-aggregation multigrid, the counterpart of the reference's
    default pyamg / AmgX preconditioners; mixed precision, 1, 2 or 3 DOFs per
    node).  None picks the default: TORCHFEM_GB300_PRECOND if set, else 'amg'
    where it applies and 'jacobi' elsewhere (FP64, shells)."""
    import os

    p = preconditioner if preconditioner is not None else os.environ.get("TORCHFEM_GB300_PRECOND", "amg")
    if p not in _PRECONDITIONERS:
        raise ValueError(f"preconditioner must be one of {_PRECONDITIONERS}")
    if p == "amg" and (precision != "mixed" or n_dof_per_node not in (1, 2, 3)):
        if preconditioner is not None:
            raise ValueError("the multigrid preconditioner runs with precision 'mixed' on 1, 2 or 3 DOFs per node")
        p = "jacobi"
    if precision == "mixed" and n_dof_per_node == 1 and p != "amg":
        raise NotImplementedError("mixed precision with one DOF per node runs with the multigrid preconditioner")
    return p


def resolve_precision(method: str | None, precision: str | None) -> str:
    """Maps `method` / `precision` to the solver variant.

    "cg" (and None) is the Jacobi-preconditioned CG of the reference's CUDA
    branch in FP64, "minres" its Jacobi-preconditioned MINRES (FP64);
    "gb300-mixed" or precision="mixed" selects FP32 storage and CG inside
    FP64 residual replacement.  The reference's direct and third-party
    backends are not part of this library.
    """
    if method is not None and method not in _REFERENCE_METHODS and method not in _GPU_METHODS:
        raise ValueError(
            f"Method {method} is not supported. Choose from 'cg', 'gb300' or 'gb300-mixed'."
        )
    if method in ("spsolve", "pardiso", "amgx"):
        raise RuntimeError(
            f"Method '{method}' is a CPU/third-party backend of torch-fem; torchfem_gb300 "
            "solves with its own GPU Krylov methods ('cg', 'minres', 'gb300', 'gb300-mixed')."
        )
    if method == "minres":
        if precision not in (None, "fp64"):
            raise ValueError("method 'minres' runs in FP64")
        return "fp64"
    p = _GPU_METHODS[method]
    if precision is not None:
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        p = precision
    return p


class FEM:
    """Abstract finite-element model (base.py:23-132)."""

    etype: type[Element]

    def __init__(self, nodes: Tensor, elements: Tensor, material: Material | None):
        self.nodes = nodes
        self.elements = elements
        self.n_dofs = self.n_dof_per_node * nodes.shape[0]
        self.n_nod = nodes.shape[0]
        self.n_dim = nodes.shape[1]
        self.n_elem = len(self.elements)
        self.n_int = len(self.etype.iweights())
        dev, dt = nodes.device, nodes.dtype
        self._neumann = torch.zeros(self.n_nod, self.n_dof_per_node, dtype=dt, device=dev)
        self._dirichlet = torch.zeros(self.n_nod, self.n_dof_per_node, dtype=dt, device=dev)
        self._constraints = torch.zeros(self.n_nod, self.n_dof_per_node, dtype=torch.bool, device=dev)
        self._external_gradient = torch.zeros(self.n_elem, *self.n_flux, dtype=dt, device=dev)
        # an external strain that was never set is zero: the kernels then skip it
        self._external_gradient_set = False
        idx = (self.n_dof_per_node * self.elements).unsqueeze(-1) + torch.arange(
            self.n_dof_per_node, device=elements.device
        )
        self.idx = idx.reshape(self.n_elem, -1).to(torch.int32)
        if material is None or material.is_vectorized:
            self.material = material
        else:
            self.material = material.vectorize(self.n_elem)
        self._dm: DeviceMesh | None = None
        self.last_solve: SolveContext | None = None

    # ---------------------------------------------------------- interface --
    @property
    def n_dof_per_node(self) -> int:
        raise NotImplementedError

    @property
    def n_flux(self) -> list[int]:
        raise NotImplementedError

    @property
    def initial_grad(self) -> Tensor:
        raise NotImplementedError

    @property
    def n_state(self) -> int:
        assert self.material is not None
        return self.material.n_state

    @property
    def volume_scale(self) -> Tensor:
        return torch.ones(self.n_elem, device=self.nodes.device)

    def _thickness(self) -> Tensor | None:
        return None

    # ------------------------------------------------------- device state --
    @property
    def device_mesh(self) -> DeviceMesh:
        """Pattern and geometry on the GPU, built on first use."""
        if self._dm is None:
            self._dm = DeviceMesh(self.nodes, self.elements, self.etype, self.n_dof_per_node)
        return self._dm

    @property
    def k_map(self) -> Tensor:
        """Slot of every element-matrix entry (base.py:93-104), int32."""
        return self.device_mesh.kmap().to(torch.int32)

    @property
    def glob_idx(self) -> Tensor:
        """(row, col) of every stored entry, int64 [2, nnz] (base.py:112-117)."""
        return self.device_mesh.glob_idx()

    @property
    def diag_map(self) -> Tensor:
        """Slot of each diagonal entry, int32 (base.py:106-108)."""
        return self.device_mesh.diag_map.to(torch.int32)

    # ------------------------------------------------------------ setters --
    @property
    def constraints(self) -> Tensor:
        return self._constraints

    @constraints.setter
    def constraints(self, value: Tensor):
        if not value.shape == (self.n_nod, self.n_dof_per_node):
            raise ValueError("Constraints must have the same shape as nodes.")
        if value.dtype != torch.bool:
            raise TypeError("Constraints must be a boolean tensor.")
        self._constraints = value.to(self.nodes.device)

    # ---------------------------------------------------- element matrices --
    def _device_material(self):
        """(mesh struct, material struct, keep-alive refs) on the device."""
        dm = self.device_mesh
        assert self.material is not None
        kind, data = self.material.kernel_data(self.n_elem)
        if isinstance(kind, str):
            raise NotImplementedError(f"{type(self.material).__name__} has a state-dependent tangent")
        data = data.detach().to(dm.device, torch.float64).contiguous()
        thickness = self._thickness()
        if thickness is not None:
            thickness = thickness.detach().to(dm.device, torch.float64).contiguous()
        mesh = dm.make_mesh(thickness)
        return mesh, _lib.FemMaterial(kind, data.data_ptr()), (data, thickness)

    def k0(self) -> Tensor:
        """Element stiffness (mechanics) or conductivity (heat) matrices of the
        reference state, [n_elem, n_dof_elem, n_dof_elem] (base.py:228-245),
        for materials with a constant tangent."""
        mesh, mat, refs = self._device_material()
        ke = self.device_mesh.element_stiffness(mesh, mat, torch.float64)
        del refs
        return ke.to(self.nodes.device, self.nodes.dtype)

    def solve_modes(self, n_modes: int, tol: float = 1e-10, max_iter: int = 500) -> tuple[Tensor, Tensor]:
        """Natural frequencies and mode shapes (base.py:1097-1129): the
        n_modes lowest eigenpairs of K phi = omega^2 M phi on the free DOFs.

        Returns (omega_sq [n_modes], differentiable w.r.t. the material
        parameters, the density and the thickness; modes [n_modes, n_nod,
        n_dof_per_node], detached, M-normalised), like the reference.  The
        eigenpairs come from LOBPCG on the GPU (torchfem_gb300.modal) instead
        of shift-invert eigsh; `tol` is the relative eigen-residual
        ||K phi - omega^2 M phi|| / ||K phi|| at which a mode has converged.
        """
        from .modal import ModalSolve

        dm = self.device_mesh
        dev = dm.device
        assert self.material is not None
        kind, mat_data = self.material.kernel_data(self.n_elem)
        if isinstance(kind, str):
            raise NotImplementedError(f"{type(self.material).__name__} has a state-dependent tangent")
        mat_data = mat_data.to(dev, torch.float64).contiguous()
        thickness = self._thickness()
        if thickness is not None:
            thickness = thickness.to(dev, torch.float64).contiguous()
        rho = torch.as_tensor(self.material.rho).to(dev, torch.float64).expand(self.n_elem).contiguous()
        omega_sq, phi = ModalSolve.apply(self, int(n_modes), mat_data, thickness, rho, tol, max_iter)
        modes = phi.T.reshape(n_modes, self.n_nod, self.n_dof_per_node)
        out = self.nodes.device
        return omega_sq.to(out, self.nodes.dtype), modes.detach().to(out, self.nodes.dtype)

    # -------------------------------------------------------------- solve --
    def solve(
        self,
        increments: Tensor | None = None,
        max_iter: int = 10,
        rtol: float = 1e-8,
        atol: float = 1e-6,
        stol: float = 1e-10,
        cutback_factor: float = 0.5,
        growth_factor: float = 1.1,
        max_cutbacks: int = 10,
        verbose: bool = False,
        method: str | None = None,
        device: str | None = None,
        return_intermediate: bool = False,
        aggregate_integration_points: bool = True,
        use_cached_solve: bool = False,
        nlgeom: bool = False,
        alpha: float = 0.0,
        differentiable_parameters: Tensor | Iterable[Tensor] | None = None,
        precision: str | None = None,
        cg_max_iter: int | None = None,
        preconditioner: str | None = None,
    ) -> tuple[Tensor, Tensor, Tensor, Tensor, Tensor]:
        """Quasi-static solve by load increments (base.py:597-923).

        Same arguments and results as the reference.  `method` selects the
        GPU solver ("cg"/None: FP64 Jacobi-CG; "gb300-mixed": FP32 CG with
        FP64 residual replacement) and `precision` may override it;
        `preconditioner` ("jacobi" or "amg", see resolve_preconditioner) picks
        the mixed-precision preconditioner.  `stol` is
        the relative residual of each linear solve.  `verbose` prints the
        Newton residuals and CG iteration counts.  `use_cached_solve` is
        accepted; the CG always starts from zero.
        """
        prec = resolve_precision(method, precision)
        pc = resolve_preconditioner(preconditioner, prec, self.n_dof_per_node)
        if device is not None and torch.device(device).type != "cuda":
            raise RuntimeError("torchfem_gb300 solves on a CUDA device only")
        if alpha > 0.0:
            raise NotImplementedError("viscous stabilization (alpha > 0) is not implemented")
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
        out_dev = self.nodes.device
        d = self.n_dof_per_node
        # a copy: a later in-place edit of the model's constraints must not
        # reach the mask this solve's backward uses
        con_bool = self._constraints.reshape(-1).to(dev).clone()
        con_mask = con_bool.to(torch.uint8).contiguous()
        assert self.material is not None
        mat_kind, mat_data = self.material.kernel_data(self.n_elem)
        nonlinear = isinstance(mat_kind, str)
        if not nonlinear and nlgeom:
            raise NotImplementedError("nlgeom=True is implemented for Hyperelastic3D only")
        if mat_kind == "neo_hookean" and not nlgeom:
            raise NotImplementedError("Hyperelastic3D runs with nlgeom=True on the GPU path")
        if mat_kind == "j2_plane_strain" and nlgeom:
            raise NotImplementedError("plane-strain plasticity runs with nlgeom=False")

        with torch.set_grad_enabled(track):
            mat_data = mat_data.to(dev, torch.float64)
            thickness = self._thickness()
            if thickness is not None:
                thickness = thickness.to(dev, torch.float64).contiguous()
            F_neu = self._neumann.reshape(-1).to(dev, torch.float64)
            DU_dir = self._dirichlet.reshape(-1).to(dev, torch.float64)
            de0_full = (
                self._external_gradient.to(dev, torch.float64) if self._external_gradient_set else None
            )

        if nonlinear:
            mat = self.material
            sc = NLContext(dm, con_mask, -1, prec, max_iter, rtol, atol, stol, cg_max_iter, kind=mat_kind,
                           local_tol=float(getattr(mat, "tolerance", 1e-5)),
                           local_max_iter=int(getattr(mat, "max_iter", 10)), nlgeom=nlgeom)
        else:
            sc = SolveContext(dm, con_mask, mat_kind, prec, max_iter, rtol, atol, stol, cg_max_iter)
        sc.verbose = verbose
        sc.linear = "minres" if method == "minres" else "cg"
        sc.precond = pc
        sc.precond_explicit = preconditioner is not None
        self.last_solve = sc

        shape_ip = (dm.nip, self.n_elem, *self.n_flux)
        u_cur = torch.zeros(self.n_dofs, dtype=torch.float64, device=dev)
        f_cur = torch.zeros(self.n_dofs, dtype=torch.float64, device=dev)
        flux_cur = torch.zeros(shape_ip, dtype=torch.float64, device=dev)
        grad_cur = torch.zeros(shape_ip, dtype=torch.float64, device=dev)
        grad_cur[:] = self.initial_grad.to(dev, torch.float64)
        state_cur = torch.zeros(dm.nip, self.n_elem, self.n_state, dtype=torch.float64, device=dev)
        du = torch.zeros(self.n_dofs, dtype=torch.float64, device=dev)

        outs_u, outs_f, outs_flux, outs_grad, outs_state = [u_cur], [f_cur], [flux_cur], [grad_cur], [state_cur]

        lam = float(increments[0])
        step_frac = 1.0
        # until the first substep converges, a linear material's Newton start
        # (zero increment, zero stress) gives zero internal forces when no
        # displacement is prescribed: its first residual needs no element pass
        fresh = not nonlinear and (de0_full is None) and not bool(DU_dir.any())
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
                    F_ext = (lam + step) * F_neu
                    DU = step * DU_dir
                    de0 = None if de0_full is None else (step * de0_full).contiguous()
                    sigma_prev = flux_cur if track else flux_cur.detach()
                    F_prev = grad_cur if track else grad_cur.detach()
                    st_prev = state_cur if track else state_cur.detach()
                    try:
                        if nonlinear:
                            du = NewtonNonlinear.apply(
                                sc, du.detach(), F_ext.contiguous(), DU.contiguous(), F_prev.contiguous(),
                                sigma_prev.contiguous(), st_prev.contiguous(), de0, mat_data, thickness,
                            )
                        else:
                            sc.zero_start = fresh
                            du = NewtonLinear.apply(
                                sc, du.detach(), F_ext.contiguous(), DU.contiguous(),
                                sigma_prev.contiguous(), de0, mat_data, thickness,
                            )
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
                                f"Newton-Raphson did not converge in increment {n} "
                                f"after {max_cutbacks} cutbacks."
                            ) from err
                        continue
                    du_eval = torch.where(con_bool, DU, du)
                    if nonlinear:
                        f_int, flux_new, grad_new, state_new = IntegrateNonlinear.apply(
                            sc, du_eval.contiguous(), F_prev.contiguous(), sigma_prev.contiguous(),
                            st_prev.contiguous(), de0, mat_data, thickness,
                        )
                        grad_cur = grad_new
                        state_cur = state_new
                    else:
                        f_int, flux_new, h_inc = IntegrateMaterial.apply(
                            sc, du_eval.contiguous(), sigma_prev.contiguous(), de0, mat_data, thickness
                        )
                        grad_cur = grad_cur + h_inc
                    f_cur = f_int
                    u_cur = u_cur + du_eval
                    flux_cur = flux_new
                    du = du_eval
                    fresh = False
                    lam += step
                    step_size = min(growth_factor * step_size, abs(span))
                step_frac = min(step_size / abs(span), 1.0) if span != 0.0 else 1.0
                outs_u.append(u_cur)
                outs_f.append(f_cur)
                outs_flux.append(flux_cur)
                outs_grad.append(grad_cur)
                outs_state.append(state_cur)

            u = torch.stack(outs_u).reshape(N, self.n_nod, d)
            f = torch.stack(outs_f).reshape(N, self.n_nod, d)
            flux = torch.stack(outs_flux)
            grad = torch.stack(outs_grad)
            state = torch.stack(outs_state)
            if aggregate_integration_points:
                grad = grad.mean(dim=1)
                flux = flux.mean(dim=1)
                state = state.mean(dim=1)
            flux = flux.squeeze((-2, -1))
            grad = grad.squeeze((-2, -1))
            if not track:
                u, f, flux, grad, state = (t.detach() for t in (u, f, flux, grad, state))
            dt = self.nodes.dtype
            u, f, flux, grad, state = (t.to(out_dev, dt) for t in (u, f, flux, grad, state))
        if return_intermediate:
            return u, f, flux, grad, state
        return u[-1], f[-1], flux[-1], grad[-1], state[-1]


class Mechanics(FEM):
    """Solid and structural mechanics (base.py:926-1092)."""

    @property
    def n_dof_per_node(self) -> int:
        return self.nodes.shape[1]

    @property
    def initial_grad(self) -> Tensor:
        return torch.eye(self.n_flux[0])

    @property
    def forces(self) -> Tensor:
        return self._neumann

    @forces.setter
    def forces(self, value: Tensor):
        if not value.shape == (self.n_nod, self.n_dof_per_node):
            raise ValueError("Forces must have the same shape as nodes.")
        if not torch.is_floating_point(value):
            raise TypeError("Forces must be a floating-point tensor.")
        self._neumann = value.to(self.nodes.device)

    @property
    def displacements(self) -> Tensor:
        return self._dirichlet

    @displacements.setter
    def displacements(self, value: Tensor):
        if not value.shape == (self.n_nod, self.n_dof_per_node):
            raise ValueError("Displacements must have the same shape as nodes.")
        if not torch.is_floating_point(value):
            raise TypeError("Displacements must be a floating-point tensor.")
        self._dirichlet = value.to(self.nodes.device)

    @property
    def ext_strain(self) -> Tensor:
        return self._external_gradient

    @ext_strain.setter
    def ext_strain(self, value: Tensor):
        if not value.shape == (self.n_elem, self.n_dof_per_node, self.n_dim):
            raise ValueError("External strain must have the same shape as strains.")
        if not torch.is_floating_point(value):
            raise TypeError("External strain must be a floating-point tensor.")
        self._external_gradient = value.to(self.nodes.device)
        self._external_gradient_set = True


def time_grid(t_output: Tensor, delta_t: float) -> tuple[Tensor, Tensor]:
    """Internal times of `Heat.time_integration` and the rows that hold the
    output times (base.py:1387-1411): integration starts at t = 0 even when
    it is not an output time, and every interval between consecutive knots
    is cut into the fewest equal steps of at most delta_t; a ratio within
    1e-9 (relative) of an integer takes no extra step, and each knot is kept
    exactly."""
    t_output = t_output.detach().cpu().to(torch.float64)
    knots = t_output
    if knots[0] > 0.0:
        knots = torch.cat((knots.new_zeros(1), knots))
    chunks = [knots[0:1]]
    output_rows = [] if t_output[0] > 0.0 else [0]
    row = 0
    for t_start, t_end in zip(knots[:-1], knots[1:]):
        ratio = float((t_end - t_start) / delta_t)
        n_sub = max(1, math.ceil(ratio - 1e-9 * max(1.0, ratio)))
        sub = torch.linspace(float(t_start), float(t_end), n_sub + 1, dtype=torch.float64)[1:]
        sub[-1] = t_end
        chunks.append(sub)
        row += n_sub
        output_rows.append(row)
    return torch.cat(chunks), torch.tensor(output_rows)


class Heat(FEM):
    """Steady and transient heat conduction (base.py:1132-1553): one
    temperature per node, heat flux [1, dim] per integration point."""

    @property
    def n_dof_per_node(self) -> int:
        return 1

    @property
    def n_flux(self) -> list[int]:
        return [1, self.n_dim]

    @property
    def initial_grad(self) -> Tensor:
        return torch.zeros(1)

    @property
    def heat_flux(self) -> Tensor:
        return self._neumann

    @heat_flux.setter
    def heat_flux(self, value: Tensor):
        if not value.shape == (self.n_nod, 1):
            raise ValueError("Heat flux must have the same shape as nodes.")
        if not torch.is_floating_point(value):
            raise TypeError("Heat flux must be a floating-point tensor.")
        self._neumann = value.to(self.nodes.device)

    @property
    def temperatures(self) -> Tensor:
        return self._dirichlet

    @temperatures.setter
    def temperatures(self, value: Tensor):
        if not value.shape == (self.n_nod, self.n_dof_per_node):
            raise ValueError("Temperatures must have the same shape as nodes.")
        if not torch.is_floating_point(value):
            raise TypeError("Temperatures must be a floating-point tensor.")
        self._dirichlet = value.to(self.nodes.device)

    def integrate_mass(self) -> Tensor:
        """Element capacity matrices sum_ip w detJ t rho N N^T,
        [n_elem, n_e, n_e] (base.py:376-396)."""
        mesh, _, refs = self._device_material()
        dm = self.device_mesh
        rho = torch.as_tensor(self.material.rho).detach().to(dm.device, torch.float64).expand(self.n_elem)
        me = dm.heat_mass(mesh, rho.contiguous())
        del refs
        return me.to(self.nodes.device, self.nodes.dtype)

    def time_integration(
        self,
        t_output: Tensor | None = None,
        delta_t: float = 1.0e-1,
        max_iter: int = 100,
        verbose: bool = False,
        rtol: float = 1e-8,
        atol: float = 1e-6,
        stol: float = 1e-10,
        device: str | None = None,
        method: str | None = None,
        aggregate_integration_points: bool = True,
        use_cached_solve: bool = False,
        differentiable_parameters: Tensor | Iterable[Tensor] | None = None,
    ) -> tuple[Tensor, Tensor, Tensor, Tensor, Tensor]:
        """Crank-Nicolson time integration (base.py:1288-1553), same arguments
        and results as the reference.

        The equilibrium at t = 0 under the prescribed temperatures comes from
        `solve` with every DOF constrained; each later time step runs Newton
        iterations on r = M du + dt/2 (f_old + f_int + f_ext) (r = 0 on
        constrained DOFs) with (M + dt/2 K) du = -r solved by the GPU CG to
        `stol` in FP64 (`CrankNicolsonStep`).  As in the reference, the
        internal heat flux of the first step's f_old is zero.

        Gradients flow through the whole integration as in the reference's
        autograd through its Newton steps: every step is an autograd node with
        a hand-written adjoint (`CrankNicolsonStep.backward`), and the
        converged-state evaluation of each step is `IntegrateMaterial`, so a
        loss on temperatures, internal heat fluxes and fluxes reaches the
        conductivity, density, thickness and heat sources.  Prescribed
        temperatures are not differentiable on this path.
        """
        if differentiable_parameters is None:
            params: tuple = ()
        elif isinstance(differentiable_parameters, Tensor):
            params = (differentiable_parameters,)
        else:
            params = tuple(differentiable_parameters)
        track = any(p.requires_grad for p in params)
        if track and self._dirichlet.requires_grad:
            raise NotImplementedError("prescribed temperatures are not differentiable on the GPU path")
        resolve_precision(method, None)
        if device is not None and torch.device(device).type != "cuda":
            raise RuntimeError("torchfem_gb300 solves on a CUDA device only")
        t_output = torch.tensor([0.0, 1.0]) if t_output is None else t_output
        if t_output.numel() == 0:
            raise ValueError("t_output must contain at least one time.")
        if t_output.min() < 0.0:
            raise ValueError("t_output must not contain negative times.")
        if (t_output[1:] <= t_output[:-1]).any():
            raise ValueError("t_output must be strictly increasing.")

        increments, t_rows = time_grid(t_output, delta_t)
        dts = (increments[1:] - increments[:-1]).tolist()
        n_out = len(increments)

        dm = self.device_mesh
        dev = dm.device
        con_mask = self._constraints.reshape(-1).to(dev).to(torch.uint8).contiguous()
        con = con_mask.bool()
        nip, fs = dm.nip, dm.flux_shape
        assert self.material is not None
        mat_kind, mat_data = self.material.kernel_data(self.n_elem)
        if isinstance(mat_kind, str):
            raise NotImplementedError(f"{type(self.material).__name__} has a state-dependent tangent")

        with torch.set_grad_enabled(track):
            # equilibrium at t = 0 with the temperatures imposed everywhere (the
            # constraints are swapped, not written in place: the solve's
            # autograd graph keeps the mask it ran with)
            bc_constraints = self._constraints
            self._constraints = torch.ones_like(bc_constraints)
            try:
                temp_eq, _, flux_eq, grad_eq, state_eq = self.solve(
                    aggregate_integration_points=False, stol=stol, differentiable_parameters=params)
            finally:
                self._constraints = bc_constraints
            mat_data = mat_data.to(dev, torch.float64).contiguous()
            thickness = self._thickness()
            if thickness is not None:
                thickness = thickness.to(dev, torch.float64).contiguous()
            rho = torch.as_tensor(self.material.rho).to(dev, torch.float64).expand(self.n_elem).contiguous()
            f_ext = self._neumann.reshape(-1).to(dev, torch.float64).contiguous()
            dirichlet = self._dirichlet.reshape(-1).to(dev, torch.float64).detach()
            u_cur = torch.where(con, dirichlet, temp_eq.reshape(-1).to(dev, torch.float64))
            flux_cur = flux_eq.to(dev, torch.float64).reshape(nip, self.n_elem, *fs)
            grad_cur = grad_eq.to(dev, torch.float64).reshape(nip, self.n_elem, *fs)
            state_cur = state_eq.to(dev, torch.float64).reshape(nip, self.n_elem, self.n_state)
            f_cur = torch.zeros(self.n_dofs, dtype=torch.float64, device=dev)

            # constant conductivity and capacity: both assembled once
            mesh, mat, refs = self._device_material()
            kval = dm.assemble_csr(dm.element_stiffness(mesh, mat, torch.float64), con_mask)
            mval = dm.assemble_csr(dm.heat_mass(mesh, rho.detach()), con_mask)
            del refs
            tc = TransientContext(dm, con_mask, mat_kind, mval, kval, max_iter, rtol, atol, stol, verbose)
            sc = SolveContext(dm, con_mask, mat_kind, "fp64", max_iter, rtol, atol, stol, None)
            self.iterations = tc.iterations

            us, fs_, fluxes, grads = [u_cur], [f_cur], [flux_cur], [grad_cur]
            for n in range(1, n_out):
                dt_n = dts[n - 1]
                if verbose:
                    print(f"time step {n}: t = {float(increments[n]):.6g}")
                du = CrankNicolsonStep.apply(tc, dt_n, f_cur, flux_cur, f_ext, mat_data, thickness, rho)
                f_int, flux_new, h_inc = IntegrateMaterial.apply(sc, du, flux_cur, None, mat_data, thickness)
                u_cur = u_cur + du
                f_cur = f_int
                flux_cur = flux_new
                grad_cur = grad_cur + h_inc
                us.append(u_cur)
                fs_.append(f_cur)
                fluxes.append(flux_cur)
                grads.append(grad_cur)

            rows = t_rows.tolist()
            out_u = torch.stack([us[r] for r in rows]).reshape(-1, self.n_nod, 1)
            out_f = torch.stack([fs_[r] for r in rows]).reshape(-1, self.n_nod, 1)
            out_flux = torch.stack([fluxes[r] for r in rows])
            out_grad = torch.stack([grads[r] for r in rows])
            out_state = state_cur.unsqueeze(0).expand(len(rows), *state_cur.shape)
            if aggregate_integration_points:
                out_grad = out_grad.mean(dim=1)
                out_flux = out_flux.mean(dim=1)
                out_state = out_state.mean(dim=1)
            out_flux = out_flux.squeeze((-2, -1))
            out_grad = out_grad.squeeze((-2, -1))
            if not track:
                out_u, out_f, out_flux, out_grad, out_state = (
                    t.detach() for t in (out_u, out_f, out_flux, out_grad, out_state))
        dt = self.nodes.dtype
        out_dev = self.nodes.device
        return tuple(t.to(out_dev, dt) for t in (out_u, out_f, out_flux, out_grad, out_state))

