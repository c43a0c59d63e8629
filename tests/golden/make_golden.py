"""Generates the golden fixtures in this folder by running torch-fem itself.

Run where a torch-fem checkout is available, naming its `src` folder:

    python tests/golden/make_golden.py --reference <torch-fem checkout>/src [target ...]

(or set TORCHFEM_REFERENCE_SRC instead of passing --reference).

The reference's optional plotting / AMG / IO dependencies (pyvista,
matplotlib, meshio, pyamg) are replaced by inert stub modules so that
`import torchfem` succeeds; the hot path (FEM.__init__, integrate_material,
assemble_matrix, solve with method="spsolve", NewtonRaphsonAdjoint) runs
unmodified.  Outputs are small .npz files; nothing here runs on the GPU machine.
"""

from __future__ import annotations

import contextlib
import hashlib
import importlib.abc
import importlib.machinery
import os
import sys
import time
import types
from pathlib import Path

import numpy as np
import torch

OUT = Path(__file__).resolve().parent
STUB_ROOTS = ("pyamg", "pyvista", "meshio", "matplotlib", "mpl_toolkits")


class _Any:
    def __init__(self, *a, **k):
        pass

    def __call__(self, *a, **k):
        return _Any()

    def __getattr__(self, name):
        if name.startswith("__"):
            raise AttributeError(name)
        return _Any()

    def __mro_entries__(self, bases):
        return (object,)

    def __iter__(self):
        return iter(())


for _op in ("add", "radd", "sub", "rsub", "mul", "rmul", "truediv", "rtruediv", "or", "ror", "and", "getitem"):
    setattr(_Any, f"__{_op}__", lambda self, *a: _Any())


class _StubLoader(importlib.abc.Loader):
    def create_module(self, spec):
        m = types.ModuleType(spec.name)
        m.__path__ = []

        def _getattr(attr):
            if attr.startswith("__"):
                raise AttributeError(attr)
            return _Any()

        m.__getattr__ = _getattr
        return m

    def exec_module(self, module):
        pass


class _StubFinder(importlib.abc.MetaPathFinder):
    def find_spec(self, fullname, path, target=None):
        if fullname.split(".")[0] in STUB_ROOTS:
            return importlib.machinery.ModuleSpec(fullname, _StubLoader(), is_package=True)
        return None


def import_reference(src: str):
    sys.meta_path.insert(0, _StubFinder())
    sys.path.insert(0, src)
    import torchfem  # noqa: F401

    return torchfem


def jitter(nodes: torch.Tensor, h: float, seed: int = 0) -> torch.Tensor:
    """Interior nodes moved by U(-0.1h, 0.1h) per coordinate (seeded)."""
    g = torch.Generator().manual_seed(seed)
    lo, hi = nodes.min(0).values, nodes.max(0).values
    inner = ((nodes > lo) & (nodes < hi)).all(1)
    delta = (torch.rand(nodes.shape, generator=g, dtype=torch.float64) * 2.0 - 1.0) * 0.1 * h
    return nodes + inner[:, None] * delta


def cube_problem(tf, N: int, jit: bool):
    from torchfem import Solid
    from torchfem.materials import IsotropicElasticity3D
    from torchfem.mesh import cube_hexa

    nodes, elements = cube_hexa(N + 1, N + 1, N + 1)
    if jit:
        nodes = jitter(nodes, 1.0 / N)
    model = Solid(nodes, elements, IsotropicElasticity3D(1000.0, 0.3))
    model.constraints[nodes[:, 0] == 0.0, :] = True
    model.forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    return model


def make_c1(tf):
    """10^3 Hexa1 cube: u, f, sigma and d(sum u)/d(forces), and the
    reference's element matrices (k0) and condensed assembled values
    (assemble_matrix, base.py:398-426) of the configuration."""
    model = cube_problem(tf, 10, jit=False)
    con = torch.nonzero(model.constraints.ravel()).ravel()
    ke = model.k0()
    kval = model.assemble_matrix(ke, con)._values()
    forces = model.forces.clone().requires_grad_(True)
    model.forces = forces
    u, f, s, _, _ = model.solve(method="spsolve", differentiable_parameters=forces)
    (g,) = torch.autograd.grad(u.sum(), forces)
    np.savez_compressed(
        OUT / "c1_cube10.npz", u=u.detach().numpy(), f=f.detach().numpy(), sigma=s.detach().numpy(),
        grad_forces=g.numpy(), ke=ke.numpy(), kval=kval.numpy(), torch_version=torch.__version__,
    )


def make_hexa_jitter3(tf):
    """3^3 jittered Hexa1: pattern, element matrices, assembled values,
    solution and gradients w.r.t. forces and per-element E."""
    from torchfem import Solid
    from torchfem.materials import IsotropicElasticity3D

    base = cube_problem(tf, 3, jit=True)
    nodes, elements = base.nodes, base.elements
    con = torch.nonzero(base.constraints.ravel()).ravel()
    ke = base.k0()
    kval = base.assemble_matrix(ke, con)._values()
    E = torch.full((len(elements),), 1000.0)
    E = E * (1.0 + 0.2 * torch.rand(len(elements), generator=torch.Generator().manual_seed(1)))
    E.requires_grad_(True)
    model = Solid(nodes, elements, IsotropicElasticity3D(E, 0.3))
    model.constraints = base.constraints.clone()
    forces = base.forces.clone().requires_grad_(True)
    model.forces = forces
    u, f, s, gr, _ = model.solve(method="spsolve", differentiable_parameters=(forces, E))
    (g_f,) = torch.autograd.grad(u.sum(), forces, retain_graph=True)
    compliance = torch.inner(f.ravel(), u.ravel())
    (g_E,) = torch.autograd.grad(compliance, E)
    np.savez_compressed(
        OUT / "hexa_jitter3.npz", nodes=nodes.numpy(), elements=elements.numpy(),
        constraints=base.constraints.numpy(), forces=base.forces.detach().numpy(), E=E.detach().numpy(),
        glob_idx=base.glob_idx.numpy(), k_map=base.k_map.numpy(), diag_map=base.diag_map.numpy(),
        ke=ke.numpy(), kval=kval.numpy(), u=u.detach().numpy(), f=f.detach().numpy(),
        sigma=s.detach().numpy(), grad=gr.detach().numpy(), grad_forces=g_f.numpy(), grad_E=g_E.numpy(),
        compliance=compliance.detach().numpy(),
    )


def simp_problem(Nx: int, Ny: int, seed: int = 0):
    from torchfem import Planar
    from torchfem.materials import IsotropicElasticityPlaneStress
    from torchfem.mesh import rect_quad

    nodes, elements = rect_quad(Nx + 1, Ny + 1, 2.0, 1.0)
    rho = 0.2 + 0.8 * torch.rand(len(elements), generator=torch.Generator().manual_seed(seed), dtype=torch.float64)
    rho.requires_grad_(True)
    model = Planar(nodes, elements, IsotropicElasticityPlaneStress(rho**3 * 1.0, 0.3))
    model.constraints[nodes[:, 0] == 0.0, :] = True
    tip = torch.argmin(((nodes - torch.tensor([2.0, 0.5])) ** 2).sum(1))
    model.forces[tip, 1] = -1.0
    return model, rho, tip


def make_simp(tf, Nx, Ny, name, sample=None):
    """Compliance L = f.u of the SIMP cantilever and dL/drho (reference autograd)."""
    model, rho, tip = simp_problem(Nx, Ny)
    u, f, s, _, _ = model.solve(method="spsolve", differentiable_parameters=rho)
    L = torch.inner(f.ravel(), u.ravel())
    (g,) = torch.autograd.grad(L, rho)
    out = dict(compliance=L.detach().numpy(), tip=int(tip), u_tip=u[tip].detach().numpy(),
               grad_norm=float(g.norm()), grad_sum=float(g.sum()))
    if sample is None:
        out.update(u=u.detach().numpy(), f=f.detach().numpy(), sigma=s.detach().numpy(), grad_rho=g.numpy(),
                   rho=rho.detach().numpy())
    else:
        idx = torch.randperm(len(rho), generator=torch.Generator().manual_seed(2))[:sample]
        out.update(sample_idx=idx.numpy(), grad_rho_sample=g[idx].numpy())
    np.savez_compressed(OUT / name, **out)


def make_patterns(tf):
    """Patterns of a Tetra2 mesh (reference cube_tetra + linear_to_quadratic)
    and of a quad mesh with one node that belongs to no element."""
    from torchfem import Planar, Solid
    from torchfem.elements import linear_to_quadratic
    from torchfem.materials import IsotropicElasticity3D, IsotropicElasticityPlaneStress
    from torchfem.mesh import cube_tetra, rect_quad

    n_t, e_t = linear_to_quadratic(*cube_tetra(3, 3, 3))
    mt = Solid(n_t, e_t, IsotropicElasticity3D(1000.0, 0.3))
    n_q, e_q = rect_quad(4, 3)
    n_q = torch.cat([n_q, torch.tensor([[5.0, 5.0]])])
    mq = Planar(n_q, e_q, IsotropicElasticityPlaneStress(1000.0, 0.3))
    np.savez_compressed(
        OUT / "patterns.npz",
        tet2_nodes=n_t.numpy(), tet2_elements=e_t.numpy(), tet2_glob_idx=mt.glob_idx.numpy(),
        tet2_k_map=mt.k_map.numpy(), tet2_diag_map=mt.diag_map.numpy(),
        orphan_nodes=n_q.numpy(), orphan_elements=e_q.numpy(), orphan_glob_idx=mq.glob_idx.numpy(),
        orphan_k_map=mq.k_map.numpy(), orphan_diag_map=mq.diag_map.numpy(),
    )


def _repo_mesh():
    """This repository's mesh module (the reference has no 6-tet split or O-grid)."""
    sys.path.insert(0, str(OUT.parents[1] / "torch-fem_gb300"))
    from torchfem_gb300 import mesh

    return mesh


def hyper_problem(nx, ny, nz, seed=0):
    """Config 4 geometry: box [0,3]x[0,1]^2 split into Tetra2, x=0 clamped,
    x=3 pulled by +0.5; per-element E = 1000 (1 + 0.1 N(0,1)), nu = 0.45."""
    from torchfem import Solid
    from torchfem.materials import Hyperelastic3D

    mesh = _repo_mesh()
    nodes, elements = mesh.linear_to_quadratic(*mesh.box_tetra6(nx + 1, ny + 1, nz + 1, 3.0, 1.0, 1.0))
    gen = torch.Generator().manual_seed(seed)
    E = 1000.0 * (1.0 + 0.1 * torch.randn(len(elements), generator=gen, dtype=torch.float64))
    E.requires_grad_(True)
    nu = 0.45
    mu = E / (2.0 * (1.0 + nu))
    lbd = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))

    def psi(F, params):
        MU, LBD = params[0], params[1]
        C = F.transpose(-1, -2) @ F
        logJ = 0.5 * torch.logdet(C)
        return MU / 2 * (torch.trace(C) - 3.0) - MU * logJ + LBD / 2 * logJ**2

    model = Solid(nodes, elements, Hyperelastic3D(psi, torch.stack([mu, lbd], dim=-1)))
    right = nodes[:, 0] == 3.0
    model.constraints[nodes[:, 0] == 0.0, :] = True
    model.constraints[right, 0] = True
    model.displacements[right, 0] = 0.5
    return model, E, right, nodes, elements


def make_hyper(tf, nx=6, ny=2, nz=2):
    model, E, right, nodes, elements = hyper_problem(nx, ny, nz)
    inc = torch.linspace(0.0, 1.0, 11)
    u, f, s, F, _ = model.solve(increments=inc, nlgeom=True, method="spsolve", rtol=1e-12, atol=1e-12,
                                max_iter=20, differentiable_parameters=E)
    R = f[right, 0].sum()
    (gE,) = torch.autograd.grad(R, E)
    np.savez_compressed(
        OUT / "hyper_tet2_6x2x2.npz", nodes=nodes.numpy(), elements=elements.numpy(), E=E.detach().numpy(),
        u=u.detach().numpy(), f=f.detach().numpy(), sigma=s.detach().numpy(), F=F.detach().numpy(),
        reaction=R.detach().numpy(), grad_E=gE.numpy(),
    )


def plastic_problem(n_theta, n_rad):
    """Config 5 geometry: 2 x 1 plate, centred hole r = 0.25, O-grid; left
    edge fixed in x plus one y pin, right edge pulled to u_x = 0.02."""
    from torchfem import Planar
    from torchfem.materials import IsotropicPlasticityPlaneStrain

    mesh = _repo_mesh()
    nodes, elements = mesh.plate_hole_ogrid(n_theta, n_rad)
    mat = IsotropicPlasticityPlaneStrain(
        1000.0, 0.3, lambda q: 1.0 + 100.0 * q, lambda q: 100.0 * torch.ones_like(q)
    )
    t = torch.ones(len(elements), dtype=torch.float64, requires_grad=True)
    model = Planar(nodes, elements, mat, thickness=t)
    left = torch.isclose(nodes[:, 0], torch.tensor(0.0, dtype=torch.float64))
    right = torch.isclose(nodes[:, 0], torch.tensor(2.0, dtype=torch.float64))
    model.constraints[left, 0] = True
    pin = torch.argmin(((nodes - torch.tensor([0.0, 0.5])) ** 2).sum(1))
    model.constraints[pin, 1] = True
    model.constraints[right, 0] = True
    model.displacements[right, 0] = 0.02
    return model, t, right, nodes, elements


def make_plastic(tf, n_theta=32, n_rad=8, name="plastic_ogrid_32x8.npz"):
    model, t, right, nodes, elements = plastic_problem(n_theta, n_rad)
    inc = torch.linspace(0.0, 1.0, 21)
    # the reference's plane-strain tangent is not the exact derivative of its
    # stress update, so Newton converges linearly and needs more iterations
    u, f, s, F, st = model.solve(increments=inc, method="spsolve", rtol=1e-12, atol=1e-12, max_iter=80,
                                 differentiable_parameters=t)
    R = f[right, 0].sum()
    (gt,) = torch.autograd.grad(R, t)
    np.savez_compressed(
        OUT / name, nodes=nodes.numpy(), elements=elements.numpy(),
        u=u.detach().numpy(), f=f.detach().numpy(), sigma=s.detach().numpy(), state=st.detach().numpy(),
        reaction=R.detach().numpy(), grad_t=gt.numpy(),
    )


def make_material_points(tf):
    """Per-point outputs of the reference's Material.step for the
    Neo-Hookean energy (via jacrev) and plane-strain J2 plasticity."""
    from torchfem.materials import Hyperelastic3D, IsotropicPlasticityPlaneStrain

    gen = torch.Generator().manual_seed(5)
    n = 16
    F = torch.eye(3) + 0.15 * (torch.rand(n, 3, 3, generator=gen, dtype=torch.float64) - 0.5)
    mu = 300.0 + 100.0 * torch.rand(n, generator=gen, dtype=torch.float64)
    lam = 800.0 + 400.0 * torch.rand(n, generator=gen, dtype=torch.float64)

    def psi(Fm, params):
        MU, LBD = params[0], params[1]
        Cm = Fm.transpose(-1, -2) @ Fm
        logJ = 0.5 * torch.logdet(Cm)
        return MU / 2 * (torch.trace(Cm) - 3.0) - MU * logJ + LBD / 2 * logJ**2

    hy = Hyperelastic3D(psi, torch.stack([mu, lam], dim=-1))
    zero = torch.zeros(n, 3, 3)
    P, _, A = hy.step(zero, F, zero, torch.zeros(n, 0), zero, None, 0)
    pl = IsotropicPlasticityPlaneStrain(
        1000.0, 0.3, lambda q: 1.0 + 100.0 * q, lambda q: 100.0 * torch.ones_like(q)
    ).vectorize(n)
    H = 4e-3 * (torch.rand(n, 2, 2, generator=gen, dtype=torch.float64) - 0.5)
    stress = 2.0 * (torch.rand(n, 2, 2, generator=gen, dtype=torch.float64) - 0.5)
    stress = 0.5 * (stress + stress.transpose(-1, -2))
    state = torch.stack([0.01 * torch.rand(n, generator=gen, dtype=torch.float64),
                         1e-3 * (torch.rand(n, generator=gen, dtype=torch.float64) - 0.5)], dim=-1)
    s_new, st_new, D = pl.step(H, None, stress, state, torch.zeros(n, 2, 2), None, 0)
    np.savez_compressed(
        OUT / "material_points.npz", F=F.numpy(), mu=mu.numpy(), lam=lam.numpy(), P=P.detach().numpy(),
        A=A.detach().numpy(), H=H.numpy(), stress=stress.numpy(), state=state.numpy(),
        stress_new=s_new.numpy(), state_new=st_new.numpy(), ddsdde=D.numpy(),
    )


def shell_problem(n_arc=9, n_len=7, seed=0):
    """Tria1 shell on a cylindrical roof (axis y, 80 degrees, R = 1, L = 2):
    the y = 0 edge clamped, the y = 2 edge held in x and z and pushed by a
    prescribed u_y; self-weight-like z loads, moments about x on the free
    straight edges; per-element thickness and E (seeded) for the gradients."""
    from torchfem import Shell
    from torchfem.materials import IsotropicElasticityPlaneStress

    mesh = _repo_mesh()
    nodes, elements = mesh.cylinder_patch_tria(n_arc, n_len, 1.0, 2.0, 80.0)
    gen = torch.Generator().manual_seed(seed)
    n_elem = len(elements)
    E = 1000.0 * (1.0 + 0.1 * torch.randn(n_elem, generator=gen, dtype=torch.float64))
    t = 0.05 * (1.0 + 0.2 * torch.rand(n_elem, generator=gen, dtype=torch.float64))
    E.requires_grad_(True)
    t.requires_grad_(True)
    model = Shell(nodes, elements, IsotropicElasticityPlaneStress(E, 0.3), thickness=t)
    y0 = nodes[:, 1] == 0.0
    y1 = nodes[:, 1] == 2.0
    side = (nodes[:, 0] - nodes[:, 0].min()).abs() < 1e-12
    model.constraints[y0, :] = True
    model.constraints[y1, 0] = True
    model.constraints[y1, 2] = True
    model.displacements[y1, 0] = 0.0
    model.constraints[y1, 1] = True
    model.displacements[y1, 1] = 1e-3
    model.forces[:, 2] = -1.0 / len(nodes)
    model.forces[side, 3] = 2e-3
    return model, E, t, nodes, elements


def make_shell(tf):
    model, E, t, nodes, elements = shell_problem()
    u, f, s, F, st = model.solve(method="spsolve", rtol=1e-12, atol=1e-14, differentiable_parameters=(E, t))
    _, _, s_ip, _, _ = model.solve(method="spsolve", rtol=1e-12, atol=1e-14, aggregate_integration_points=False)
    free = ~model.constraints
    L = (u * free).pow(2).sum() + (f[:, 2] * u[:, 2]).sum()
    gE, gt = torch.autograd.grad(L, (E, t))
    with torch.no_grad():
        ke = model.k0()
        con = model.constraints.reshape(-1)
        K = torch.zeros(model.n_dofs * model.n_dofs, dtype=torch.float64).index_add_(
            0, model.glob_idx[0] * model.n_dofs + model.glob_idx[1],
            torch.zeros(len(model.glob_idx[0]), dtype=torch.float64).index_add_(0, model.k_map, ke.ravel()),
        ).reshape(model.n_dofs, model.n_dofs)
        K[con, :] = 0.0
        K[:, con] = 0.0
        K[con, con] = 1.0
    np.savez_compressed(
        OUT / "shell_roof_9x7.npz", nodes=nodes.numpy(), elements=elements.numpy(), E=E.detach().numpy(),
        ke=ke.numpy(), glob_idx=model.glob_idx.numpy(), k_map=model.k_map.numpy(),
        t=t.detach().numpy(), u=u.detach().numpy(), f=f.detach().numpy(), sigma=s.detach().numpy(),
        sigma_ip=s_ip.detach().numpy(), F=F.detach().numpy(), loss=L.detach().numpy(),
        grad_E=gE.numpy(), grad_t=gt.numpy(), K=K.numpy(),
    )


def make_hexa2(tf):
    """Hexa2 (20-node serendipity): the reference's linear_to_quadratic of a
    jittered 2^3 Hexa1 cube, its pattern, element matrices and the solution."""
    from torchfem import Solid
    from torchfem.elements import linear_to_quadratic
    from torchfem.materials import IsotropicElasticity3D
    from torchfem.mesh import cube_hexa

    nodes, elements = cube_hexa(3, 3, 3)
    nodes = jitter(nodes, 1.0 / 2.0)
    nodes, elements = linear_to_quadratic(nodes, elements)
    model = Solid(nodes, elements, IsotropicElasticity3D(1000.0, 0.3))
    model.constraints[nodes[:, 0] == 0.0, :] = True
    model.forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    u, f, s, F, _ = model.solve(method="spsolve", rtol=1e-12)
    with torch.no_grad():
        ke = model.k0()
    np.savez_compressed(
        OUT / "hexa2_jitter2.npz", nodes=nodes.numpy(), elements=elements.numpy(), ke=ke.numpy(),
        glob_idx=model.glob_idx.numpy(), k_map=model.k_map.numpy(), u=u.numpy(), f=f.numpy(),
        sigma=s.numpy(), F=F.numpy(),
    )


def make_heat(tf):
    """Heat conduction: a jittered 4^3 SolidHeat with per-element
    conductivity, a PlanarHeat with thickness rho^3 and a rotated orthotropic
    PlanarHeat (temperatures, heat fluxes, element conductivity matrices and
    gradients of the thermal compliance f.T), and the Crank-Nicolson time
    integration of the heated plate of tests/test_time_integration.py."""
    from torchfem import PlanarHeat, SolidHeat
    from torchfem.materials import (IsotropicConductivity2D, IsotropicConductivity3D,
                                    OrthotropicConductivity2D)
    from torchfem.mesh import cube_hexa, rect_quad

    out = {}
    # (a) SolidHeat, Hexa1, kappa per element, T = 0 on x = 0, uniform source
    nodes, elements = cube_hexa(5, 5, 5)
    nodes = jitter(nodes, 0.25, seed=3)
    kappa = 400.0 * (1.0 + 0.5 * torch.rand(len(elements), generator=torch.Generator().manual_seed(4)))
    kappa.requires_grad_(True)
    model = SolidHeat(nodes, elements, IsotropicConductivity3D(kappa))
    model.constraints[nodes[:, 0] == 0.0] = True
    model.temperatures[nodes[:, 0] == 0.0, 0] = 1.0
    q = torch.full((len(nodes), 1), 10.0 / len(nodes)).requires_grad_(True)
    model.heat_flux = q
    T, f, flux, grad, _ = model.solve(differentiable_parameters=(kappa, q))
    L = torch.inner(f.ravel(), T.ravel())
    g_kappa, g_q = torch.autograd.grad(L, (kappa, q))
    with torch.no_grad():
        k0 = model.k0()
    out.update(solid_nodes=nodes.numpy(), solid_elements=elements.numpy(), solid_kappa=kappa.detach().numpy(),
               solid_con=model.constraints.numpy(), solid_temp=model.temperatures.numpy(),
               solid_q=q.detach().numpy(), solid_T=T.detach().numpy(), solid_f=f.detach().numpy(),
               solid_flux=flux.detach().numpy(), solid_grad=grad.detach().numpy(), solid_L=L.detach().numpy(),
               solid_g_kappa=g_kappa.numpy(), solid_g_q=g_q.numpy(), solid_k0=k0.numpy())

    # (b) PlanarHeat, Quad1, thickness rho^3 per element, T = 0 west and north
    nodes, elements = rect_quad(7, 5, 1.5, 1.0)
    rho = 0.3 + 0.7 * torch.rand(len(elements), generator=torch.Generator().manual_seed(5), dtype=torch.float64)
    rho.requires_grad_(True)
    model = PlanarHeat(nodes, elements, IsotropicConductivity2D(kappa=400.0))
    model.thickness = rho**3
    west = torch.isclose(nodes[:, 0], nodes[:, 0].min())
    north = torch.isclose(nodes[:, 1], nodes[:, 1].max())
    model.constraints[west | north] = True
    model.heat_flux[:, 0] = 1000.0 / len(nodes)
    T, f, flux, grad, _ = model.solve(differentiable_parameters=rho)
    L = torch.inner(f.ravel(), T.ravel())
    (g_rho,) = torch.autograd.grad(L, rho)
    out.update(planar_nodes=nodes.numpy(), planar_elements=elements.numpy(), planar_rho=rho.detach().numpy(),
               planar_con=model.constraints.numpy(), planar_q=model.heat_flux.numpy(),
               planar_T=T.detach().numpy(), planar_f=f.detach().numpy(), planar_flux=flux.detach().numpy(),
               planar_L=L.detach().numpy(), planar_g_rho=g_rho.numpy())

    # (c) rotated orthotropic conductivity on the same mesh, T prescribed on x = 0 and x = 1.5
    c = torch.cos(torch.tensor(0.5)), torch.sin(torch.tensor(0.5))
    R = torch.stack([torch.stack([c[0], -c[1]]), torch.stack([c[1], c[0]])])
    mat = OrthotropicConductivity2D(50.0, 5.0).rotate(R)
    model = PlanarHeat(nodes, elements, mat, thickness=0.1)
    east = torch.isclose(nodes[:, 0], nodes[:, 0].max())
    model.constraints[west | east] = True
    model.temperatures[west, 0] = 10.0
    model.temperatures[east, 0] = -5.0
    T, f, flux, grad, _ = model.solve()
    with torch.no_grad():
        k0 = model.k0()
    out.update(ortho_kappa=mat.KAPPA.numpy(), ortho_con=model.constraints.numpy(),
               ortho_temp=model.temperatures.numpy(), ortho_T=T.numpy(), ortho_f=f.numpy(),
               ortho_flux=flux.numpy(), ortho_grad=grad.numpy(), ortho_k0=k0.numpy())

    # (d) transient: heated plate, Crank-Nicolson with dt = 1 to t = 24, and a
    # late-starting output grid with dt = 0.5
    def plate():
        m = PlanarHeat(*rect_quad(5, 5, 1.0, 1.0), IsotropicConductivity2D(kappa=400.0, rho=1.0e5))
        w = torch.isclose(m.nodes[:, 0], m.nodes[:, 0].min())
        e = torch.isclose(m.nodes[:, 0], m.nodes[:, 0].max())
        m.constraints[w | e] = True
        m.temperatures[w, 0] = 5.0
        m.temperatures[e, 0] = 20.0
        return m

    m = plate()
    with torch.no_grad():
        me = m.integrate_mass()
    t_out = torch.tensor([0.0, 6.0, 12.0, 18.0, 24.0])
    temp, rfl, flux, grad, _ = m.time_integration(t_out, delta_t=1.0)
    out.update(plate_mass=me.numpy(), plate_t=t_out.numpy(), plate_temp=temp.numpy(), plate_f=rfl.numpy(),
               plate_flux=flux.numpy(), plate_grad=grad.numpy())
    m = plate()
    t_late = torch.tensor([2.5, 5.0])
    temp, rfl, flux, grad, _ = m.time_integration(t_late, delta_t=0.5, aggregate_integration_points=False)
    out.update(late_t=t_late.numpy(), late_temp=temp.numpy(), late_f=rfl.numpy(), late_flux=flux.numpy(),
               late_grad=grad.numpy())
    np.savez_compressed(OUT / "heat_cases.npz", **out)


def make_heat_transient_grad(tf):
    """Gradients through Heat.time_integration: the heated plate with
    per-element conductivity and density and nodal heat sources as
    differentiable parameters, loss sum_k c_k . T(t_k) with seeded weights c,
    on a grid with unequal steps (knots 0, 2, 5 and delta_t 0.8)."""
    from torchfem import PlanarHeat
    from torchfem.materials import IsotropicConductivity2D
    from torchfem.mesh import rect_quad

    nodes, elements = rect_quad(6, 5, 1.0, 0.8)
    g = torch.Generator().manual_seed(11)
    kappa = (400.0 * (1.0 + torch.rand(len(elements), generator=g))).requires_grad_(True)
    rho = (1.0e5 * (1.0 + torch.rand(len(elements), generator=g))).requires_grad_(True)
    q = (50.0 * torch.rand(len(nodes), 1, generator=g)).requires_grad_(True)
    model = PlanarHeat(nodes, elements, IsotropicConductivity2D(kappa, rho))
    west = torch.isclose(nodes[:, 0], nodes[:, 0].min())
    east = torch.isclose(nodes[:, 0], nodes[:, 0].max())
    model.constraints[west | east] = True
    model.temperatures[west, 0] = 5.0
    model.temperatures[east, 0] = 20.0
    model.heat_flux = q
    t_out = torch.tensor([0.0, 2.0, 5.0])
    temp, rfl, flux, grad, _ = model.time_integration(t_out, delta_t=0.8, differentiable_parameters=(kappa, rho, q))
    c = torch.rand(temp.shape, generator=g)
    L = (c * temp).sum()
    gk, gr, gq = torch.autograd.grad(L, (kappa, rho, q))
    np.savez_compressed(
        OUT / "heat_transient_grad.npz", nodes=nodes.numpy(), elements=elements.numpy(),
        kappa=kappa.detach().numpy(), rho=rho.detach().numpy(), q=q.detach().numpy(),
        con=model.constraints.numpy(), temp_bc=model.temperatures.numpy(), t_out=t_out.numpy(), delta_t=0.8,
        temp=temp.detach().numpy(), c=c.numpy(), L=L.detach().numpy(), g_kappa=gk.numpy(), g_rho=gr.numpy(),
        g_q=gq.numpy(),
    )


def make_modes(tf):
    """Modal analysis (FEM.solve_modes): the six lowest squared angular
    frequencies of a jittered 3^3 Hexa1 cube clamped on x = 0, with
    per-element E and rho, and d(sum omega^2)/d(E, rho)."""
    from torchfem import Solid
    from torchfem.materials import IsotropicElasticity3D

    base = cube_problem(tf, 3, jit=True)
    nodes, elements = base.nodes, base.elements
    g = torch.Generator().manual_seed(21)
    E = (1000.0 * (1.0 + 0.5 * torch.rand(len(elements), generator=g))).requires_grad_(True)
    rho = (1.0 + torch.rand(len(elements), generator=g)).requires_grad_(True)
    model = Solid(nodes, elements, IsotropicElasticity3D(E, 0.3, rho))
    model.constraints[nodes[:, 0] == 0.0, :] = True
    omega_sq, modes = model.solve_modes(6)
    gE, gr = torch.autograd.grad(omega_sq.sum(), (E, rho))
    np.savez_compressed(
        OUT / "modes_hexa_jitter3.npz", nodes=nodes.numpy(), elements=elements.numpy(), E=E.detach().numpy(),
        rho=rho.detach().numpy(), con=model.constraints.numpy(), omega_sq=omega_sq.detach().numpy(),
        modes=modes.numpy(), g_E=gE.numpy(), g_rho=gr.numpy(),
    )


class _JacobiAMG:
    """Stand-in for pyamg on the reference's iterative CPU route.

    `_solve_cpu` (sparse.py:477-512) builds its CG/MINRES preconditioner with
    `pyamg.smoothed_aggregation_solver(A, B, smooth="jacobi").aspreconditioner()`.
    pyamg is not installed here, so this object answers that call with the
    Jacobi operator diag(A)^-1, the preconditioner the reference's GPU CG branch
    builds (sparse.py:406-421).  Each operator counts its applications, which
    is the CG iteration count plus one.
    """

    applications = 0

    @classmethod
    def smoothed_aggregation_solver(cls, A, B=None, smooth=None):
        from scipy.sparse.linalg import LinearOperator

        dinv = 1.0 / A.diagonal()

        def matvec(x):
            cls.applications += 1
            return dinv * x.ravel()

        class _Hierarchy:
            def aspreconditioner(self):
                return LinearOperator(A.shape, matvec=matvec, dtype=A.dtype)

        return _Hierarchy()


@contextlib.contextmanager
def jacobi_cg_route(tf):
    """The reference's `sparse_solve(method="cg")` with the Jacobi stand-in."""
    old = tf.sparse.pyamg
    tf.sparse.pyamg = _JacobiAMG
    try:
        yield _JacobiAMG
    finally:
        tf.sparse.pyamg = old


class _OracleAMG:
    """Stand-in for pyamg on the reference's iterative CPU route, with a
    multigrid preconditioner: `smoothed_aggregation_solver(A, B, smooth)`
    answers with one V-cycle of the oracle's smoothed-aggregation hierarchy
    (oracle/amg_oracle.py, the algorithm family of pyamg's solver) of the
    condensed matrix A.  The node coordinates come from the rotation columns
    of the reference's rigid-body modes B (FEM.compute_B, base.py:316-344)
    and the constrained DOFs are the rows the reference's condensation made
    unit rows (base.py:414-419).  CG still stops at the reference's stol, so
    the preconditioner changes only how fast the reference's solves get
    there.  3D models only."""

    applications = 0

    @classmethod
    def smoothed_aggregation_solver(cls, A, B=None, smooth=None):
        import scipy.sparse as sp
        from scipy.sparse.linalg import LinearOperator

        sys.path.insert(0, str(OUT.parents[1]))
        from oracle import amg_oracle as AO

        A = sp.csr_matrix(A)
        B = np.asarray(B)
        coords = np.stack([B[1::3, 5], B[2::3, 3], B[0::3, 4]], axis=1)
        diag = A.diagonal()
        off = np.asarray(abs(A).sum(axis=1)).ravel() - np.abs(diag)
        con = ((off == 0.0) & (diag == 1.0)).reshape(-1, 3)
        levels = AO.hierarchy(A, coords, con, 3)

        def matvec(x):
            cls.applications += 1
            return AO.vcycle(levels, np.asarray(x, dtype=np.float64).ravel())

        class _Hierarchy:
            def aspreconditioner(self):
                return LinearOperator(A.shape, matvec=matvec, dtype=A.dtype)

        return _Hierarchy()


@contextlib.contextmanager
def oracle_amg_cg_route(tf):
    """The reference's `sparse_solve(method="cg")` with the multigrid stand-in."""
    old = tf.sparse.pyamg
    tf.sparse.pyamg = _OracleAMG
    try:
        yield _OracleAMG
    finally:
        tf.sparse.pyamg = old


def c2_problem(n: int):
    """Config 2 geometry: Hexa1 cube of n^3 elements, interior nodes jittered
    by U(-0.1, 0.1)/n per coordinate from torch seed 0, E = 1000, nu = 0.3,
    x = 0 clamped, z-force -1/n_nodes on every node of x = 1."""
    from torchfem import Solid
    from torchfem.materials import IsotropicElasticity3D
    from torchfem.mesh import cube_hexa

    nodes, elements = cube_hexa(n + 1, n + 1, n + 1)
    gen = torch.Generator().manual_seed(0)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    nodes = nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen, dtype=torch.float64) * 2 - 1) * (0.1 / n)
    model = Solid(nodes, elements, IsotropicElasticity3D(1000.0, 0.3))
    model.constraints[nodes[:, 0] == 0.0, :] = True
    forces = torch.zeros_like(nodes)
    forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    forces.requires_grad_(True)
    model.forces = forces
    return model, forces, nodes, elements


def c2_solve(tf, n: int, method: str, stol: float):
    """The reference's solve + d(sum u)/d(forces) on the config-2 cube."""
    model, forces, nodes, elements = c2_problem(n)
    with jacobi_cg_route(tf) as amg:
        amg.applications = 0
        t0 = time.perf_counter()
        u, f, s, _, _ = model.solve(method=method, stol=stol, differentiable_parameters=forces)
        t1 = time.perf_counter()
        fwd_apps = amg.applications
        (g,) = torch.autograd.grad(u.sum(), forces)
        t2 = time.perf_counter()
        adj_apps = amg.applications - fwd_apps
    return dict(nodes=nodes, elements=elements, u=u.detach().numpy(), f=f.detach().numpy(),
                sigma=s.detach().numpy(), grad=g.numpy(), t_fwd=t1 - t0, t_adj=t2 - t1,
                cg_fwd=fwd_apps - 1, cg_adj=adj_apps - 1)


def _sample(rng, n, k):
    return np.sort(rng.choice(n, size=min(k, n), replace=False)).astype(np.int64)


def _projection_weights(n):
    """Deterministic weights for full-field checksums <w, x>."""
    return np.cos(np.arange(n, dtype=np.float64) * 0.6180339887498949)


def make_c2(tf, n=70, stol=1e-13, name="c2_cube70_sample.npz"):
    """Config 2 at full size (70^3 jittered Hexa1, 1,073,733 DOF) by the
    reference's own pattern, k0, assembly and autograd, with its CG route
    (`sparse_solve(method="cg")`, Jacobi, stol 1e-13) for the forward and the
    adjoint of sum(u).  SuperLU cannot factor this size.  Stored: seeded
    samples of u, f, sigma and the gradient, their max-abs and 2-norms, and
    full-field checksums <w, x> with the weights of `_projection_weights`."""
    r = c2_solve(tf, n, "cg", stol)
    rng = np.random.default_rng(20261204)
    u, f, s, g = r["u"].ravel(), r["f"].ravel(), r["sigma"].ravel(), r["grad"].ravel()
    out = dict(n=n, stol=stol, n_dofs=u.size,
               nodes_sha256=hashlib.sha256(np.ascontiguousarray(r["nodes"].numpy())).hexdigest(),
               t_fwd=r["t_fwd"], t_adj=r["t_adj"], cg_fwd=r["cg_fwd"], cg_adj=r["cg_adj"],
               torch_version=torch.__version__, host_threads=torch.get_num_threads(), cpu_count=os.cpu_count())
    for key, x in (("u", u), ("f", f), ("sigma", s), ("grad", g)):
        idx = _sample(rng, x.size, 10000)
        out[f"{key}_idx"] = idx
        out[f"{key}_sample"] = x[idx]
        out[f"{key}_maxabs"] = float(np.abs(x).max())
        out[f"{key}_norm"] = float(np.linalg.norm(x))
        w = _projection_weights(x.size)
        out[f"{key}_proj"] = float(w @ x)
        out[f"{key}_projscale"] = float(np.abs(w) @ np.abs(x))
    np.savez_compressed(OUT / name, **out)
    print(f"c2 n={n}: fwd {r['t_fwd']:.1f} s ({r['cg_fwd']} CG its), adjoint {r['t_adj']:.1f} s ({r['cg_adj']} its)")


def make_c2_crosscheck(tf, sizes=(20, 30), stol=1e-13, name="c2_route_crosscheck.npz"):
    """Shows that the CG route of `make_c2` reproduces the reference's direct
    solve (SuperLU, method="spsolve") on smaller cubes of the same kind: the
    max-abs relative differences of u, sigma and the gradient."""
    out = {}
    for n in sizes:
        a = c2_solve(tf, n, "spsolve", stol)
        b = c2_solve(tf, n, "cg", stol)
        for key in ("u", "sigma", "grad"):
            d = float(np.abs(a[key] - b[key]).max() / np.abs(a[key]).max())
            out[f"n{n}_{key}"] = d
        out[f"n{n}_t_spsolve"] = a["t_fwd"] + a["t_adj"]
        out[f"n{n}_t_cg"] = b["t_fwd"] + b["t_adj"]
        out[f"n{n}_cg_its"] = np.array([b["cg_fwd"], b["cg_adj"]])
        print(n, {k: v for k, v in out.items() if k.startswith(f"n{n}_")})
    np.savez_compressed(OUT / name, sizes=np.array(sizes), stol=stol, **out)


def make_hyper_full(tf, name="hyper_tet2_30x10x10.npz", counts=(10, 20, 40)):
    """Config 4 at full size (30 x 10 x 10 box, 6 Tetra2 per hex, 80,703 DOF,
    Neo-Hookean, nlgeom, x = 3 face pulled to +0.5) by the reference's own
    solve and autograd, with the CG route of `oracle_amg_cg_route` (SuperLU
    needs minutes per Newton step at this size, Jacobi CG about 2,500
    iterations per solve).  The load is first applied in 10
    increments as the configuration states; when the reference's own solve
    raises there, its message is stored and the next count of `counts` is
    tried.  Stored: u, f, the tip reaction and its gradient w.r.t. the
    per-element E of the first count that completes, a seeded sample of the
    element stresses, and the wall times and CG iteration counts."""
    out = {"counts_tried": np.array(counts)}
    for n_inc in counts:
        model, E, right, nodes, elements = hyper_problem(30, 10, 10)
        inc = torch.linspace(0.0, 1.0, n_inc + 1)
        with oracle_amg_cg_route(tf) as amg:
            amg.applications = 0
            t0 = time.perf_counter()
            try:
                u, f, s, F, _ = model.solve(increments=inc, nlgeom=True, method="cg", rtol=1e-10, atol=1e-10,
                                            max_iter=20, stol=1e-12, differentiable_parameters=E, verbose=True)
            except RuntimeError as err:
                out[f"inc{n_inc}_error"] = str(err)
                out[f"inc{n_inc}_seconds"] = time.perf_counter() - t0
                print(f"{n_inc} increments: the reference raised: {err}", flush=True)
                continue
            t1 = time.perf_counter()
            fwd_apps = amg.applications
            R = f[right, 0].sum()
            (gE,) = torch.autograd.grad(R, E)
            t2 = time.perf_counter()
        rng = np.random.default_rng(4)
        sig = s.detach().numpy().ravel()
        idx = _sample(rng, sig.size, 10000)
        out.update(increments=n_inc, nodes=nodes.numpy(), elements=elements.numpy(), E=E.detach().numpy(),
                   u=u.detach().numpy(), f=f.detach().numpy(), sigma_idx=idx, sigma_sample=sig[idx],
                   sigma_maxabs=float(np.abs(sig).max()), reaction=R.detach().numpy(), grad_E=gE.numpy(),
                   t_fwd=t1 - t0, t_adj=t2 - t1, precond_applications_fwd=fwd_apps,
                   precond_applications_adj=amg.applications - fwd_apps, torch_version=torch.__version__)
        print(f"{n_inc} increments: fwd {t1 - t0:.1f} s, adjoint {t2 - t1:.1f} s", flush=True)
        break
    np.savez_compressed(OUT / name, **out)


def make_hyper_mid(tf, name="hyper_tet2_15x5x5.npz", counts=(10, 20)):
    """Config 4's problem at half the resolution (15 x 5 x 5 box, 6 Tetra2
    per hex, 11,163 DOF), where the reference's own direct solve
    (method="spsolve") is affordable: the load is applied in 10 increments
    as the configuration states, and when the reference raises there its
    message is stored and 20 increments are run.  Stored: u, f, the tip
    reaction and its gradient w.r.t. the per-element E of the count that
    completes, with the wall times."""
    out = {"counts_tried": np.array(counts)}
    for n_inc in counts:
        model, E, right, nodes, elements = hyper_problem(15, 5, 5)
        inc = torch.linspace(0.0, 1.0, n_inc + 1)
        t0 = time.perf_counter()
        try:
            u, f, s, F, _ = model.solve(increments=inc, nlgeom=True, method="spsolve", rtol=1e-10, atol=1e-10,
                                        max_iter=20, differentiable_parameters=E)
        except RuntimeError as err:
            out[f"inc{n_inc}_error"] = str(err)
            out[f"inc{n_inc}_seconds"] = time.perf_counter() - t0
            print(f"{n_inc} increments: the reference raised: {err}", flush=True)
            continue
        t1 = time.perf_counter()
        R = f[right, 0].sum()
        (gE,) = torch.autograd.grad(R, E)
        out.update(increments=n_inc, nodes=nodes.numpy(), elements=elements.numpy(), E=E.detach().numpy(),
                   u=u.detach().numpy(), f=f.detach().numpy(), sigma=s.detach().numpy(), reaction=R.detach().numpy(),
                   grad_E=gE.numpy(), t_fwd=t1 - t0, t_adj=time.perf_counter() - t1, torch_version=torch.__version__)
        print(f"{n_inc} increments: ok, reaction {float(R):.12g}", flush=True)
        break
    np.savez_compressed(OUT / name, **out)

def make_assembly(tf):
    """Assemblies of coupled parts (assembly.py), solved by the reference with
    spsolve: two tied Hexa1 blocks (with intermediate increments), a cube
    driven by a 3D reference point's moment, a tied Tria1 shell plate with the
    thickness gradient of the tip work, a Hexa2 solid beam continued by a
    shell, a conducting cube held by a thermal reference point, and a Quad1
    plate turned by a 2D reference point."""
    from torchfem import Assembly, Planar, ReferencePoint, ReferencePointHeat, Shell, Solid, SolidHeat
    from torchfem.elements import linear_to_quadratic
    from torchfem.materials import (IsotropicConductivity3D, IsotropicElasticity3D,
                                    IsotropicElasticityPlaneStress)
    from torchfem.mesh import cube_hexa, rect_quad, rect_tri

    E, NU = 1000.0, 0.3
    SOLID = IsotropicElasticity3D(E, NU)
    PLANE = IsotropicElasticityPlaneStress(E, NU)
    L, B, T, P = 10.0, 1.0, 0.4, 0.05
    out = {}

    def block(z0, z1):
        nodes = torch.tensor([[x, y, z] for z in (z0, z1) for y in (0.0, 1.0) for x in (0.0, 1.0)])
        return nodes, torch.tensor([[0, 1, 3, 2, 4, 5, 7, 6]])

    def plate(x0, Lx, Nx):
        nodes, elements = rect_tri(Nx, 3, Lx, B)
        nodes = nodes + torch.tensor([x0, 0.0])
        return torch.cat([nodes, torch.zeros(len(nodes), 1)], dim=1), elements

    # two tied blocks, five increments
    n_a, e_a = block(0.0, 1.0)
    n_b, e_b = block(1.0, 2.0)
    a, b = Solid(n_a, e_a, SOLID), Solid(n_b, e_b, SOLID)
    a.constraints[n_a[:, 2] == 0.0] = True
    b.forces[n_b[:, 2] == 2.0, 2] = 25.0
    b.forces[n_b[:, 2] == 2.0, 0] = 5.0
    asm = Assembly([a, b])
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    u, f, s, _, _ = asm.solve(increments=torch.linspace(0.0, 1.0, 5), return_intermediate=True, method="spsolve")
    for j in range(2):
        out[f"blocks_u{j}"], out[f"blocks_f{j}"], out[f"blocks_s{j}"] = u[j].numpy(), f[j].numpy(), s[j].numpy()

    # a cube turned by a reference point
    nodes, elements = cube_hexa(3, 3, 3)
    solid = Solid(nodes, elements, SOLID)
    solid.constraints[nodes[:, 2] == 0.0] = True
    point = ReferencePoint([0.5, 0.5, 2.0])
    point.forces[0, 3] = 50.0
    point.forces[0, 1] = 7.0
    asm = Assembly([solid, point])
    asm.coupling(solid, nodes[:, 2] == nodes[:, 2].max(), point)
    u, f, s, _, _ = asm.solve(method="spsolve")
    out.update(rp_u0=u[0].numpy(), rp_u1=u[1].numpy(), rp_f0=f[0].numpy(), rp_f1=f[1].numpy(), rp_s0=s[0].numpy())

    # a tied shell plate and the thickness gradient of its tip work
    n_sa, e_sa = plate(0.0, L / 2, 5)
    n_sb, e_sb = plate(L / 2, L / 2, 5)

    def work(thickness):
        sa = Shell(n_sa, e_sa, PLANE, thickness=thickness)
        sb = Shell(n_sb, e_sb, PLANE, thickness=T)
        sa.constraints[n_sa[:, 0] == 0.0] = True
        sb.forces[n_sb[:, 0] == L, 2] = P / (n_sb[:, 0] == L).sum()
        asm = Assembly([sa, sb])
        asm.coupling(sb, n_sb[:, 0] == L / 2, sa, n_sa[:, 0] == L / 2)
        u, f, _, _, _ = asm.solve(differentiable_parameters=thickness, method="spsolve")
        return torch.inner(sb.forces.ravel(), u[1].ravel()), u, f

    th = torch.full((len(e_sa),), T, requires_grad=True)
    w, u, f = work(th)
    (g,) = torch.autograd.grad(w, th)
    out.update(shell_na=n_sa.numpy(), shell_ea=e_sa.numpy(), shell_nb=n_sb.numpy(), shell_eb=e_sb.numpy(),
               shell_u0=u[0].detach().numpy(), shell_u1=u[1].detach().numpy(), shell_f1=f[1].detach().numpy(),
               shell_work=w.detach().numpy(), shell_grad=g.numpy())

    # a Hexa2 solid beam continued by a shell
    n_s, e_s = linear_to_quadratic(*cube_hexa(11, 3, 3, L / 2, B, T))
    n_s = n_s - torch.tensor([0.0, 0.0, T / 2])
    solid = Solid(n_s, e_s, SOLID)
    solid.constraints[n_s[:, 0] == 0.0] = True
    n_h, e_h = plate(L / 2, L / 2, 11)
    shell = Shell(n_h, e_h, PLANE, thickness=T)
    shell.forces[n_h[:, 0] == L, 2] = P / (n_h[:, 0] == L).sum()
    asm = Assembly([solid, shell])
    asm.coupling(solid, n_s[:, 0] == L / 2, shell, n_h[:, 0] == L / 2)
    u, f, _, _, _ = asm.solve(method="spsolve")
    out.update(ss_ns=n_s.numpy(), ss_es=e_s.numpy(), ss_nh=n_h.numpy(), ss_eh=e_h.numpy(),
               ss_u0=u[0].numpy(), ss_u1=u[1].numpy())

    # a conducting cube held isothermal on top by a thermal point
    nodes, elements = cube_hexa(4, 4, 4)
    heat = SolidHeat(nodes, elements, IsotropicConductivity3D(1.0))
    heat.constraints[nodes[:, 2] == 0.0] = True
    heat.heat_flux[nodes[:, 0] == 0.0, 0] = 0.1
    hp = ReferencePointHeat([0.5, 0.5, 1.5])
    hp.heat_flux[0, 0] = 4.0
    asm = Assembly([heat, hp])
    asm.coupling(heat, nodes[:, 2] == 1.0, hp)
    T_, q, flux, _, _ = asm.solve(method="spsolve")
    out.update(heat_T0=T_[0].numpy(), heat_T1=T_[1].numpy(), heat_q0=q[0].numpy(), heat_q1=q[1].numpy(),
               heat_flux0=flux[0].numpy())

    # a Quad1 plate turned by a 2D reference point
    nodes, elements = rect_quad(5, 5)
    pl = Planar(nodes, elements, PLANE)
    pl.constraints[nodes[:, 1] == 0.0] = True
    p2 = ReferencePoint([0.5, 1.5])
    p2.forces[0, 2] = 20.0
    p2.forces[0, 0] = 3.0
    asm = Assembly([pl, p2])
    asm.coupling(pl, nodes[:, 1] == 1.0, p2)
    u, f, s, _, _ = asm.solve(method="spsolve")
    out.update(planar_u0=u[0].numpy(), planar_u1=u[1].numpy(), planar_f1=f[1].numpy(), planar_s0=s[0].numpy())
    np.savez_compressed(OUT / "assembly_cases.npz", **out)


MAKERS = {
    "material_points": make_material_points,
    "c1": make_c1, "hexa_jitter3": make_hexa_jitter3, "patterns": make_patterns,
    "simp_small": lambda tf: make_simp(tf, 20, 10, "simp_20x10.npz"),
    "simp_full": lambda tf: make_simp(tf, 400, 200, "simp_400x200.npz", sample=20),
    "hyper": make_hyper, "plastic": make_plastic, "shell": make_shell,
    "plastic_full": lambda tf: make_plastic(tf, 256, 64, "plastic_ogrid_256x64.npz"),
    "hexa2": make_hexa2, "heat": make_heat, "heat_transient_grad": make_heat_transient_grad,
    "modes": make_modes, "assembly": make_assembly,
    "c2": make_c2, "c2_crosscheck": make_c2_crosscheck, "hyper_full": make_hyper_full, "hyper_mid": make_hyper_mid,
}
# targets that take minutes to an hour of CPU; run only when named
SLOW = {"c2", "c2_crosscheck", "hyper_full", "hyper_mid", "plastic_full", "simp_full"}


def main():
    import argparse
    import os

    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reference", default=os.environ.get("TORCHFEM_REFERENCE_SRC"),
                    help="the src folder of a torch-fem checkout (or TORCHFEM_REFERENCE_SRC)")
    ap.add_argument("targets", nargs="*")
    args = ap.parse_args()
    if not args.reference:
        ap.error("name the torch-fem src folder with --reference or TORCHFEM_REFERENCE_SRC")
    torch.set_default_dtype(torch.float64)
    tf = import_reference(args.reference)
    names = args.targets or [n for n in MAKERS if n not in SLOW]
    for name in names:
        MAKERS[name](tf)
    print("fixtures written to", OUT, names)


if __name__ == "__main__":
    main()
