"""GPU tests of the heat-conduction path (SolidHeat / PlanarHeat).

Steady solves, their adjoint gradients and the Crank-Nicolson time
integration against golden vectors produced by the reference itself
(tests/golden/heat_cases.npz) and against the CPU oracle
(oracle/heat_oracle.py) on a larger mesh, in FP64 and in mixed precision
(FP32 multigrid-preconditioned CG with FP64 residual replacement; one DOF per
node, the constant near-null vector): temperatures, heat fluxes and
gradients agree to 1e-8 relative (CG stopped at 1e-12).
"""

import numpy as np
import pytest
import torch

from oracle import heat_oracle as H
from torchfem_gb300 import PlanarHeat, SolidHeat, mesh
from torchfem_gb300.materials import (IsotropicConductivity2D, IsotropicConductivity3D,
                                      OrthotropicConductivity2D)

pytestmark = pytest.mark.gpu

RTOL = 1e-8


def rel(a, b):
    a = a.detach().cpu().double().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a.reshape(b.shape) - b).max() / max(np.abs(b).max(), 1e-300))


def test_solid_heat_solve_and_gradients(cuda, golden):
    g = golden("heat_cases.npz")
    nodes = torch.tensor(g["solid_nodes"], device=cuda)
    el = torch.tensor(g["solid_elements"], device=cuda)
    kappa = torch.tensor(g["solid_kappa"], device=cuda, requires_grad=True)
    model = SolidHeat(nodes, el, IsotropicConductivity3D(kappa))
    model.constraints = torch.tensor(g["solid_con"], device=cuda)
    model.temperatures = torch.tensor(g["solid_temp"], device=cuda)
    q = torch.tensor(g["solid_q"], device=cuda, requires_grad=True)
    model.heat_flux = q
    T, f, flux, grad, state = model.solve(stol=1e-12, differentiable_parameters=(kappa, q))
    assert T.shape == (len(nodes), 1) and flux.shape == (len(el), 3) and state.shape == (len(el), 0)
    for name, out in (("T", T), ("f", f), ("flux", flux), ("grad", grad)):
        assert rel(out, g[f"solid_{name}"]) < RTOL, name
    L = torch.inner(f.ravel(), T.ravel())
    assert rel(L, g["solid_L"]) < RTOL
    gk, gq = torch.autograd.grad(L, (kappa, q))
    assert rel(gk, g["solid_g_kappa"]) < RTOL
    assert rel(gq, g["solid_g_q"]) < RTOL
    assert rel(model.k0(), g["solid_k0"]) < 1e-13


def test_planar_heat_thickness_gradient(cuda, golden):
    g = golden("heat_cases.npz")
    nodes = torch.tensor(g["planar_nodes"], device=cuda)
    el = torch.tensor(g["planar_elements"], device=cuda)
    rho = torch.tensor(g["planar_rho"], device=cuda, requires_grad=True)
    model = PlanarHeat(nodes, el, IsotropicConductivity2D(kappa=400.0))
    model.thickness = rho**3
    model.constraints = torch.tensor(g["planar_con"], device=cuda)
    model.heat_flux = torch.tensor(g["planar_q"], device=cuda)
    T, f, flux, _, _ = model.solve(stol=1e-12, differentiable_parameters=rho)
    assert rel(T, g["planar_T"]) < RTOL and rel(f, g["planar_f"]) < RTOL and rel(flux, g["planar_flux"]) < RTOL
    L = torch.inner(f.ravel(), T.ravel())
    (g_rho,) = torch.autograd.grad(L, rho)
    assert rel(L, g["planar_L"]) < RTOL
    assert rel(g_rho, g["planar_g_rho"]) < RTOL


def test_planar_heat_rotated_orthotropic(cuda, golden):
    g = golden("heat_cases.npz")
    nodes = torch.tensor(g["planar_nodes"])
    el = torch.tensor(g["planar_elements"])
    c, s = np.cos(0.5), np.sin(0.5)
    R = torch.tensor([[c, -s], [s, c]])
    model = PlanarHeat(nodes, el, OrthotropicConductivity2D(50.0, 5.0).rotate(R), thickness=0.1)
    model.constraints = torch.tensor(g["ortho_con"])
    model.temperatures = torch.tensor(g["ortho_temp"])
    T, f, flux, grad, _ = model.solve(stol=1e-12)
    assert T.device.type == "cpu"  # results come back on the device of the nodes
    for name, out in (("T", T), ("f", f), ("flux", flux), ("grad", grad), ("k0", model.k0())):
        assert rel(out, g[f"ortho_{name}"]) < RTOL, name


def _plate():
    model = PlanarHeat(*mesh.rect_quad(5, 5, 1.0, 1.0), IsotropicConductivity2D(kappa=400.0, rho=1.0e5))
    west = torch.isclose(model.nodes[:, 0], model.nodes[:, 0].min())
    east = torch.isclose(model.nodes[:, 0], model.nodes[:, 0].max())
    model.constraints[west | east] = True
    model.temperatures[west, 0] = 5.0
    model.temperatures[east, 0] = 20.0
    return model


def test_time_integration_heated_plate(cuda, golden):
    g = golden("heat_cases.npz")
    model = _plate()
    assert rel(model.integrate_mass(), g["plate_mass"]) < 1e-13
    temp, rfl, flux, grad, state = model.time_integration(torch.tensor(g["plate_t"]), delta_t=1.0, stol=1e-12)
    assert temp.shape == (5, 25, 1) and flux.shape == (5, 16, 2) and state.shape == (5, 16, 0)
    assert rel(temp, g["plate_temp"]) < RTOL
    assert rel(rfl, g["plate_f"]) < RTOL
    assert rel(flux, g["plate_flux"]) < RTOL
    assert rel(grad, g["plate_grad"]) < RTOL
    # late start, per-point outputs: integration still starts at t = 0
    temp, rfl, flux, grad, _ = _plate().time_integration(torch.tensor(g["late_t"]), delta_t=0.5, stol=1e-12,
                                                         aggregate_integration_points=False)
    assert flux.shape == (2, 4, 16, 2)
    for name, out in (("temp", temp), ("f", rfl), ("flux", flux), ("grad", grad)):
        assert rel(out, g[f"late_{name}"]) < RTOL, name


def test_time_integration_sparse_output_matches_dense(cuda):
    """Fewer output times do not change the internal stepping
    (tests/test_time_integration.py of the reference)."""
    dense_t = torch.arange(0.0, 3.0 + 0.25, 0.25)
    dense, *_ = _plate().time_integration(dense_t, 0.25, stol=1e-12)
    sparse_t = torch.tensor([0.0, 0.5, 2.0, 3.0])
    sparse, *_ = _plate().time_integration(sparse_t, 0.25, stol=1e-12)
    rows = torch.searchsorted(dense_t.contiguous(), sparse_t)
    assert torch.allclose(sparse, dense[rows], atol=1e-9)


def _transient_grad_model(g, cuda, kappa, rho, q):
    nodes = torch.tensor(g["nodes"], device=cuda)
    el = torch.tensor(g["elements"], device=cuda)
    model = PlanarHeat(nodes, el, IsotropicConductivity2D(kappa, rho))
    model.constraints = torch.tensor(g["con"], device=cuda)
    model.temperatures = torch.tensor(g["temp_bc"], device=cuda)
    model.heat_flux = q
    return model


def test_time_integration_gradients_vs_reference(cuda, golden):
    """Gradients through Heat.time_integration: per-element conductivity and
    density and the nodal heat sources, loss sum_k c_k . T(t_k) on a grid of
    unequal steps, against the reference's autograd through its own
    integration (heat_transient_grad.npz), to 1e-8."""
    g = golden("heat_transient_grad.npz")
    kappa = torch.tensor(g["kappa"], device=cuda, requires_grad=True)
    rho = torch.tensor(g["rho"], device=cuda, requires_grad=True)
    q = torch.tensor(g["q"], device=cuda, requires_grad=True)
    model = _transient_grad_model(g, cuda, kappa, rho, q)
    temp, *_ = model.time_integration(torch.tensor(g["t_out"]), delta_t=float(g["delta_t"]), stol=1e-13,
                                      differentiable_parameters=(kappa, rho, q))
    assert rel(temp, g["temp"]) < RTOL
    L = (torch.tensor(g["c"], device=cuda) * temp).sum()
    assert rel(L, g["L"]) < RTOL
    gk, gr, gq = torch.autograd.grad(L, (kappa, rho, q))
    assert rel(gk, g["g_kappa"]) < RTOL
    assert rel(gr, g["g_rho"]) < RTOL
    assert rel(gq, g["g_q"]) < RTOL


def test_time_integration_flux_and_thickness_gradients_central_differences(cuda, golden):
    """A loss on every output of time_integration (temperatures, internal
    heat fluxes and element fluxes) differentiated w.r.t. conductivity,
    density and thickness, against central differences of the GPU path on
    the three most sensitive elements of each parameter."""
    g = golden("heat_transient_grad.npz")
    gen = torch.Generator().manual_seed(5)
    k0 = torch.tensor(g["kappa"])
    r0 = torch.tensor(g["rho"])
    t0 = 0.5 + torch.rand(len(k0), generator=gen, dtype=torch.float64)
    q = torch.tensor(g["q"], device=cuda)
    t_out = torch.tensor(g["t_out"])
    w = []

    def loss(kappa, rho, th, track):
        model = _transient_grad_model(g, cuda, kappa, rho, q)
        model.thickness = th
        temp, rfl, flux, _, _ = model.time_integration(t_out, delta_t=float(g["delta_t"]), stol=1e-13,
                                                       differentiable_parameters=(kappa, rho, th) if track else None)
        if not w:
            w.extend(torch.rand(x.shape, generator=gen, dtype=torch.float64).to(cuda) for x in (temp, rfl, flux))
        return (w[0] * temp).sum() + 1e-3 * (w[1] * rfl).sum() + 1e-3 * (w[2] * flux).sum()

    kappa, rho, th = (x.to(cuda).clone().requires_grad_(True) for x in (k0, r0, t0))
    grads = torch.autograd.grad(loss(kappa, rho, th, True), (kappa, rho, th))
    base = (k0, r0, t0)
    for which, gvec in enumerate(grads):
        for e in torch.argsort(gvec.abs(), descending=True)[:3].tolist():
            h = 1e-5 * float(base[which][e])
            vals = []
            for sgn in (1.0, -1.0):
                args = [b.clone() for b in base]
                args[which][e] += sgn * h
                with torch.no_grad():
                    vals.append(float(loss(*(a.to(cuda) for a in args), False)))
            fd = (vals[0] - vals[1]) / (2 * h)
            assert abs(fd - float(gvec[e])) <= 1e-6 * abs(float(gvec[e])), (which, e, fd, float(gvec[e]))


def test_solid_heat_larger_mesh_against_oracle(cuda):
    """16^3 jittered Hexa1 cube, conductivity varying per element: temperatures
    and the compliance gradient against the oracle."""
    n = 16
    nodes, el = mesh.cube_hexa(n + 1, n + 1, n + 1)
    gen = torch.Generator().manual_seed(7)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    nodes = nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen, dtype=torch.float64) * 2 - 1) * 0.1 / n
    kappa = 1.0 + torch.rand(len(el), generator=gen, dtype=torch.float64)
    kappa_g = kappa.clone().to(cuda).requires_grad_(True)
    model = SolidHeat(nodes.to(cuda), el.to(cuda), IsotropicConductivity3D(kappa_g))
    model.constraints[(nodes[:, 0] == 0.0).to(cuda)] = True
    model.heat_flux[:] = 1.0 / len(nodes)
    T, f, _, _, _ = model.solve(stol=1e-12, differentiable_parameters=kappa_g)
    L = torch.inner(f.ravel(), T.ravel())
    (gk,) = torch.autograd.grad(L, kappa_g)
    om = H.HeatModel(nodes.numpy(), el.numpy(), kappa.numpy()[:, None, None] * np.eye(3))
    To, fo, _, _ = om.solve(np.full(len(nodes), 1.0 / len(nodes)), (nodes[:, 0] == 0.0).numpy())
    gko, _, _ = om.compliance_grads(To, fo)
    assert rel(T, To) < RTOL and rel(f, fo) < RTOL
    assert rel(gk, np.einsum("Eaa->E", gko)) < RTOL


def _jittered_heat_cube(n, seed=7):
    nodes, el = mesh.cube_hexa(n + 1, n + 1, n + 1)
    gen = torch.Generator().manual_seed(seed)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    nodes = nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen, dtype=torch.float64) * 2 - 1) * 0.1 / n
    kappa = 1.0 + torch.rand(len(el), generator=gen, dtype=torch.float64)
    return nodes, el, kappa


def test_solid_heat_mixed_multigrid_vs_reference(cuda, golden):
    """The reference's SolidHeat case through FP32 multigrid-preconditioned CG
    with FP64 residual replacement: temperatures, fluxes and gradients to
    1e-8 of the reference's FP64 results."""
    g = golden("heat_cases.npz")
    kappa = torch.tensor(g["solid_kappa"], device=cuda, requires_grad=True)
    model = SolidHeat(torch.tensor(g["solid_nodes"], device=cuda), torch.tensor(g["solid_elements"], device=cuda),
                      IsotropicConductivity3D(kappa))
    model.constraints = torch.tensor(g["solid_con"], device=cuda)
    model.temperatures = torch.tensor(g["solid_temp"], device=cuda)
    q = torch.tensor(g["solid_q"], device=cuda, requires_grad=True)
    model.heat_flux = q
    T, f, flux, grad, _ = model.solve(stol=1e-12, precision="mixed", differentiable_parameters=(kappa, q))
    assert model.last_solve.system.amg is not None
    for name, out in (("T", T), ("f", f), ("flux", flux), ("grad", grad)):
        assert rel(out, g[f"solid_{name}"]) < RTOL, name
    L = torch.inner(f.ravel(), T.ravel())
    gk, gq = torch.autograd.grad(L, (kappa, q))
    assert rel(gk, g["solid_g_kappa"]) < RTOL
    assert rel(gq, g["solid_g_q"]) < RTOL


def test_planar_heat_mixed_thickness_gradient(cuda, golden):
    g = golden("heat_cases.npz")
    rho = torch.tensor(g["planar_rho"], device=cuda, requires_grad=True)
    model = PlanarHeat(torch.tensor(g["planar_nodes"], device=cuda), torch.tensor(g["planar_elements"], device=cuda),
                       IsotropicConductivity2D(kappa=400.0))
    model.thickness = rho**3
    model.constraints = torch.tensor(g["planar_con"], device=cuda)
    model.heat_flux = torch.tensor(g["planar_q"], device=cuda)
    T, f, _, _, _ = model.solve(stol=1e-12, precision="mixed", differentiable_parameters=rho)
    L = torch.inner(f.ravel(), T.ravel())
    (g_rho,) = torch.autograd.grad(L, rho)
    assert rel(T, g["planar_T"]) < RTOL
    assert rel(g_rho, g["planar_g_rho"]) < RTOL


def test_heat_multigrid_hierarchy_matches_oracle(cuda):
    """One DOF per node: the constant near-null vector, aggregation bit for
    bit and the tentative prolongator against the oracle, level sizes of the
    oracle's hierarchy, and the solution against the oracle's FP64 solve."""
    from test_gpu_amg import fetch

    from oracle import amg_oracle as AO

    nodes, el, kappa = _jittered_heat_cube(14)
    model = SolidHeat(nodes, el, IsotropicConductivity3D(kappa))
    x0 = nodes[:, 0] == 0.0
    model.constraints[x0] = True
    model.heat_flux[:] = 1.0 / len(nodes)
    T, f, _, _, _ = model.solve(stol=1e-12, precision="mixed")
    assert max(model.last_solve.iterations) <= 40
    om = H.HeatModel(nodes.numpy(), el.numpy(), kappa.numpy()[:, None, None] * np.eye(3))
    To, fo, _, _ = om.solve(np.full(len(nodes), 1.0 / len(nodes)), x0.numpy())
    assert rel(T, To) < RTOL and rel(f, fo) < RTOL

    amg = model.last_solve.system.amg
    levels = amg.levels()
    assert levels[0].block == 1 and levels[1].block == 1
    dm = model.device_mesh
    n = len(nodes)
    con = x0.numpy()
    ptr = dm.nbr_ptr.cpu().numpy()
    idx = dm.nbr.cpu().numpy().astype(np.int64)
    agg = fetch(amg.lib, levels[0].agg, n, torch.int32)
    agg_o, na_o = AO.aggregate(ptr, idx, ~con)
    assert levels[0].n_agg == na_o and np.array_equal(agg, agg_o)
    T_o, _ = AO.tentative(agg_o, na_o, 1, 1, coords=nodes.numpy(), con=con)
    Tg = fetch(amg.lib, levels[0].tval, n, torch.float32).reshape(n, 1, 1)
    assert np.abs(Tg - T_o).max() <= 1e-6 * np.abs(T_o).max()
    K = om.matrix(np.nonzero(con)[0]).tocsr()
    lo = AO.hierarchy(K, nodes.numpy(), con, 1, rhos=[lv.rho for lv in levels[:-1]])
    assert [lv.n for lv in levels] == [x.A.shape[0] // x.b for x in lo]


def test_heat_mixed_needs_multigrid(cuda):
    model = _plate()
    with pytest.raises(NotImplementedError, match="multigrid"):
        model.solve(precision="mixed", preconditioner="jacobi")
