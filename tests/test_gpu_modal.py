"""GPU modal analysis (FEM.solve_modes, base.py:1097-1129) against the
reference and the oracle.

- the reference's six lowest squared angular frequencies, mode shapes and
  d(sum omega^2)/d(E, rho) of a jittered 3^3 Hexa1 cube with per-element E
  and rho (modes_hexa_jitter3.npz, written by the reference itself): omega^2
  and the gradients to 1e-8 relative, mode shapes to 1e-7 up to sign;
- a jittered 8^3 cube (2,187 DOF) against the oracle's dense generalized
  eigensolve: ten modes and the gradients to 1e-8;
- a planar model with per-element thickness against central differences of
  omega^2.
"""

import numpy as np
import pytest
import torch

from oracle import modal_oracle as MO
from torchfem_gb300 import Planar, Solid, mesh
from torchfem_gb300.materials import IsotropicElasticity3D, IsotropicElasticityPlaneStress

pytestmark = pytest.mark.gpu

RTOL = 1e-8


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = np.asarray(b)
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_modes_vs_reference(cuda, golden):
    g = golden("modes_hexa_jitter3.npz")
    E = torch.tensor(g["E"], requires_grad=True)
    rho = torch.tensor(g["rho"], requires_grad=True)
    m = Solid(torch.tensor(g["nodes"], device=cuda), torch.tensor(g["elements"], device=cuda),
              IsotropicElasticity3D(E, 0.3, rho))
    m.constraints = torch.tensor(g["con"], device=cuda)
    omega_sq, modes = m.solve_modes(6)
    assert omega_sq.shape == (6,) and modes.shape == (6, 64, 3) and not modes.requires_grad
    assert rel(omega_sq, g["omega_sq"]) < RTOL
    sign = np.sign(np.einsum("mnd,mnd->m", modes.cpu().numpy(), g["modes"]))
    assert rel(modes.cpu().numpy() * sign[:, None, None], g["modes"]) < 1e-7
    gE, gr = torch.autograd.grad(omega_sq.sum(), (E, rho))
    assert rel(gE, g["g_E"]) < RTOL
    assert rel(gr, g["g_rho"]) < RTOL


def test_modes_larger_cube_vs_oracle(cuda):
    n = 8
    nodes, el = mesh.cube_hexa(n + 1, n + 1, n + 1)
    gen = torch.Generator().manual_seed(4)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    nodes = nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen, dtype=torch.float64) * 2 - 1) * (0.1 / n)
    E0 = 1000.0 * (1.0 + 0.5 * torch.rand(len(el), generator=gen, dtype=torch.float64))
    r0 = 1.0 + torch.rand(len(el), generator=gen, dtype=torch.float64)
    con = torch.zeros(nodes.shape, dtype=torch.bool)
    con[nodes[:, 0] == 0.0, :] = True
    E, rho = E0.clone().requires_grad_(True), r0.clone().requires_grad_(True)
    m = Solid(nodes.to(cuda), el.to(cuda), IsotropicElasticity3D(E, 0.3, rho))
    m.constraints = con.to(cuda)
    omega_sq, _ = m.solve_modes(10)
    lam, _, gE_o, gr_o = MO.solve_modes(nodes.numpy(), el.numpy(), E0.numpy(), 0.3, r0.numpy(), con.numpy(), 10)
    assert rel(omega_sq, lam) < RTOL
    gE, gr = torch.autograd.grad(omega_sq.sum(), (E, rho))
    assert rel(gE, gE_o) < RTOL
    assert rel(gr, gr_o) < RTOL


def test_modes_planar_thickness_central_differences(cuda):
    nodes, el = mesh.rect_quad(17, 9, 2.0, 1.0)
    gen = torch.Generator().manual_seed(8)
    t0 = 0.5 + torch.rand(len(el), generator=gen, dtype=torch.float64)
    con = torch.zeros(nodes.shape, dtype=torch.bool)
    con[nodes[:, 0] == 0.0, :] = True
    w = torch.tensor([1.0, 0.5, 0.25, 0.125], dtype=torch.float64)

    def omega(t):
        m = Planar(nodes.to(cuda), el.to(cuda), IsotropicElasticityPlaneStress(1000.0, 0.3, 2.0), thickness=t)
        m.constraints = con.to(cuda)
        return (w * m.solve_modes(4)[0].cpu()).sum()

    t = t0.clone().to(cuda).requires_grad_(True)
    (gt,) = torch.autograd.grad(omega(t), t)
    for e in torch.argsort(gt.abs(), descending=True)[:3].tolist():
        h = 1e-5 * float(t0[e])
        tp, tm = t0.clone(), t0.clone()
        tp[e] += h
        tm[e] -= h
        with torch.no_grad():
            fd = (float(omega(tp.to(cuda))) - float(omega(tm.to(cuda)))) / (2 * h)
        assert abs(fd - float(gt[e])) <= 1e-6 * abs(float(gt[e])), (e, fd, float(gt[e]))
