"""GPU tests of Assembly: parts coupled by kinematic constraints.

Against the reference's own results (tests/golden/assembly_cases.npz, made
by make_golden.py assembly with spsolve): tied Hexa1 blocks over five
increments, a cube turned by a 3D reference point, a tied Tria1 shell plate
with the thickness gradient of its tip work, a Hexa2 beam continued by a
shell, a conducting cube held by a thermal point, and a Quad1 plate turned by
a 2D point; displacements, forces, fluxes and the gradient to 1e-8 relative
(CG to stol 1e-12).  Then the reference's own physical checks
(tests/test_assembly.py of torch-fem): a tie reproduces the monolithic model,
coupled nodes follow the rigid relation exactly, a part carried by a point
stays unstrained, dofs=[2] leaves the rest free, incremental loading equals
one step, an uncoupled part solves alone, the gradient matches central
differences.
"""

import numpy as np
import pytest
import torch

from torchfem_gb300 import Assembly, Planar, ReferencePoint, ReferencePointHeat, Shell, Solid, SolidHeat, mesh
from torchfem_gb300.materials import (IsotropicConductivity3D, IsotropicElasticity3D,
                                      IsotropicElasticityPlaneStress)

pytestmark = pytest.mark.gpu

RTOL = 1e-8
E, NU = 1000.0, 0.3
SOLID = IsotropicElasticity3D(E, NU)
PLANE = IsotropicElasticityPlaneStress(E, NU)
L, B, T, P = 10.0, 1.0, 0.4, 0.05
STOL = 1e-12


def rel(a, b):
    a = a.detach().cpu().double().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().double().numpy() if torch.is_tensor(b) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _block(z0, z1):
    nodes = torch.tensor([[x, y, z] for z in (z0, z1) for y in (0.0, 1.0) for x in (0.0, 1.0)],
                         dtype=torch.float64)
    return nodes, torch.tensor([[0, 1, 3, 2, 4, 5, 7, 6]])


def _t(a):
    return torch.as_tensor(a)


# ------------------------------------------------------- reference parity --
def test_tied_blocks_over_increments_vs_reference(cuda, golden):
    g = golden("assembly_cases.npz")
    n_a, e_a = _block(0.0, 1.0)
    n_b, e_b = _block(1.0, 2.0)
    a, b = Solid(n_a, e_a, SOLID), Solid(n_b, e_b, SOLID)
    a.constraints[n_a[:, 2] == 0.0] = True
    b.forces[n_b[:, 2] == 2.0, 2] = 25.0
    b.forces[n_b[:, 2] == 2.0, 0] = 5.0
    asm = Assembly([a, b])
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    u, f, s, _, _ = asm.solve(increments=torch.linspace(0.0, 1.0, 5), return_intermediate=True, stol=STOL)
    for j in range(2):
        assert rel(u[j], g[f"blocks_u{j}"]) < RTOL
        assert rel(f[j], g[f"blocks_f{j}"]) < RTOL
        assert rel(s[j], g[f"blocks_s{j}"]) < RTOL


def test_reference_point_moment_vs_reference(cuda, golden):
    g = golden("assembly_cases.npz")
    nodes, elements = mesh.cube_hexa(3, 3, 3)
    solid = Solid(nodes, elements, SOLID)
    solid.constraints[nodes[:, 2] == 0.0] = True
    point = ReferencePoint([0.5, 0.5, 2.0])
    point.forces[0, 3] = 50.0
    point.forces[0, 1] = 7.0
    asm = Assembly([solid, point])
    top = nodes[:, 2] == nodes[:, 2].max()
    asm.coupling(solid, top, point)
    u, f, s, _, _ = asm.solve(stol=STOL)
    assert rel(u[0], g["rp_u0"]) < RTOL and rel(u[1], g["rp_u1"]) < RTOL
    assert rel(f[0], g["rp_f0"]) < RTOL and rel(f[1], g["rp_f1"]) < RTOL
    assert rel(s[0], g["rp_s0"]) < RTOL
    # coupled nodes follow the rigid relation exactly (to rounding)
    u_p, theta = u[1][0, :3], u[1][0, 3:]
    expected = u_p + torch.cross(theta.expand(int(top.sum()), 3), nodes[top] - point.nodes[0], dim=-1)
    assert torch.allclose(u[0][top], expected, rtol=1e-12, atol=1e-14)
    assert float(f[1][0, 3]) == pytest.approx(50.0, rel=1e-9)


def _shell_work(g, thickness):
    n_sa, e_sa, n_sb, e_sb = (_t(g[k]) for k in ("shell_na", "shell_ea", "shell_nb", "shell_eb"))
    sa = Shell(n_sa, e_sa, PLANE, thickness=thickness)
    sb = Shell(n_sb, e_sb, PLANE, thickness=T)
    sa.constraints[n_sa[:, 0] == 0.0] = True
    sb.forces[n_sb[:, 0] == L, 2] = P / (n_sb[:, 0] == L).sum()
    asm = Assembly([sa, sb])
    asm.coupling(sb, n_sb[:, 0] == L / 2, sa, n_sa[:, 0] == L / 2)
    u, f, _, _, _ = asm.solve(differentiable_parameters=thickness, stol=STOL)
    return torch.inner(sb.forces.ravel().to(u[1].dtype), u[1].ravel()), u, f


def test_tied_shell_and_thickness_gradient_vs_reference(cuda, golden):
    g = golden("assembly_cases.npz")
    th = torch.full((len(g["shell_ea"]),), T, dtype=torch.float64, requires_grad=True)
    w, u, f = _shell_work(g, th)
    (gt,) = torch.autograd.grad(w, th)
    assert rel(u[0], g["shell_u0"]) < RTOL and rel(u[1], g["shell_u1"]) < RTOL
    assert rel(f[1], g["shell_f1"]) < RTOL
    assert abs(float(w.detach()) - float(g["shell_work"])) <= RTOL * abs(float(g["shell_work"]))
    assert rel(gt, g["shell_grad"]) < 1e-7


def test_shell_gradient_matches_central_differences(cuda, golden):
    g = golden("assembly_cases.npz")
    th = torch.full((len(g["shell_ea"]),), T, dtype=torch.float64, requires_grad=True)
    (gt,) = torch.autograd.grad(_shell_work(g, th)[0], th)
    h = 1e-4
    for i in (0, 3, len(th) - 1):
        plus, minus = th.detach().clone(), th.detach().clone()
        plus[i] += h
        minus[i] -= h
        fd = (_shell_work(g, plus)[0] - _shell_work(g, minus)[0]) / (2 * h)
        assert float(gt[i]) == pytest.approx(float(fd), rel=1e-5, abs=1e-10)


def test_solid_continued_by_shell_vs_reference(cuda, golden):
    g = golden("assembly_cases.npz")
    n_s, e_s, n_h, e_h = (_t(g[k]) for k in ("ss_ns", "ss_es", "ss_nh", "ss_eh"))
    solid = Solid(n_s, e_s, SOLID)
    solid.constraints[n_s[:, 0] == 0.0] = True
    shell = Shell(n_h, e_h, PLANE, thickness=T)
    shell.forces[n_h[:, 0] == L, 2] = P / (n_h[:, 0] == L).sum()
    asm = Assembly([solid, shell])
    asm.coupling(solid, n_s[:, 0] == L / 2, shell, n_h[:, 0] == L / 2)
    u, _, _, _, _ = asm.solve(stol=STOL)
    assert rel(u[0], g["ss_u0"]) < RTOL and rel(u[1], g["ss_u1"]) < RTOL
    tip = u[1][n_h[:, 0] == L][:, 2].mean()
    assert float(tip) == pytest.approx(P * L**3 / (3 * E * B * T**3 / 12), rel=0.02)


def test_thermal_point_vs_reference(cuda, golden):
    g = golden("assembly_cases.npz")
    nodes, elements = mesh.cube_hexa(4, 4, 4)
    heat = SolidHeat(nodes, elements, IsotropicConductivity3D(1.0))
    heat.constraints[nodes[:, 2] == 0.0] = True
    heat.heat_flux[nodes[:, 0] == 0.0, 0] = 0.1
    hp = ReferencePointHeat([0.5, 0.5, 1.5])
    hp.heat_flux[0, 0] = 4.0
    asm = Assembly([heat, hp])
    asm.coupling(heat, nodes[:, 2] == 1.0, hp)
    Tt, q, flux, _, _ = asm.solve(stol=STOL)
    assert rel(Tt[0], g["heat_T0"]) < RTOL and rel(Tt[1], g["heat_T1"]) < RTOL
    assert rel(q[0], g["heat_q0"]) < RTOL and rel(q[1], g["heat_q1"]) < RTOL
    assert rel(flux[0], g["heat_flux0"]) < RTOL


def test_planar_point_vs_reference(cuda, golden):
    g = golden("assembly_cases.npz")
    nodes, elements = mesh.rect_quad(5, 5)
    pl = Planar(nodes, elements, PLANE)
    pl.constraints[nodes[:, 1] == 0.0] = True
    p2 = ReferencePoint([0.5, 1.5])
    p2.forces[0, 2] = 20.0
    p2.forces[0, 0] = 3.0
    asm = Assembly([pl, p2])
    top = nodes[:, 1] == 1.0
    asm.coupling(pl, top, p2)
    u, f, s, _, _ = asm.solve(stol=STOL)
    assert rel(u[0], g["planar_u0"]) < RTOL and rel(u[1], g["planar_u1"]) < RTOL
    assert rel(f[1], g["planar_f1"]) < RTOL and rel(s[0], g["planar_s0"]) < RTOL
    u_p, theta = u[1][0, :2], u[1][0, 2]
    r = nodes[top] - p2.nodes[0]
    assert torch.allclose(u[0][top], u_p + theta * torch.stack([-r[:, 1], r[:, 0]], dim=1), rtol=1e-12, atol=1e-14)


# ------------------------------------------------ the reference's physics --
def test_tie_reproduces_monolithic_solid(cuda):
    nodes = torch.tensor([[x, y, z] for z in (0.0, 1.0, 2.0) for y in (0.0, 1.0) for x in (0.0, 1.0)],
                         dtype=torch.float64)
    elements = torch.tensor([[0, 1, 3, 2, 4, 5, 7, 6], [4, 5, 7, 6, 8, 9, 11, 10]])
    ref = Solid(nodes, elements, SOLID)
    ref.constraints[nodes[:, 2] == 0.0] = True
    ref.forces[nodes[:, 2] == 2.0, 2] = 25.0
    u_ref = ref.solve(stol=STOL)[0]
    n_a, e_a = _block(0.0, 1.0)
    n_b, e_b = _block(1.0, 2.0)
    a, b = Solid(n_a, e_a, SOLID), Solid(n_b, e_b, SOLID)
    a.constraints[n_a[:, 2] == 0.0] = True
    b.forces[n_b[:, 2] == 2.0, 2] = 25.0
    asm = Assembly([a, b])
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    u, _, _, _, _ = asm.solve(stol=STOL)
    assert rel(u[0], u_ref[:8]) < RTOL and rel(u[1], u_ref[4:]) < RTOL
    # the tie is exact: the interface closes to the last bit
    assert torch.equal(u[1][n_b[:, 2] == 1.0], u[0][n_a[:, 2] == 1.0])


def test_tie_reproduces_monolithic_planar_and_shell(cuda):
    nodes, elements = mesh.rect_quad(5, 3, 2.0, 1.0)
    ref = Planar(nodes, elements, PLANE)
    ref.constraints[nodes[:, 0] == 0.0] = True
    ref.forces[nodes[:, 0] == 2.0, 1] = -1.0
    u_ref = ref.solve(stol=STOL)[0]
    n_a, e_a = mesh.rect_quad(3, 3, 1.0, 1.0)
    n_b, e_b = mesh.rect_quad(3, 3, 1.0, 1.0)
    n_b = n_b + torch.tensor([1.0, 0.0], dtype=torch.float64)
    a, b = Planar(n_a, e_a, PLANE), Planar(n_b, e_b, PLANE)
    a.constraints[n_a[:, 0] == 0.0] = True
    b.forces[n_b[:, 0] == 2.0, 1] = -1.0
    asm = Assembly([a, b])
    asm.coupling(b, n_b[:, 0] == 1.0, a, n_a[:, 0] == 1.0)
    u, _, _, _, _ = asm.solve(stol=STOL)
    assert rel(u[0], u_ref[nodes[:, 0] <= 1.0]) < RTOL and rel(u[1], u_ref[nodes[:, 0] >= 1.0]) < RTOL

    nodes, elements = mesh.strip_tria(21, 3, L, B)
    ref = Shell(nodes, elements, PLANE, thickness=T)
    ref.constraints[nodes[:, 0] == 0.0] = True
    ref.forces[nodes[:, 0] == L, 2] = P / (nodes[:, 0] == L).sum()
    u_ref = ref.solve(stol=STOL)[0]
    n_a, e_a = mesh.strip_tria(11, 3, L / 2, B)
    n_b, e_b = mesh.strip_tria(11, 3, L / 2, B)
    n_b = n_b + torch.tensor([L / 2, 0.0, 0.0], dtype=torch.float64)
    a = Shell(n_a, e_a, PLANE, thickness=T)
    b = Shell(n_b, e_b, PLANE, thickness=T)
    a.constraints[n_a[:, 0] == 0.0] = True
    b.forces[n_b[:, 0] == L, 2] = P / (n_b[:, 0] == L).sum()
    asm = Assembly([a, b])
    asm.coupling(b, n_b[:, 0] == L / 2, a, n_a[:, 0] == L / 2)
    u, _, _, _, _ = asm.solve(stol=STOL)
    assert rel(u[0], u_ref[nodes[:, 0] <= L / 2]) < 1e-7 and rel(u[1], u_ref[nodes[:, 0] >= L / 2]) < 1e-7


def test_whole_part_moves_without_stress(cuda):
    nodes, elements = mesh.cube_hexa(3, 3, 3)
    solid = Solid(nodes, elements, SOLID)
    point = ReferencePoint([0.5, 0.5, 0.5])
    point.constraints[0, :] = True
    point.displacements[0, :3] = torch.tensor([0.3, -0.2, 0.7])
    asm = Assembly([solid, point])
    asm.coupling(solid, torch.ones(len(nodes), dtype=torch.bool), point)
    u, _, flux, _, _ = asm.solve(stol=STOL)
    assert torch.allclose(u[0], torch.tensor([0.3, -0.2, 0.7], dtype=u[0].dtype).expand_as(u[0]), atol=1e-14)
    assert float(flux[0].abs().max()) < 1e-10


def test_subset_of_dofs_leaves_the_rest_free(cuda):
    nodes, elements = mesh.cube_hexa(3, 3, 3)
    top = nodes[:, 2] == nodes[:, 2].max()
    solid = Solid(nodes, elements, SOLID)
    solid.constraints[nodes[:, 2] == 0.0] = True
    point = ReferencePoint([0.5, 0.5, 2.0])
    point.constraints[0, :] = True
    point.displacements[0, 2] = 0.1
    asm = Assembly([solid, point])
    asm.coupling(solid, top, point, dofs=[2])
    u, _, _, _, _ = asm.solve(stol=STOL)
    assert torch.allclose(u[0][top][:, 2], torch.full((int(top.sum()),), 0.1, dtype=u[0].dtype), atol=1e-14)
    assert float(u[0][top][:, 0].max() - u[0][top][:, 0].min()) > 1e-3


def test_incremental_equals_single_step_and_intermediate(cuda):
    n_a, e_a = _block(0.0, 1.0)
    n_b, e_b = _block(1.0, 2.0)

    def solve(increments, **kw):
        a, b = Solid(n_a, e_a, SOLID), Solid(n_b, e_b, SOLID)
        a.constraints[n_a[:, 2] == 0.0] = True
        b.forces[n_b[:, 2] == 2.0, 2] = 25.0
        asm = Assembly([a, b])
        asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
        return asm.solve(increments=increments, stol=STOL, **kw)[0]

    single = solve(None)
    stepped = solve(torch.linspace(0.0, 1.0, 5))
    assert rel(single[0], stepped[0]) < RTOL and rel(single[1], stepped[1]) < RTOL
    inc = torch.linspace(0.0, 1.0, 4)
    every = solve(inc, return_intermediate=True)
    assert [x.shape[0] for x in every] == [4, 4]
    tip = every[1][:, n_b[:, 2] == 2.0, 2].mean(dim=1)
    assert torch.allclose(tip / tip[-1], inc.to(tip.dtype), atol=1e-12)


def test_uncoupled_part_solves_alone(cuda):
    n_a, e_a = _block(0.0, 1.0)
    a = Solid(n_a, e_a, SOLID)
    a.constraints[n_a[:, 2] == 0.0] = True
    a.forces[n_a[:, 2] == 1.0, 2] = 25.0
    alone = a.solve(stol=STOL)[0]
    b = Solid(n_a, e_a, SOLID)
    b.constraints[n_a[:, 2] == 0.0] = True
    b.forces[n_a[:, 2] == 1.0, 2] = 25.0
    u, _, _, _, _ = Assembly([b]).solve(stol=STOL)
    assert rel(u[0], alone) < RTOL


def test_thermal_tie_and_isothermal_point(cuda):
    nodes = torch.tensor([[x, y, z] for z in (0.0, 1.0, 2.0) for y in (0.0, 1.0) for x in (0.0, 1.0)],
                         dtype=torch.float64)
    elements = torch.tensor([[0, 1, 3, 2, 4, 5, 7, 6], [4, 5, 7, 6, 8, 9, 11, 10]])
    ref = SolidHeat(nodes, elements, IsotropicConductivity3D(1.0))
    ref.constraints[nodes[:, 2] == 0.0] = True
    ref.heat_flux[nodes[:, 2] == 2.0, 0] = 0.25
    T_ref = ref.solve(stol=STOL)[0]
    n_a, e_a = _block(0.0, 1.0)
    n_b, e_b = _block(1.0, 2.0)
    a = SolidHeat(n_a, e_a, IsotropicConductivity3D(1.0))
    b = SolidHeat(n_b, e_b, IsotropicConductivity3D(1.0))
    a.constraints[n_a[:, 2] == 0.0] = True
    b.heat_flux[n_b[:, 2] == 2.0, 0] = 0.25
    asm = Assembly([a, b])
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    Tt, _, _, _, _ = asm.solve(stol=STOL)
    assert rel(Tt[0], T_ref[:8]) < RTOL and rel(Tt[1], T_ref[4:]) < RTOL
    assert torch.equal(Tt[1][n_b[:, 2] == 1.0], Tt[0][n_a[:, 2] == 1.0])

    nodes, elements = mesh.cube_hexa(4, 4, 4)
    solid = SolidHeat(nodes, elements, IsotropicConductivity3D(1.0))
    solid.constraints[nodes[:, 2] == 0.0] = True
    top = nodes[:, 2] == 1.0
    point = ReferencePointHeat([0.5, 0.5, 1.5])
    point.heat_flux[0, 0] = 4.0
    asm = Assembly([solid, point])
    asm.coupling(solid, top, point)
    Tt, q, _, _, _ = asm.solve(stol=STOL)
    assert torch.allclose(Tt[0][top], torch.full_like(Tt[0][top], 4.0), rtol=1e-9)
    assert float(Tt[1][0, 0]) == pytest.approx(4.0, rel=1e-9)
    assert float(q[1][0, 0]) == pytest.approx(4.0, rel=1e-9)


def test_nearest_primary_pairing(cuda):
    n_a, e_a = _block(0.0, 1.0)
    n_b, e_b = _block(1.0, 2.0)
    a, b = Solid(n_a, e_a, SOLID), Solid(n_b, e_b, SOLID)
    a.constraints[:] = True
    a.displacements[:, 2] = 0.1 * n_a[:, 0] + 0.2 * n_a[:, 1]
    asm = Assembly([a, b])
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    u, _, _, _, _ = asm.solve(stol=STOL)
    interface, top = n_b[:, 2] == 1.0, n_a[:, 2] == 1.0
    assert float(u[1][interface][:, 2].std()) > 0.0
    assert torch.allclose(u[1][interface], u[0][top], atol=1e-14)


def test_minres_and_the_cg_agree(cuda):
    nodes, elements = mesh.cube_hexa(3, 3, 3)
    solid = Solid(nodes, elements, SOLID)
    solid.constraints[nodes[:, 2] == 0.0] = True
    point = ReferencePoint([0.5, 0.5, 2.0])
    point.forces[0, 3] = 50.0
    asm = Assembly([solid, point])
    asm.coupling(solid, nodes[:, 2] == nodes[:, 2].max(), point)
    u_cg = asm.solve(stol=STOL)[0]
    u_mr = asm.solve(stol=STOL, method="minres")[0]
    assert rel(u_mr[0], u_cg[0]) < 1e-7


def test_state_dependent_parts_are_refused(cuda):
    from torchfem_gb300.materials import IsotropicPlasticityPlaneStrain

    nodes, elements = mesh.rect_quad(3, 3)
    mat = IsotropicPlasticityPlaneStrain(E, NU, lambda q: 10.0 + 5.0 * q, lambda q: 5.0 + 0.0 * q)
    plate = Planar(nodes, elements, mat)
    with pytest.raises(NotImplementedError, match="constant tangent"):
        Assembly([plate]).solve()


def test_long_point_rows_vs_oracle(cuda):
    """Two tied jittered 12^3 cubes and a point driving the far 13 x 13-node
    face: each point row of T^T K T holds every DOF of the face's two node
    layers (about a thousand entries), past what the persistent CG gives one
    lane group, so those rows take the CTA-wide reduction.  Displacements and
    forces of all three parts match the oracle's direct solve."""
    import bench
    from oracle import assembly_oracle as A
    from oracle import fem_oracle as O

    n = 12
    asm, a, E0, point = bench.assembly_workload(n, cuda)
    u, f, _, _, _ = asm.solve(stol=STOL)
    rp = asm.last_solve.pattern.row_ptr.cpu().numpy()
    assert np.diff(rp).max() > 512
    nodes, el = (t.numpy() for t in bench.cube_nodes(n))
    nodes_b = nodes.copy()
    nodes_b[:, 0] += 1.0
    E_np = E0.cpu().numpy()
    pa = A.ModelPart(O.LinearModel(nodes, el, O.elastic_c("3d", E_np, 0.3, len(el))), 3)
    pb = A.ModelPart(O.LinearModel(nodes_b, el, O.elastic_c("3d", 1000.0, 0.3, len(el))), 3)
    pa.constraints[nodes[:, 0] == 0.0] = True
    pp = A.PointPart([2.5, 0.5, 0.5])
    pp.forces[0, 3] = 1.0
    pp.forces[0, 2] = 1.0
    oracle = A.AssemblyOracle([pa, pb, pp])
    oracle.coupling(1, nodes_b[:, 0] == 1.0, 0, nodes[:, 0] == 1.0)
    oracle.coupling(1, nodes_b[:, 0] == 2.0, 2)
    ou, of = oracle.solve()
    for k in range(3):
        assert rel(u[k], ou[k]) < RTOL, k
        assert rel(f[k], of[k]) < RTOL, k
