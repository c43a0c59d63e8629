"""GPU parity of the Tria1 flat-facet shell (fem_shell_* kernels) against the
reference's own outputs (tests/golden/shell_roof_9x7.npz, written by
tests/golden/make_golden.py from torch-fem's Shell) and the reference's
Timoshenko-strip check.

Tolerances: element matrices 1e-13 relative (different summation order than
the reference's einsums); assembly given the reference's element matrices bit
for bit; u, f and stresses 1e-8 with the CG run to 1e-12; gradients 1e-7.
"""

import numpy as np
import pytest
import torch

from torchfem_gb300 import Shell, mesh
from torchfem_gb300.materials import IsotropicElasticityPlaneStress

pytestmark = pytest.mark.gpu


def rel(a, b):
    a = a.detach().cpu().double().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().double().numpy() if torch.is_tensor(b) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def roof(g):
    nodes = torch.tensor(g["nodes"])
    el = torch.tensor(g["elements"])
    E = torch.tensor(g["E"], requires_grad=True)
    t = torch.tensor(g["t"], requires_grad=True)
    m = Shell(nodes, el, IsotropicElasticityPlaneStress(E, 0.3), thickness=t)
    y0, y1 = nodes[:, 1] == 0.0, nodes[:, 1] == 2.0
    side = (nodes[:, 0] - nodes[:, 0].min()).abs() < 1e-12
    m.constraints[y0, :] = True
    m.constraints[y1, 0] = True
    m.constraints[y1, 2] = True
    m.constraints[y1, 1] = True
    m.displacements[y1, 1] = 1e-3
    m.forces[:, 2] = -1.0 / len(nodes)
    m.forces[side, 3] = 2e-3
    return m, E, t


def test_shell_element_matrices_and_assembly(cuda, golden):
    import ctypes as C

    from torchfem_gb300 import _lib
    from torchfem_gb300.shell import ShellContext

    g = golden("shell_roof_9x7.npz")
    m, E, t = roof(g)
    dm = m.device_mesh
    assert np.array_equal(m.glob_idx.cpu().numpy(), g["glob_idx"])
    assert np.array_equal(m.k_map.cpu().numpy().astype(np.int64), g["k_map"])
    sc = ShellContext(m, dm, m.constraints.reshape(-1).to(cuda), 10, 1e-8, 1e-6, 1e-12, None)
    mat = m.kernel_data().detach().to(cuda).contiguous()
    thick = m.thickness.detach().to(cuda).contiguous()
    sc.prepare(mat, thick)
    assert rel(sc.ke.view(-1, 18, 18), g["ke"]) <= 1e-13
    # bit-exact assembly given the reference's element matrices
    ke_ref = torch.tensor(g["ke"], device=cuda).contiguous()
    val = dm.assemble_csr(ke_ref, sc.con_mask)
    gi = g["glob_idx"]
    assert np.array_equal(val.cpu().numpy(), g["K"][gi[0], gi[1]])
    del C, _lib


def test_shell_roof_vs_reference(cuda, golden):
    """u, f, station stresses and d(loss)/d(E, t) of the cylindrical roof
    against the reference's spsolve + autograd."""
    g = golden("shell_roof_9x7.npz")
    m, E, t = roof(g)
    u, f, s, F, st = m.solve(rtol=1e-12, atol=1e-14, stol=1e-12, differentiable_parameters=(E, t))
    assert rel(u, g["u"]) <= 1e-8
    assert rel(f, g["f"]) <= 1e-8
    assert rel(s, g["sigma"]) <= 1e-8
    assert rel(F, g["F"]) == 0.0
    assert st.shape == (len(g["elements"]), 0)
    free = ~m.constraints
    L = (u * free).pow(2).sum() + (f[:, 2] * u[:, 2]).sum()
    assert abs(float(L.detach()) - float(g["loss"])) <= 1e-8 * abs(float(g["loss"]))
    gE, gt = torch.autograd.grad(L, (E, t))
    assert rel(gE, g["grad_E"]) <= 1e-7
    assert rel(gt, g["grad_t"]) <= 1e-7
    _, _, s_ip, _, _ = m.solve(rtol=1e-12, atol=1e-14, stol=1e-12, aggregate_integration_points=False)
    assert s_ip.shape == (3, len(g["elements"]), 2, 2)
    assert rel(s_ip, g["sigma_ip"]) <= 1e-8


@pytest.mark.parametrize("t", [2.0, 0.5])
def test_shell_strip_matches_timoshenko(cuda, t):
    """A narrow strip with nu = 0 is a Timoshenko beam: tip deflection =
    bending + shear within 1 % (the reference's tests/test_models.py:130-151)."""
    E, L, b, P, kappa = 1000.0, 10.0, 1.0, 1.0, 5.0 / 6.0
    nodes, elements = mesh.strip_tria(41, 3, L, b)
    beam = Shell(nodes, elements, IsotropicElasticityPlaneStress(E=E, nu=0.0), thickness=t)
    tip = nodes[:, 0] > L - 1e-9
    beam.forces[tip, 2] = P / int(tip.sum())
    beam.constraints[nodes[:, 0] < 1e-9, :] = True
    u, _, _, _, _ = beam.solve(stol=1e-12)
    bending = P * L**3 / (3 * E * b * t**3 / 12)
    shear = P * L / (kappa * (E / 2) * b * t)
    assert float(u[:, 2].abs().max()) == pytest.approx(bending + shear, rel=0.01)


def test_shell_rejects_mixed_and_nlgeom(cuda):
    nodes, elements = mesh.strip_tria(3, 2, 1.0, 1.0)
    m = Shell(nodes, elements, IsotropicElasticityPlaneStress(1000.0, 0.3), thickness=0.1)
    with pytest.raises(NotImplementedError):
        m.solve(precision="mixed")
    with pytest.raises(NotImplementedError):
        m.solve(nlgeom=True)
