"""GPU tests of the mixed solvers' FP64 residual from the FP64 copy of the
sliced matrix (fem_assemble_sell_pair + fem_sell_apply64).

The copy is the condensed stiffness matrix itself, so one FP64 sliced SpMV
over it must equal the FP64 element pass on the same system (fem_apply64:
K x with constrained entries zeroed, x at constrained DOFs) up to summation
order: 1e-13 relative, for 3x3 blocks (Hexa1), 2x2 blocks (Quad1) and scalar
rows (SolidHeat).  The FP32 values are the FP64 sums rounded once.  Mixed
solves with either residual reach the same FP64 solution to 1e-8 relative
(CG stopped at 1e-12), and the oracle's.
"""

import ctypes as C

import numpy as np
import pytest
import torch

from oracle import fem_oracle as O
from oracle import heat_oracle as H
from torchfem_gb300 import Planar, Solid, SolidHeat, _lib, mesh
from torchfem_gb300._device import LinearSystem
from torchfem_gb300.materials import (IsotropicConductivity3D, IsotropicElasticity3D,
                                      IsotropicElasticityPlaneStress)

pytestmark = pytest.mark.gpu

RTOL = 1e-8


def rel(a, b):
    a = a.detach().cpu().double().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().double().numpy() if torch.is_tensor(b) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def _jitter(nodes, n, seed):
    gen = torch.Generator().manual_seed(seed)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    return nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen, dtype=torch.float64) * 2 - 1) * 0.1 / n


def _elastic_cube():
    n = 10
    nodes, el = mesh.cube_hexa(n + 1, n + 1, n + 1)
    nodes = _jitter(nodes, n, 3)
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    m.constraints[nodes[:, 0] == 1.0, 0] = True  # partially constrained nodes
    m.forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    return m


def _planar():
    nodes, el = mesh.rect_quad(41, 21, 2.0, 1.0)
    m = Planar(nodes, el, IsotropicElasticityPlaneStress(200.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    m.forces[(nodes[:, 0] == 2.0) & (nodes[:, 1] == 0.0), 1] = -1.0
    return m


def _heat_cube():
    n = 12
    nodes, el = mesh.cube_hexa(n + 1, n + 1, n + 1)
    nodes = _jitter(nodes, n, 7)
    kappa = 1.0 + torch.rand(len(el), generator=torch.Generator().manual_seed(7), dtype=torch.float64)
    m = SolidHeat(nodes, el, IsotropicConductivity3D(kappa))
    m.constraints[nodes[:, 0] == 0.0] = True
    m.heat_flux[:] = 1.0 / len(nodes)
    return m


CASES = {"hexa1_3x3": _elastic_cube, "quad1_2x2": _planar, "heat_scalar": _heat_cube}


@pytest.fixture
def residual_copy():
    old = LinearSystem.RESIDUAL_COPY
    yield
    LinearSystem.RESIDUAL_COPY = old


def _solve(m, copy):
    LinearSystem.RESIDUAL_COPY = copy
    out = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")
    return out, m.last_solve.system


@pytest.mark.parametrize("case", sorted(CASES))
def test_fp64_copy_apply_equals_element_pass(cuda, residual_copy, case):
    m = CASES[case]()
    _, sysm = _solve(m, True)
    assert sysm.bval64 is not None
    # the FP32 values are the FP64 sums rounded once
    assert torch.equal(sysm.bval, sysm.bval64.float())
    dm = sysm.dm
    lib = dm.lib
    x = torch.rand(dm.n_dofs, generator=torch.Generator().manual_seed(11), dtype=torch.float64).to(cuda)
    y_copy = torch.empty_like(x)
    st = torch.cuda.current_stream().cuda_stream
    _lib.check(lib.fem_sell_apply64(C.byref(sysm.matrix), sysm.bval64.data_ptr(), x.data_ptr(), y_copy.data_ptr(), st),
               "fem_sell_apply64")
    ws = torch.empty(max(int(lib.fem_apply64_workspace_bytes(C.byref(sysm.op))), 1), dtype=torch.uint8, device=cuda)
    y_el = torch.empty_like(x)
    _lib.check(lib.fem_apply64(C.byref(sysm.op), x.data_ptr(), y_el.data_ptr(), ws.data_ptr(), ws.numel(), st),
               "fem_apply64")
    torch.cuda.synchronize()
    assert rel(y_copy, y_el) <= 1e-13
    # constrained DOFs: identity rows
    con = m.constraints.reshape(-1).to(cuda)
    assert torch.equal(y_copy[con], x[con])


@pytest.mark.parametrize("case", sorted(CASES))
def test_mixed_solve_same_with_either_residual(cuda, residual_copy, case):
    m = CASES[case]()
    (u1, f1, *_), s1 = _solve(m, True)
    assert s1.bval64 is not None
    u1, f1 = u1.clone(), f1.clone()
    (u2, f2, *_), s2 = _solve(m, False)
    assert s2.bval64 is None
    assert rel(u1, u2) <= RTOL and rel(f1, f2) <= RTOL


def test_fp64_copy_solution_against_oracle(cuda, residual_copy):
    m = _elastic_cube()
    (u, f, s, _, _), _ = _solve(m, True)
    nodes = m.nodes.cpu().numpy()
    om = O.LinearModel(nodes, m.elements.cpu().numpy(), O.elastic_c("3d", 1000.0, 0.3, len(m.elements)))
    uo, fo, so = om.solve(m.forces.cpu().numpy(), m.constraints.cpu().numpy())
    assert rel(u, uo) <= RTOL and rel(f, fo) <= RTOL and rel(s, so) <= RTOL

    h = _heat_cube()
    (T, fh, *_), _ = _solve(h, True)
    hn = h.nodes.cpu().numpy()
    con = h.constraints.cpu().numpy().reshape(-1)
    k = 1.0 + torch.rand(len(h.elements), generator=torch.Generator().manual_seed(7), dtype=torch.float64)
    oh = H.HeatModel(hn, h.elements.cpu().numpy(), k.numpy()[:, None, None] * np.eye(3))
    To, fo, _, _ = oh.solve(np.full(len(hn), 1.0 / len(hn)), con)
    assert rel(T.reshape(-1), To) <= RTOL and rel(fh.reshape(-1), fo) <= RTOL


def test_default_residual_choice(cuda, residual_copy):
    """By default the FP64 copy serves heat conduction (element matrices
    integrated in FP64 anyway) and isotropic elasticity (the moment form);
    per-point tangents keep the element pass."""
    LinearSystem.RESIDUAL_COPY = None
    h = _heat_cube()
    h.solve(stol=1e-12, precision="mixed")
    assert h.last_solve.system.bval64 is not None
    m = _planar()
    m.solve(stol=1e-12, precision="mixed", preconditioner="amg")
    assert m.last_solve.system.bval64 is not None
    dm = m.device_mesh
    tangent = _lib.FemMaterial(_lib.FEM_MAT_TANGENT_IP, 0)
    assert not LinearSystem.residual_copy(dm, tangent)


def _iso_models():
    nodes, el = mesh.cube_tetra(4, 3, 3)
    nodes2, el2 = mesh.linear_to_quadratic(nodes, el)
    tet2 = Solid(nodes2, el2, IsotropicElasticity3D(210.0, 0.25))
    return {"hexa1": _elastic_cube(), "quad1": _planar(), "tetra2": tet2}


def test_iso64_element_matrices_equal_fp64_stiffness(cuda):
    """fem_element_stiffness_iso64 (moment form, a thread per node pair)
    equals fem_element_stiffness in FP64 up to summation order, with a
    per-element thickness on the planar mesh."""
    for name, m in _iso_models().items():
        if name == "quad1":
            m.thickness = 0.5 + torch.rand(len(m.elements), generator=torch.Generator().manual_seed(5),
                                           dtype=torch.float64)
        dm = m.device_mesh
        mesh_, mat, _refs = m._device_material()
        k64 = dm.element_stiffness(mesh_, mat, torch.float64)
        kiso = dm.element_stiffness_iso64(mesh_, mat)
        torch.cuda.synchronize()
        assert rel(kiso, k64) <= 1e-13, name
        assert torch.equal(kiso, kiso.transpose(1, 2)), name
