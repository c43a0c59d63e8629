"""Host-side logic that needs no GPU: API validation, element tables, mesh
numbering against the reference, method resolution, failure without CUDA."""

import numpy as np
import pytest
import torch

from oracle import fem_oracle as O
from torchfem_gb300 import Planar, Solid
from torchfem_gb300 import elements as E
from torchfem_gb300 import mesh
from torchfem_gb300.base import resolve_precision
from torchfem_gb300.materials import (
    IsotropicElasticity3D,
    IsotropicElasticityPlaneStrain,
    IsotropicElasticityPlaneStress,
)


def test_element_tables_match_oracle():
    for cls, name in ((E.Hexa1, "Hexa1"), (E.Quad1, "Quad1"), (E.Tetra2, "Tetra2"), (E.Tetra1, "Tetra1"),
                      (E.Tria1, "Tria1"), (E.Hexa2, "Hexa2")):
        n_e, dim, ip, w, dn = O.ELEMENTS[name]
        np.testing.assert_allclose(cls.gradient_table().numpy(), dn(ip), rtol=0, atol=1e-15)
        assert np.array_equal(cls.iweights().numpy().astype(np.float64), w)


def test_shape_functions_partition_of_unity():
    for cls in (E.Hexa1, E.Quad1, E.Quad2, E.Tria1, E.Tria2, E.Tetra1, E.Tetra2, E.Hexa2):
        xi = cls.ipoints()
        assert torch.allclose(cls.N(xi).sum(-1), torch.ones(len(xi), dtype=torch.float64))
        assert torch.allclose(cls.B(xi).sum(-1), torch.zeros(len(xi), cls.iso_dim, dtype=torch.float64), atol=1e-14)


def test_mesh_numbering_matches_reference(golden):
    # numpy and torch linspace may differ in the last bit: coordinates to 1 ulp,
    # connectivity exactly
    n, e = mesh.cube_hexa(11, 11, 11)
    on, oe = O.cube_hexa(11, 11, 11)
    assert np.allclose(n.numpy(), on, rtol=0, atol=1e-15) and np.array_equal(e.numpy(), oe)
    n, e = mesh.rect_quad(21, 11, 2.0, 1.0)
    on, oe = O.rect_quad(21, 11, 2.0, 1.0)
    assert np.allclose(n.numpy(), on, rtol=0, atol=1e-15) and np.array_equal(e.numpy(), oe)
    g = golden("patterns.npz")
    n, e = mesh.linear_to_quadratic(*mesh.cube_tetra(3, 3, 3))
    assert np.array_equal(e.numpy(), g["tet2_elements"])
    assert np.array_equal(n.numpy(), g["tet2_nodes"])


def test_box_tetra6_and_ogrid_positive_volumes():
    n, e = mesh.box_tetra6(4, 3, 3, 3.0, 1.0, 1.0)
    x = n[e]
    vol = torch.linalg.det(torch.stack([x[:, 1] - x[:, 0], x[:, 2] - x[:, 0], x[:, 3] - x[:, 0]], 1))
    assert (vol > 0).all() and torch.isclose(vol.sum() / 6.0, torch.tensor(3.0, dtype=torch.float64))
    n, e = mesh.plate_hole_ogrid(32, 8)
    assert n.shape == (32 * 9, 2) and e.shape == (32 * 8, 4)
    x = n[e]
    a = (x[:, 1, 0] - x[:, 0, 0]) * (x[:, 3, 1] - x[:, 0, 1]) - (x[:, 1, 1] - x[:, 0, 1]) * (x[:, 3, 0] - x[:, 0, 0])
    assert (a > 0).all()
    assert torch.isclose(n[:, 0].min(), torch.tensor(0.0, dtype=torch.float64))
    assert torch.isclose(n[:, 0].max(), torch.tensor(2.0, dtype=torch.float64))


def test_setters_validate_like_reference():
    n, e = mesh.cube_hexa(3, 3, 3)
    m = Solid(n, e, IsotropicElasticity3D(1000.0, 0.3))
    with pytest.raises(ValueError):
        m.forces = torch.zeros(3, 3)
    with pytest.raises(TypeError):
        m.forces = torch.zeros(len(n), 3, dtype=torch.int64)
    with pytest.raises(TypeError):
        m.constraints = torch.zeros(len(n), 3)
    with pytest.raises(ValueError):
        m.displacements = torch.zeros(2, 3)
    assert m.n_dofs == 81 and m.n_int == 8 and m.idx.dtype == torch.int32
    q = Planar(*mesh.rect_quad(3, 3), IsotropicElasticityPlaneStress(1.0, 0.3))
    assert q.thickness.shape == (4,) and q.n_int == 4


def test_method_resolution():
    assert resolve_precision(None, None) == "fp64"
    assert resolve_precision("cg", None) == "fp64"
    assert resolve_precision("gb300-mixed", None) == "mixed"
    assert resolve_precision(None, "mixed") == "mixed"
    with pytest.raises(ValueError):
        resolve_precision("foo", None)
    with pytest.raises(RuntimeError):
        resolve_precision("spsolve", None)
    assert resolve_precision("minres", None) == "fp64"
    with pytest.raises(ValueError):
        resolve_precision("minres", "mixed")


def test_material_kernel_data_and_step():
    n_elem = 5
    for mat, d in ((IsotropicElasticity3D(1000.0, 0.3), 3), (IsotropicElasticityPlaneStress(2.0, 0.25), 2),
                   (IsotropicElasticityPlaneStrain(3.0, 0.2), 2)):
        kind, data = mat.vectorize(n_elem).kernel_data(n_elem)
        assert kind == 1 and data.shape == (n_elem, 2)
        lam, G = data[0]
        I = torch.eye(d, dtype=torch.float64)
        rec = lam * torch.einsum("ij,kl->ijkl", I, I) + G * (
            torch.einsum("ik,jl->ijkl", I, I) + torch.einsum("il,jk->ijkl", I, I))
        assert torch.allclose(rec, mat.C.to(torch.float64), rtol=1e-14)
        H = torch.randn(4, d, d, dtype=torch.float64)
        s, _, C = mat.step(H, None, torch.zeros(4, d, d, dtype=torch.float64), None, torch.zeros(d, d), None, 0)
        assert torch.allclose(s, torch.einsum("ijkl,nkl->nij", mat.C.to(torch.float64), 0.5 * (H + H.transpose(1, 2))))


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU failure path")
def test_solve_without_cuda_fails_loudly():
    n, e = mesh.cube_hexa(3, 3, 3)
    m = Solid(n, e, IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[n[:, 0] == 0, :] = True
    with pytest.raises(RuntimeError, match="CUDA"):
        m.solve()


def test_shell_constructor_validates_like_reference():
    """Shell keeps the reference's section checks (shell.py:134-170)."""
    from torchfem_gb300 import Shell
    from torchfem_gb300.materials import IsotropicElasticityPlaneStress

    nodes = torch.tensor([[0.0, 0.0, 0.0], [1.0, 0.0, 0.0], [0.0, 1.0, 0.0]])
    el = torch.tensor([[0, 1, 2]])
    mat = IsotropicElasticityPlaneStress(1000.0, 0.3)
    with pytest.raises(ValueError, match="odd integer"):
        Shell(nodes, el, mat, n_simpson=4)
    s = Shell(nodes, el, mat, thickness=torch.tensor([0.2]))
    assert s.n_dof_per_node == 6 and s.n_int == 3 and "Tria1" in repr(s)
    assert torch.allclose(s.As[0], 0.2 * mat.G * torch.eye(2))
    data = s.kernel_data()
    assert data.shape == (1, 11)
    f = 1000.0 / (1 - 0.09)
    assert torch.allclose(data[0, :9], torch.tensor([f, 0.3 * f, 0, 0.3 * f, f, 0, 0, 0, f * 0.35]))
    assert torch.allclose(data[0, 9:], mat.G * torch.ones(2))


def test_preconditioner_resolution(monkeypatch):
    from torchfem_gb300.base import resolve_preconditioner

    monkeypatch.delenv("TORCHFEM_GB300_PRECOND", raising=False)
    assert resolve_preconditioner(None, "mixed", 3) == "amg"
    assert resolve_preconditioner(None, "mixed", 2) == "amg"
    assert resolve_preconditioner(None, "fp64", 3) == "jacobi"
    assert resolve_preconditioner(None, "mixed", 6) == "jacobi"  # shells
    assert resolve_preconditioner("jacobi", "mixed", 3) == "jacobi"
    with pytest.raises(ValueError):
        resolve_preconditioner("amg", "fp64", 3)
    with pytest.raises(ValueError):
        resolve_preconditioner("ilu", "mixed", 3)
    # one DOF per node (heat): multigrid in mixed precision, Jacobi in FP64
    assert resolve_preconditioner(None, "mixed", 1) == "amg"
    assert resolve_preconditioner(None, "fp64", 1) == "jacobi"
    with pytest.raises(NotImplementedError):
        resolve_preconditioner("jacobi", "mixed", 1)
    monkeypatch.setenv("TORCHFEM_GB300_PRECOND", "jacobi")
    assert resolve_preconditioner(None, "mixed", 3) == "jacobi"


def test_default_multigrid_falls_back_to_block_jacobi():
    """A hierarchy that cannot be built (here: a fake device mesh that refuses
    it) falls back to block Jacobi when the preconditioner was the default,
    and raises when it was asked for by name."""
    import torch

    from torchfem_gb300 import _lib
    from torchfem_gb300.sparse import SolveContext

    class FakeMesh:
        def __init__(self, d=3):
            self.calls = []
            self.d = d

        def build_system(self, mesh, mat, con_mask, precision, keep_refs=(), precond="jacobi", amg_reuse=False):
            self.calls.append(precond)
            if precond == "amg":
                raise _lib.FemError(_lib.FEM_BOUNDS, "fem_amg_create: a row exceeds its size limit")
            return f"system-{precision}-{precond}"

    con = torch.zeros(6, dtype=torch.uint8)
    sc = SolveContext(FakeMesh(), con, 1, "mixed", 10, 1e-8, 1e-6, 1e-10, None)
    sc.precond = "amg"
    with pytest.warns(RuntimeWarning, match="block Jacobi"):
        assert sc.build_system(None, None, ()) == "system-mixed-jacobi"
    assert sc.precond == "jacobi" and sc.dm.calls == ["amg", "jacobi"]

    # one DOF per node (heat conduction): the fallback is the FP64 Jacobi CG
    sc = SolveContext(FakeMesh(d=1), con, 16, "mixed", 10, 1e-8, 1e-6, 1e-10, None)
    sc.precond = "amg"
    with pytest.warns(RuntimeWarning, match="FP64 Jacobi CG"):
        assert sc.build_system(None, None, ()) == "system-fp64-jacobi"

    sc = SolveContext(FakeMesh(), con, 1, "mixed", 10, 1e-8, 1e-6, 1e-10, None)
    sc.precond, sc.precond_explicit = "amg", True
    with pytest.raises(_lib.FemError):
        sc.build_system(None, None, ())


def test_heat_models_and_setters_like_reference():
    """Heat boundary conditions validate like the reference
    (tests/test_base.py TestHeatBoundaryConditions)."""
    from torchfem_gb300 import PlanarHeat, SolidHeat
    from torchfem_gb300.materials import IsotropicConductivity2D, IsotropicConductivity3D

    model = PlanarHeat(*mesh.rect_quad(3, 3), IsotropicConductivity2D(kappa=400.0))
    assert model.n_dof_per_node == 1 and model.n_flux == [1, 2]
    assert model.constraints.shape == (9, 1)
    for prop in ("heat_flux", "temperatures"):
        value = torch.randn(model.n_nod, 1)
        setattr(model, prop, value)
        assert torch.equal(getattr(model, prop), value)
        with pytest.raises(ValueError, match="same shape as nodes"):
            setattr(model, prop, torch.zeros(model.n_nod, 2))
        with pytest.raises(TypeError, match="floating-point"):
            setattr(model, prop, torch.zeros(model.n_nod, 1, dtype=torch.int64))
    solid = SolidHeat(*mesh.cube_hexa(3, 3, 3), IsotropicConductivity3D(400.0))
    assert solid.n_flux == [1, 3] and solid.material.KAPPA.shape == (8, 3, 3)


def test_heat_time_integration_validates_t_output():
    from torchfem_gb300 import PlanarHeat
    from torchfem_gb300.materials import IsotropicConductivity2D

    model = PlanarHeat(*mesh.rect_quad(3, 3), IsotropicConductivity2D(kappa=400.0))
    with pytest.raises(ValueError, match="at least one time"):
        model.time_integration(torch.tensor([]))
    with pytest.raises(ValueError, match="negative"):
        model.time_integration(torch.tensor([-1.0, 1.0]))
    with pytest.raises(ValueError, match="strictly increasing"):
        model.time_integration(torch.tensor([0.0, 2.0, 2.0]))
    # prescribed temperatures are the one input the GPU adjoint does not differentiate
    model = PlanarHeat(*mesh.rect_quad(3, 3), IsotropicConductivity2D(kappa=400.0))
    temps = torch.zeros(model.n_nod, 1, requires_grad=True)
    model.temperatures = temps
    with pytest.raises(NotImplementedError, match="prescribed temperatures"):
        model.time_integration(differentiable_parameters=temps)


def test_conductivity_kernel_data():
    from torchfem_gb300 import _lib
    from torchfem_gb300.materials import OrthotropicConductivity2D, OrthotropicConductivity3D

    c, s = np.cos(0.3), np.sin(0.3)
    R = torch.tensor([[c, -s], [s, c]])
    mat = OrthotropicConductivity2D(3.0, 1.0).rotate(R).vectorize(4)
    kind, data = mat.kernel_data(4)
    assert kind == _lib.FEM_MAT_CONDUCTIVITY and data.shape == (4, 4)
    expect = R @ torch.diag(torch.tensor([3.0, 1.0])) @ R.T
    assert torch.allclose(data[2].view(2, 2), expect, rtol=1e-14, atol=0)
    k3 = OrthotropicConductivity3D(1.0, 2.0, 3.0)
    assert torch.equal(k3.KAPPA, torch.diag(torch.tensor([1.0, 2.0, 3.0])))
    flux, _, tangent = k3.step(torch.ones(1, 3), None, torch.zeros(1, 3), None, torch.zeros(1, 3), None, 0)
    assert torch.equal(flux, torch.tensor([[1.0, 2.0, 3.0]])) and tangent is k3.KAPPA


def test_heat_time_grid_matches_oracle():
    """The internal time grid of time_integration: starts at t = 0, steps of
    at most delta_t per knot interval, exact multiples take no extra step,
    knots are kept exactly; the same grid as the oracle's restatement."""
    from oracle import heat_oracle as H
    from torchfem_gb300.base import time_grid

    cases = [
        (torch.tensor([0.0, 6.0, 12.0, 18.0, 24.0]), 1.0),
        (torch.tensor([2.5, 5.0]), 0.5),
        (torch.tensor([0.0, 1.0]), 99.0),
        (torch.tensor([0.0, 0.3, 1.0]), 0.1),
        (torch.tensor([10.0]), 1.0),
        (torch.arange(0.0, 3.0 + 0.25, 0.25), 0.25),
    ]
    for t_out, dt in cases:
        times, rows = time_grid(t_out, dt)
        times_o, rows_o = H.time_grid(t_out.numpy(), dt)
        # torch.linspace (as in the reference) and numpy's may differ in the last bit
        assert np.allclose(times.numpy(), times_o, rtol=1e-15, atol=1e-15) and np.array_equal(rows.numpy(), rows_o)
        assert times[0] == 0.0 and torch.equal(times[rows], t_out.to(torch.float64))
        assert ((times[1:] - times[:-1]) <= dt * (1 + 1e-9)).all()
    times, rows = time_grid(torch.tensor([0.0, 0.3, 1.0]), 0.1)
    assert len(times) == 11 and rows.tolist() == [0, 3, 10]
    assert len(time_grid(torch.tensor([0.0, 1.0]), 99.0)[0]) == 2  # clamped to one step


def test_conductivity_kernel_data_carries_gradients():
    """kernel_data is differentiable: the adjoint's gradient for the per-element
    conductivity reaches kappa, and the SIMP pattern of the reference's thermal
    benchmark (KAPPA replaced by a scaled copy) reaches the densities."""
    from torchfem_gb300.materials import IsotropicConductivity2D, IsotropicConductivity3D

    kappa = torch.tensor([1.0, 2.0, 3.0], requires_grad=True)
    _, data = IsotropicConductivity2D(kappa).kernel_data(3)
    data.sum().backward()
    assert torch.equal(kappa.grad, torch.full((3,), 2.0))

    mat = IsotropicConductivity3D(1.0).vectorize(4)
    rho = torch.full((4,), 0.5, requires_grad=True)
    mat.KAPPA = (1e-3 + (1 - 1e-3) * rho**3)[:, None, None] * mat.KAPPA
    _, data = mat.kernel_data(4)
    data.view(4, 3, 3)[:, 0, 0].sum().backward()
    assert torch.allclose(rho.grad, 3 * (1 - 1e-3) * rho.detach() ** 2, rtol=1e-15, atol=0)
