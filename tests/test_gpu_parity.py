"""GPU parity of the C-ABI kernels against the reference's golden vectors and
the CPU oracle.

Tolerances: integer pattern data and assembly given the reference's element
matrices are compared bit for bit; element matrices to 1e-13 relative (the
GPU sums Gauss points in a different floating-point order than the
reference's batched einsum); solutions and gradients to 1e-8 relative, the
accuracy target of the forward + adjoint path, with the CG run to 1e-12.
"""

import numpy as np
import pytest
import torch

from oracle import fem_oracle as O
from torchfem_gb300 import Planar, Solid, mesh
from torchfem_gb300.materials import IsotropicElasticity3D, IsotropicElasticityPlaneStress

pytestmark = pytest.mark.gpu

RTOL = 1e-8


def rel(a, b):
    a = a.detach().cpu().double().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().double().numpy() if torch.is_tensor(b) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def cube_model(g, E=None):
    nodes = torch.tensor(g["nodes"])
    el = torch.tensor(g["elements"])
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0 if E is None else E, 0.3))
    m.constraints = torch.tensor(g["constraints"])
    m.forces = torch.tensor(g["forces"])
    return m


def test_pattern_parity_hexa(cuda, golden):
    g = golden("hexa_jitter3.npz")
    m = cube_model(g)
    assert np.array_equal(m.glob_idx.cpu().numpy(), g["glob_idx"])
    assert np.array_equal(m.k_map.cpu().numpy(), g["k_map"])
    assert np.array_equal(m.diag_map.cpu().numpy(), g["diag_map"])


@pytest.mark.parametrize("which", ["tet2", "orphan"])
def test_pattern_parity_tet2_orphan(cuda, golden, which):
    g = golden("patterns.npz")
    nodes = torch.tensor(g[f"{which}_nodes"])
    el = torch.tensor(g[f"{which}_elements"])
    if nodes.shape[1] == 3:
        m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    else:
        m = Planar(nodes, el, IsotropicElasticityPlaneStress(1000.0, 0.3))
    assert np.array_equal(m.glob_idx.cpu().numpy(), g[f"{which}_glob_idx"])
    assert np.array_equal(m.k_map.cpu().numpy(), g[f"{which}_k_map"])
    assert np.array_equal(m.diag_map.cpu().numpy(), g[f"{which}_diag_map"])


def test_assembly_bit_exact_given_reference_ke(cuda, golden):
    g = golden("hexa_jitter3.npz")
    m = cube_model(g)
    dm = m.device_mesh
    ke = torch.tensor(g["ke"], device=cuda).contiguous()
    con = m.constraints.reshape(-1).to(cuda, torch.uint8).contiguous()
    val = dm.assemble_csr(ke, con).cpu().numpy()
    assert np.array_equal(val, g["kval"])  # bit for bit


def test_element_stiffness_vs_reference(cuda, golden):
    g = golden("hexa_jitter3.npz")
    m = cube_model(g)
    dm = m.device_mesh
    kind, data = m.material.kernel_data(m.n_elem)
    data = data.to(cuda).contiguous()
    from torchfem_gb300 import _lib

    ke = dm.element_stiffness(dm.make_mesh(None), _lib.FemMaterial(kind, data.data_ptr()))
    assert rel(ke, torch.tensor(g["ke"])) <= 1e-13


@pytest.mark.parametrize("precision,precond", [("fp64", None), ("mixed", "jacobi"), ("mixed", "amg")])
def test_hexa2_vs_reference(cuda, golden, precision, precond):
    """Hexa2 (20-node serendipity): pattern, element matrices and the solution
    of the reference's jittered quadratic cube."""
    g = golden("hexa2_jitter2.npz")
    nodes, el = torch.tensor(g["nodes"]), torch.tensor(g["elements"])
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    assert m.etype.__name__ == "Hexa2"
    assert np.array_equal(m.glob_idx.cpu().numpy(), g["glob_idx"])
    assert np.array_equal(m.k_map.cpu().numpy(), g["k_map"])
    from torchfem_gb300 import _lib

    kind, data = m.material.kernel_data(m.n_elem)
    dm = m.device_mesh
    ke = dm.element_stiffness(dm.make_mesh(None), _lib.FemMaterial(kind, data.to(cuda).contiguous().data_ptr()))
    assert rel(ke, torch.tensor(g["ke"])) <= 1e-13
    m.constraints[nodes[:, 0] == 0.0, :] = True
    m.forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    u, f, s, _, _ = m.solve(stol=1e-12, precision=precision, preconditioner=precond)
    assert rel(u, g["u"]) <= RTOL
    assert rel(f, g["f"]) <= RTOL
    assert rel(s, g["sigma"]) <= RTOL


def test_c1_forward_and_adjoint(cuda, golden):
    g = golden("c1_cube10.npz")
    nodes, el = mesh.cube_hexa(11, 11, 11)
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    forces = torch.zeros_like(nodes)
    forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    forces.requires_grad_(True)
    m.forces = forces
    u, f, s, _, _ = m.solve(stol=1e-12, differentiable_parameters=forces)
    assert rel(u, g["u"]) <= RTOL
    assert rel(f, g["f"]) <= RTOL
    assert rel(s, g["sigma"]) <= RTOL
    (gf,) = torch.autograd.grad(u.sum(), forces)
    assert rel(gf, g["grad_forces"]) <= RTOL


@pytest.mark.parametrize("precision,precond", [("fp64", None), ("mixed", "jacobi"), ("mixed", "amg")])
def test_jittered_cube_gradients(cuda, golden, precision, precond):
    g = golden("hexa_jitter3.npz")
    E = torch.tensor(g["E"], requires_grad=True)
    m = cube_model(g, E)
    forces = m.forces.clone().requires_grad_(True)
    m.forces = forces
    u, f, s, gr, _ = m.solve(stol=1e-12, precision=precision, preconditioner=precond,
                             differentiable_parameters=(forces, E))
    assert rel(u, g["u"]) <= RTOL
    assert rel(f, g["f"]) <= RTOL
    assert rel(s, g["sigma"]) <= RTOL
    assert rel(gr, g["grad"]) <= RTOL
    (gf,) = torch.autograd.grad(u.sum(), forces, retain_graph=True)
    assert rel(gf, g["grad_forces"]) <= RTOL
    L = torch.inner(f.ravel(), u.ravel())
    assert abs(float(L.detach()) - float(g["compliance"])) <= RTOL * abs(float(g["compliance"]))
    (gE,) = torch.autograd.grad(L, E)
    assert rel(gE, g["grad_E"]) <= RTOL


def test_minres_jittered_cube_vs_reference(cuda, golden):
    """method="minres" (Jacobi MINRES, the reference GPU branch's other
    Krylov method): forward and adjoint against the reference."""
    g = golden("hexa_jitter3.npz")
    E = torch.tensor(g["E"], requires_grad=True)
    m = cube_model(g, E)
    forces = m.forces.clone().requires_grad_(True)
    m.forces = forces
    u, f, s, _, _ = m.solve(stol=1e-12, method="minres", differentiable_parameters=(forces, E))
    assert m.last_solve.linear == "minres"
    assert rel(u, g["u"]) <= RTOL
    assert rel(f, g["f"]) <= RTOL
    assert rel(s, g["sigma"]) <= RTOL
    (gf,) = torch.autograd.grad(u.sum(), forces, retain_graph=True)
    assert rel(gf, g["grad_forces"]) <= RTOL
    L = torch.inner(f.ravel(), u.ravel())
    (gE,) = torch.autograd.grad(L, E)
    assert rel(gE, g["grad_E"]) <= RTOL


def simp(Nx, Ny, rho):
    nodes, el = mesh.rect_quad(Nx + 1, Ny + 1, 2.0, 1.0)
    m = Planar(nodes, el, IsotropicElasticityPlaneStress(rho**3 * 1.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    tip = torch.argmin(((nodes - torch.tensor([2.0, 0.5])) ** 2).sum(1))
    m.forces[tip, 1] = -1.0
    return m


def compliance(m, rho, **kw):
    u, f, _, _, _ = m.solve(differentiable_parameters=rho, **kw)
    return torch.inner(f.ravel(), u.ravel())


def test_simp_small_vs_reference(cuda, golden):
    g = golden("simp_20x10.npz")
    rho = torch.tensor(g["rho"], requires_grad=True)
    m = simp(20, 10, rho)
    L = compliance(m, rho, stol=1e-12)
    assert abs(float(L.detach()) - float(g["compliance"])) <= RTOL * abs(float(g["compliance"]))
    (gr,) = torch.autograd.grad(L, rho)
    assert rel(gr, g["grad_rho"]) <= RTOL


def test_simp_central_differences(cuda, golden):
    g = golden("simp_20x10.npz")
    rho0 = torch.tensor(g["rho"])
    rho = rho0.clone().requires_grad_(True)
    L = compliance(simp(20, 10, rho), rho, stol=1e-13)
    (gr,) = torch.autograd.grad(L, rho)
    idx = torch.randperm(len(rho0), generator=torch.Generator().manual_seed(3))[:5]
    h = 1e-6
    for i in idx.tolist():
        rp, rm = rho0.clone(), rho0.clone()
        rp[i] += h
        rm[i] -= h
        with torch.no_grad():
            Lp = float(compliance(simp(20, 10, rp), rp, stol=1e-13))
            Lm = float(compliance(simp(20, 10, rm), rm, stol=1e-13))
        fd = (Lp - Lm) / (2 * h)
        # each compliance carries the solve's relative error (stol) times |L|;
        # the difference quotient divides it by 2h
        noise = 2 * 1e-13 * abs(Lp) / (2 * h)
        assert abs(fd - float(gr[i])) <= 1e-5 * abs(float(gr[i])) + noise


PATCH_2D = torch.tensor([[1.0e-3, 2.0e-4], [3.0e-4, -1.0e-3]])
PATCH_3D = torch.tensor([[1.0e-3, 2.0e-4, -1.0e-4], [3.0e-4, -1.0e-3, 5.0e-5], [1.0e-4, 2.0e-4, 7.0e-4]])


@pytest.mark.parametrize("etype", ["Quad1", "Hexa1", "Tetra1", "Tetra2", "Tria1", "Tria2", "Quad2", "Hexa2"])
def test_patch(cuda, etype):
    """A linear displacement field prescribed on the boundary is reproduced
    inside, with uniform stress (reference tests/test_models.py:54-71)."""
    if etype in ("Quad1", "Quad2"):
        nodes, el = mesh.rect_quad(4, 4)
    elif etype in ("Tria1", "Tria2"):
        nodes, q = mesh.rect_quad(4, 4)
        el = torch.cat([q[:, [0, 1, 2]], q[:, [0, 2, 3]]])
    elif etype in ("Hexa1", "Hexa2"):
        nodes, el = mesh.cube_hexa(3, 3, 3)
    else:
        nodes, el = mesh.cube_tetra(3, 3, 3)
    if etype in ("Quad2", "Tria2", "Tetra2", "Hexa2"):
        nodes, el = mesh.linear_to_quadratic(nodes, el)
    dim = nodes.shape[1]
    if dim == 2:
        m = Planar(nodes, el, IsotropicElasticityPlaneStress(1000.0, 0.3))
        G = PATCH_2D
    else:
        m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
        G = PATCH_3D
    assert m.etype.__name__ == etype
    u_exact = nodes @ G.T
    bnd = torch.zeros(len(nodes), dtype=torch.bool)
    for k in range(dim):
        c = nodes[:, k]
        bnd |= torch.isclose(c, c.min()) | torch.isclose(c, c.max())
    m.constraints = bnd[:, None].repeat(1, dim)
    m.displacements = u_exact
    u, _, sigma, _, _ = m.solve(stol=1e-14)
    assert torch.allclose(u, u_exact, atol=1e-12)
    assert torch.allclose(sigma, sigma[0].expand_as(sigma), atol=1e-10)


def test_plain_and_mixed_agree_on_jittered_cube(cuda):
    nodes, el = mesh.cube_hexa(13, 13, 13)
    gen = torch.Generator().manual_seed(0)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    nodes = nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen) * 2 - 1) * 0.1 / 12
    res = {}
    for p in ("fp64", "mixed"):
        m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
        m.constraints[nodes[:, 0] == 0.0, :] = True
        m.forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
        res[p] = m.solve(precision=p, stol=1e-10)
        if p == "mixed":
            assert m.last_solve.iterations[0] > 0
    assert rel(res["mixed"][0], res["fp64"][0]) <= RTOL
    assert rel(res["mixed"][2], res["fp64"][2]) <= RTOL
    # oracle at the same size
    om = O.LinearModel(nodes.numpy(), el.numpy(), O.elastic_c("3d", 1000.0, 0.3, len(el)))
    con = np.zeros(nodes.shape, dtype=bool)
    con[nodes[:, 0].numpy() == 0.0, :] = True
    F = np.zeros(nodes.shape)
    F[nodes[:, 0].numpy() == 1.0, 2] = -1.0 / len(nodes)
    u, f, s = om.solve(F, con)
    assert rel(res["fp64"][0], u) <= RTOL
    assert rel(res["mixed"][0], u) <= RTOL


def test_assembly_and_solve_deterministic(cuda, golden):
    g = golden("hexa_jitter3.npz")
    outs = []
    for _ in range(3):
        m = cube_model(g)
        outs.append(m.solve()[0].cpu().numpy())
    assert all(np.array_equal(outs[0], o) for o in outs[1:])


def test_negative_jacobian_raises(cuda):
    nodes, el = mesh.cube_hexa(3, 3, 3)
    el = el[:, [1, 0, 3, 2, 5, 4, 7, 6]]  # mirrored numbering: detJ < 0
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    with pytest.raises(ValueError, match="Jacobian"):
        m.solve()


def test_barrier_wait_runs_out_cleanly(cuda):
    """A grid-barrier wait that can never complete gives up after its cycle
    limit and reports the timeout; the context stays usable afterwards."""
    from torchfem_gb300 import _lib

    lib = _lib.load()
    ws = torch.zeros(lib.fem_diag_workspace_bytes(), dtype=torch.uint8, device=cuda)
    rc = lib.fem_diag_barrier_timeout(ws.data_ptr(), ws.numel(), 2_000_000, _lib.stream_handle(cuda))
    assert rc == _lib.FEM_CUDA_ERROR
    assert b"barrier timeout" in lib.fem_last_error()
    torch.cuda.synchronize()
    nodes, el = mesh.cube_hexa(3, 3, 3)
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    m.forces[nodes[:, 0] == 1.0, 2] = -1.0
    u = m.solve(stol=1e-12)[0]
    assert torch.isfinite(u).all() and float(u.abs().max()) > 0.0


def test_cg_iteration_cap_cuts_back_then_raises(cuda):
    nodes, el = mesh.cube_hexa(5, 5, 5)
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    m.forces[nodes[:, 0] == 1.0, 2] = -1.0
    with pytest.raises(RuntimeError, match="did not converge"):
        m.solve(cg_max_iter=2, max_cutbacks=2)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_persistent_and_kernel_cg_paths_agree(cuda, precision):
    """The persistent cooperative CG (with and without the TMA-staged SpMV)
    and the three-kernels-per-iteration CG: same solution to 1e-10, iteration
    counts within a few percent."""
    from torchfem_gb300 import _lib

    lib = _lib.load()
    nodes, el = mesh.cube_hexa(11, 11, 11)
    gen = torch.Generator().manual_seed(0)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    nodes = nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen) * 2 - 1) * 0.01
    out, iters = {}, {}
    try:
        for path in (1, 2, 0):
            lib.fem_set_cg_path(path)
            m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
            m.constraints[nodes[:, 0] == 0.0, :] = True
            m.forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
            out[path] = m.solve(precision=precision, stol=1e-12, preconditioner="jacobi")[0]
            iters[path] = m.last_solve.iterations
    finally:
        lib.fem_set_cg_path(1)
    for path in (1, 2):
        assert rel(out[path], out[0]) <= 1e-10
        for a, b in zip(iters[path], iters[0]):
            # path 1 carries q = A p by recurrence inside a launch (FP32
            # rounding differs from the explicit product: a few % more steps)
            assert abs(a - b) <= max(2, (0.1 if path == 1 else 0.02) * b), (path, iters)


# ----------------------------------------------------------------- nonlinear --
def _hyper_model(g):
    from torchfem_gb300.materials import Hyperelastic3D, neo_hookean_psi

    nodes = torch.tensor(g["nodes"])
    el = torch.tensor(g["elements"])
    E = torch.tensor(g["E"], requires_grad=True)
    nu = 0.45
    mu = E / (2.0 * (1.0 + nu))
    lbd = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))

    def psi(F, params):  # the user's energy, as in the reference benchmark
        MU, LBD = params[0], params[1]
        C = F.transpose(-1, -2) @ F
        logJ = 0.5 * torch.logdet(C)
        return MU / 2 * (torch.trace(C) - 3.0) - MU * logJ + LBD / 2 * logJ**2

    m = Solid(nodes, el, Hyperelastic3D(psi, torch.stack([mu, lbd], dim=-1)))
    right = nodes[:, 0] == 3.0
    m.constraints[nodes[:, 0] == 0.0, :] = True
    m.constraints[right, 0] = True
    m.displacements[right, 0] = 0.5
    return m, E, right


@pytest.mark.parametrize("precision,precond", [("fp64", None), ("mixed", "jacobi"), ("mixed", "amg")])
def test_neo_hookean_tetra2_vs_reference(cuda, golden, precision, precond):
    """Config 4 at small size: Tetra2, Neo-Hookean, nlgeom, 10 increments;
    tip reaction and its gradient w.r.t. per-element E against the reference."""
    g = golden("hyper_tet2_6x2x2.npz")
    m, E, right = _hyper_model(g)
    # Newton to 1e-10 relative: 1e-12 is at this problem's FP64 residual floor
    u, f, s, F, _ = m.solve(increments=torch.linspace(0.0, 1.0, 11), nlgeom=True, rtol=1e-10, atol=1e-10,
                            max_iter=20, stol=1e-13, precision=precision, preconditioner=precond,
                            differentiable_parameters=E)
    assert rel(u, g["u"]) <= 1e-8
    assert rel(f, g["f"]) <= 1e-8
    assert rel(s, g["sigma"]) <= 1e-8
    assert rel(F, g["F"]) <= 1e-8
    R = f[right, 0].sum()
    assert abs(float(R.detach()) - float(g["reaction"])) <= 1e-8 * abs(float(g["reaction"]))
    (gE,) = torch.autograd.grad(R, E)
    assert rel(gE, g["grad_E"]) <= 1e-7


def test_neo_hookean_with_minres(cuda, golden):
    """MINRES also carries the Newton solves of the indefinite Neo-Hookean
    tangents (config 4 at small size)."""
    g = golden("hyper_tet2_6x2x2.npz")
    m, E, right = _hyper_model(g)
    u, f, s, F, _ = m.solve(increments=torch.linspace(0.0, 1.0, 11), nlgeom=True, rtol=1e-10, atol=1e-10,
                            max_iter=20, stol=1e-13, method="minres", differentiable_parameters=E)
    assert rel(u, g["u"]) <= 1e-8
    R = f[right, 0].sum()
    (gE,) = torch.autograd.grad(R, E)
    assert rel(gE, g["grad_E"]) <= 1e-7


def _plastic_model(g):
    from torchfem_gb300.materials import IsotropicPlasticityPlaneStrain

    nodes = torch.tensor(g["nodes"])
    el = torch.tensor(g["elements"])
    mat = IsotropicPlasticityPlaneStrain(1000.0, 0.3, lambda q: 1.0 + 100.0 * q,
                                         lambda q: 100.0 * torch.ones_like(q))
    t = torch.ones(len(el), dtype=torch.float64, requires_grad=True)
    m = Planar(nodes, el, mat, thickness=t)
    left = torch.isclose(nodes[:, 0], torch.tensor(0.0, dtype=torch.float64))
    right = torch.isclose(nodes[:, 0], torch.tensor(2.0, dtype=torch.float64))
    m.constraints[left, 0] = True
    pin = torch.argmin(((nodes - torch.tensor([0.0, 0.5])) ** 2).sum(1))
    m.constraints[pin, 1] = True
    m.constraints[right, 0] = True
    m.displacements[right, 0] = 0.02
    return m, t, right


@pytest.mark.parametrize("precision,precond", [("fp64", None), ("mixed", "jacobi"), ("mixed", "amg")])
def test_plane_strain_plasticity_vs_reference(cuda, golden, precision, precond):
    """Config 5 at small size: O-grid plate with hole, J2 plane strain,
    20 increments; reaction and its gradient w.r.t. element thickness through
    the per-increment checkpointed adjoint, against the reference."""
    g = golden("plastic_ogrid_32x8.npz")
    m, t, right = _plastic_model(g)
    u, f, s, _, st = m.solve(increments=torch.linspace(0.0, 1.0, 21), rtol=1e-12, atol=1e-12, max_iter=80,
                             stol=1e-13, precision=precision, preconditioner=precond, differentiable_parameters=t)
    assert float(st[:, 0].max()) > 0.0  # the plate yields
    assert rel(u, g["u"]) <= 1e-8
    assert rel(f, g["f"]) <= 1e-8
    assert rel(s, g["sigma"]) <= 1e-8
    assert rel(st, g["state"]) <= 1e-8
    R = f[right, 0].sum()
    assert abs(float(R.detach()) - float(g["reaction"])) <= 1e-8 * abs(float(g["reaction"]))
    (gt,) = torch.autograd.grad(R, t)
    assert rel(gt, g["grad_t"]) <= 1e-7


def _simp_rho(n_elem):
    return 0.2 + 0.8 * torch.rand(n_elem, generator=torch.Generator().manual_seed(0), dtype=torch.float64)


@pytest.mark.parametrize("precision", ["fp64"])
def test_simp_full_size_vs_reference(cuda, golden, precision):
    """Config 3 at full size (Quad1 400 x 200, 161,202 DOF): compliance and
    dL/drho on 20 seeded elements against the reference's autograd.  FP64
    only: with the 125x stiffness contrast of SIMP, conditioning times FP32
    epsilon exceeds one and FP32 storage cannot be refined to 1e-12."""
    g = golden("simp_400x200.npz")
    rho = _simp_rho(80000).requires_grad_(True)
    m = simp(400, 200, rho)
    L = compliance(m, rho, stol=1e-12, precision=precision)
    assert abs(float(L.detach()) - float(g["compliance"])) <= RTOL * abs(float(g["compliance"]))
    (gr,) = torch.autograd.grad(L, rho)
    idx = torch.tensor(g["sample_idx"])
    assert rel(gr[idx], g["grad_rho_sample"]) <= RTOL
    assert abs(float(gr.norm()) - float(g["grad_norm"])) <= RTOL * float(g["grad_norm"])


def test_simp_full_size_central_differences(cuda, golden):
    """dL/drho at config 3's size against central differences on the same 20
    seeded elements.  h = 1e-4 here: with an iterative solve at 161k DOF the
    compliance carries ~1e-13 relative stopping noise, which h = 1e-6 would
    amplify past the gradient (h = 1e-6 is checked at 20 x 10 above)."""
    g = golden("simp_400x200.npz")
    rho0 = _simp_rho(80000)
    rho = rho0.clone().requires_grad_(True)
    (gr,) = torch.autograd.grad(compliance(simp(400, 200, rho), rho, stol=1e-14), rho)
    h = 1e-4
    errs = []
    for i in torch.tensor(g["sample_idx"]).tolist():
        rp, rm = rho0.clone(), rho0.clone()
        rp[i] += h
        rm[i] -= h
        with torch.no_grad():
            Lp = float(compliance(simp(400, 200, rp), rp, stol=1e-14))
            Lm = float(compliance(simp(400, 200, rm), rm, stol=1e-14))
        errs.append(abs((Lp - Lm) / (2 * h) - float(gr[i])) / abs(float(gr[i])))
    assert max(errs) <= 1e-3, errs


# ------------------------------------------------------------ full sizes ---
def test_config4_full_size_gradient_central_differences(cuda):
    """Config 4 at full size (30 x 10 x 10 box, 6 Tetra2 per hex, 80,703 DOF,
    Neo-Hookean, nlgeom, x = 3 face pulled to +0.5): d(tip reaction)/dE_e
    through the adjoint against central differences on the 2 most sensitive
    elements (h = 1e-3 E_e).  40 load increments: the substepping keeps the
    reference's warm start (the previous substep's du, unscaled), which on
    this mesh overshoots into inverted elements after a cutback with 10 or 20
    increments, the same in the reference's algorithm as here."""
    from torchfem_gb300.materials import Hyperelastic3D, neo_hookean_psi

    nodes, el = mesh.linear_to_quadratic(*mesh.box_tetra6(31, 11, 11, 3.0, 1.0, 1.0))
    gen = torch.Generator().manual_seed(0)
    E0 = 1000.0 * (1.0 + 0.1 * torch.randn(len(el), generator=gen, dtype=torch.float64))
    nu = 0.45
    right = nodes[:, 0] == 3.0

    def reaction(E):
        mu = E / (2.0 * (1.0 + nu))
        lbd = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
        m = Solid(nodes, el, Hyperelastic3D(neo_hookean_psi, torch.stack([mu, lbd], dim=-1)))
        m.constraints[nodes[:, 0] == 0.0, :] = True
        m.constraints[right, 0] = True
        m.displacements[right, 0] = 0.5
        assert m.n_dofs == 80_703
        _, f, _, _, _ = m.solve(increments=torch.linspace(0.0, 1.0, 41), nlgeom=True, rtol=1e-10, atol=1e-10,
                                max_iter=20, stol=1e-12, differentiable_parameters=E)
        return f[right, 0].sum()

    E = E0.clone().requires_grad_(True)
    (gE,) = torch.autograd.grad(reaction(E), E)
    # the two most sensitive elements: their difference quotients stand well
    # above the solves' stopping noise
    idx = torch.argsort(gE.abs(), descending=True)[:2]
    for i in idx.tolist():
        h = 1e-3 * float(E0[i])
        Ep, Em = E0.clone(), E0.clone()
        Ep[i] += h
        Em[i] -= h
        with torch.no_grad():
            fd = (float(reaction(Ep)) - float(reaction(Em))) / (2 * h)
        assert abs(fd - float(gE[i])) <= 1e-4 * abs(float(gE[i])) + 1e-12


def test_config5_full_size_vs_reference(cuda, golden):
    """Config 5 at full size (O-grid 256 x 64 plate with a hole, J2 plane
    strain, 20 increments, 33,280 DOF): u, f, state and the reaction's
    thickness gradient through the checkpointed adjoint against the
    reference (its own solve and autograd at the same size)."""
    g = golden("plastic_ogrid_256x64.npz")
    m, t, right = _plastic_model(g)
    assert m.n_dofs == 33_280
    u, f, s, _, st = m.solve(increments=torch.linspace(0.0, 1.0, 21), rtol=1e-12, atol=1e-12, max_iter=80,
                             stol=1e-13, differentiable_parameters=t)
    assert float(st[:, 0].max()) > 0.0
    assert rel(u, g["u"]) <= 1e-8
    assert rel(f, g["f"]) <= 1e-8
    assert rel(s, g["sigma"]) <= 1e-8
    assert rel(st, g["state"]) <= 1e-8
    R = f[right, 0].sum()
    assert abs(float(R.detach()) - float(g["reaction"])) <= 1e-8 * abs(float(g["reaction"]))
    (gt,) = torch.autograd.grad(R, t)
    assert rel(gt, g["grad_t"]) <= 1e-7
