"""The configurations at their stated sizes, pinned to the reference.

Each test runs one configuration at full size on the GPU, through the public
API, and compares it with fixtures written by the reference itself
(`tests/golden/make_golden.py`):

- config 1, the 10^3 Hexa1 cube (268,119 stored values): FP64 assembly bit for
  bit against the reference's own assemble_matrix given its element
  matrices, and on the jittered 10^3 cube (where summing in another order
  changes thousands of slots) against the oracle's serial-order assembly,
  which the CPU tests pin to the reference's;
- config 2, the 70^3 jittered Hexa1 cube (1,073,733 DOF): the reference's own
  pattern, element matrices, assembly and autograd with its CG route
  (`sparse_solve(method="cg")`, Jacobi, stol 1e-13), which reproduces its
  direct solve to 1e-13 on the 20^3 and 30^3 cubes of the same kind
  (`c2_route_crosscheck.npz`).  The fixture holds seeded samples of u, f,
  sigma and d(sum u)/d(forces), their max-abs values and 2-norms, and
  full-field checksums <w, x>.

- config 3, the SIMP cantilever (Quad1 400 x 200, 161,202 DOF) in mixed
  precision: compliance and dL/drho on the reference's 20 seeded elements
  against simp_400x200.npz.  The 125x stiffness contrast limits how deep
  FP64 refinement of an FP32 matrix reaches: the tests refine to 1e-10
  (the configuration's mixed-precision target) and check that 1e-12 is
  refused with an error rather than returned inaccurate;
- config 5, the O-grid plate with a hole (256 x 64, 33,280 DOF, J2 plane
  strain, 20 increments) in mixed precision against the reference's own
  full-size run (plastic_ogrid_256x64.npz).

Tolerance: 1e-8 relative (max-abs error over max-abs value), the accuracy
target of the forward + adjoint path; gradients of nonlinear solves 1e-7.
"""

import hashlib

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

RTOL = 1e-8


def _weights(n):
    """The checksum weights of make_golden.py (_projection_weights)."""
    return np.cos(np.arange(n, dtype=np.float64) * 0.6180339887498949)


def _check_sampled(name, x, g, rtol=RTOL):
    """x (full field, host) against the fixture's sample, norm and checksum."""
    x = np.asarray(x, dtype=np.float64).ravel()
    ref = g[f"{name}_sample"]
    err = float(np.abs(x[g[f"{name}_idx"]] - ref).max() / float(g[f"{name}_maxabs"]))
    assert err <= rtol, (name, "sample", err)
    nrm = float(np.linalg.norm(x))
    assert abs(nrm - float(g[f"{name}_norm"])) <= rtol * float(g[f"{name}_norm"]), (name, "norm")
    proj = float(_weights(x.size) @ x)
    perr = abs(proj - float(g[f"{name}_proj"])) / float(g[f"{name}_projscale"])
    assert perr <= rtol, (name, "checksum", perr)
    return err


@pytest.mark.parametrize("precision,precond", [("mixed", "amg"), ("mixed", "jacobi"), ("fp64", None)])
def test_config2_full_size_vs_reference(cuda, golden, precision, precond):
    """Config 2 (70^3 jittered Hexa1, 1,073,733 DOF): u, f, sigma and
    d(sum u)/d(forces) of the mixed path (multigrid and block Jacobi) and of
    the FP64 path against the reference's FP64 solve, to 1e-8, with the
    solves refined to the configuration's relative residual 1e-10."""
    import bench

    g = golden("c2_cube70_sample.npz")
    nodes, _ = bench.cube_nodes(70)
    assert hashlib.sha256(np.ascontiguousarray(nodes.numpy())).hexdigest() == str(g["nodes_sha256"])
    m, forces = bench.cube_workload(70, cuda)
    assert m.n_dofs == int(g["n_dofs"]) == 1_073_733
    u, f, s, _, _, gr = bench.step(m, forces, precision, 1e-10, precond=precond)
    errs = {k: _check_sampled(k, v.detach().cpu().numpy(), g)
            for k, v in (("u", u), ("f", f), ("sigma", s), ("grad", gr))}
    print(precision, precond, errs)


def test_config1_assembly_bit_exact(cuda, golden):
    """Config 1: the GPU's atomic-free assembly of the reference's element
    matrices equals the reference's condensed values bit for bit."""
    from torchfem_gb300 import Solid, mesh
    from torchfem_gb300.materials import IsotropicElasticity3D

    g = golden("c1_cube10.npz")
    nodes, el = mesh.cube_hexa(11, 11, 11)
    m = Solid(nodes.to(cuda), el.to(cuda), IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[(nodes[:, 0] == 0.0).to(cuda), :] = True
    dm = m.device_mesh
    assert dm.nnz == 268_119
    con = m.constraints.reshape(-1).to(torch.uint8).contiguous()
    val = dm.assemble_csr(torch.tensor(g["ke"], device=cuda).contiguous(), con).cpu().numpy()
    assert np.array_equal(val, g["kval"])  # bit for bit


def test_jittered_cube10_assembly_order_bit_exact(cuda):
    """On the jittered 10^3 cube every element matrix differs, so the order
    of the up to 8 contributions to a slot shows in the last bits.  The GPU
    assembly of the GPU's own element matrices equals the oracle's serial
    ascending-order sums (np.add.at, the order of the reference's CPU
    index_add_) bit for bit, and reversing that order changes thousands of
    slots (so the test can see an order change)."""
    import bench
    from oracle import fem_oracle as O

    nodes, el = bench.cube_nodes(10)
    m, _ = bench.cube_workload(10, cuda)
    dm = m.device_mesh
    con = m.constraints.reshape(-1).to(torch.uint8).contiguous()
    mesh_s, mat, refs = m._device_material()
    ke = dm.element_stiffness(mesh_s, mat, torch.float64)
    val = dm.assemble_csr(ke, con).cpu().numpy()
    k = ke.cpu().numpy()
    om = O.LinearModel(nodes.numpy(), el.numpy(), O.elastic_c("3d", 1000.0, 0.3, len(el)))
    con_idx = np.flatnonzero(m.constraints.reshape(-1).cpu().numpy())
    ref = O.assemble_matrix(k, om.k_map, om.glob_idx.shape[1], om.glob_idx, om.diag_map, con_idx)
    assert np.array_equal(val, ref)  # bit for bit
    rev = np.zeros_like(ref)
    order = np.arange(om.k_map.size)[::-1]
    np.add.at(rev, om.k_map[order], k.ravel()[order])
    is_con = np.zeros(om.n_dofs, dtype=bool)
    is_con[con_idx] = True
    free = ~(is_con[om.glob_idx[0]] | is_con[om.glob_idx[1]])
    assert int((rev[free] != ref[free]).sum()) > 1000


def _simp(rho):
    from torchfem_gb300 import Planar, mesh
    from torchfem_gb300.materials import IsotropicElasticityPlaneStress

    nodes, el = mesh.rect_quad(401, 201, 2.0, 1.0)
    m = Planar(nodes, el, IsotropicElasticityPlaneStress(rho**3 * 1.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    tip = torch.argmin(((nodes - torch.tensor([2.0, 0.5])) ** 2).sum(1))
    m.forces[tip, 1] = -1.0
    return m


def _simp_rho():
    return 0.2 + 0.8 * torch.rand(80000, generator=torch.Generator().manual_seed(0), dtype=torch.float64)


def test_config3_mixed_vs_reference(cuda, golden):
    """Config 3 in mixed precision with the multigrid preconditioner (FP32 K
    and CG, FP64 refinement to 1e-10): compliance and the reference's 20
    sampled dL/drho to 1e-8.  (With block Jacobi the adjoint's FP32 CG runs
    to the 10 n iteration cap on this contrast, so config 3 in mixed
    precision needs the multigrid.)"""
    precond = "amg"
    g = golden("simp_400x200.npz")
    rho = _simp_rho().requires_grad_(True)
    m = _simp(rho)
    u, f, _, _, _ = m.solve(stol=1e-10, precision="mixed", preconditioner=precond, differentiable_parameters=rho)
    L = torch.inner(f.ravel(), u.ravel())
    assert abs(float(L.detach()) - float(g["compliance"])) <= RTOL * abs(float(g["compliance"]))
    (gr,) = torch.autograd.grad(L, rho)
    idx = torch.tensor(g["sample_idx"])
    ref = torch.tensor(g["grad_rho_sample"])
    err = float((gr[idx].cpu() - ref).abs().max() / ref.abs().max())
    assert err <= RTOL, err
    assert abs(float(gr.norm()) - float(g["grad_norm"])) <= RTOL * float(g["grad_norm"])


def test_config3_mixed_refinement_floor_is_refused(cuda):
    """FP64 refinement of the FP32 SIMP matrix stagnates above 1e-12: the
    solve stops with an error (the stagnation or iteration-cap message,
    chained under the reference's cutback message) instead of returning an
    inaccurate result.  The FP32 CG is capped at 5,000 iterations: with the
    default cap of 10 n it runs 1.6M iterations (400 s) before it stops."""
    m = _simp(_simp_rho())
    with pytest.raises(RuntimeError) as info:
        m.solve(stol=1e-12, precision="mixed", preconditioner="jacobi", cg_max_iter=5000)
    msg = str(info.value) + " " + str(info.value.__cause__)
    assert "stagnated" in msg or "did not converge" in msg or "failed" in msg, msg


@pytest.mark.parametrize("precond", ["amg", "jacobi"])
def test_config5_mixed_vs_reference(cuda, golden, precond):
    """Config 5 in mixed precision: u, f, sigma, state, the reaction and its
    thickness gradient against the reference's full-size run (1e-8, the
    gradient 1e-7)."""
    from torchfem_gb300 import Planar
    from torchfem_gb300.materials import IsotropicPlasticityPlaneStrain

    g = golden("plastic_ogrid_256x64.npz")
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
    assert m.n_dofs == 33_280
    u, f, s, _, st = m.solve(increments=torch.linspace(0.0, 1.0, 21), rtol=1e-12, atol=1e-12, max_iter=80,
                             stol=1e-12, precision="mixed", preconditioner=precond, differentiable_parameters=t)

    def rel(a, b):
        return float(np.abs(a.detach().cpu().numpy() - b).max() / np.abs(b).max())

    assert rel(u, g["u"]) <= RTOL
    assert rel(f, g["f"]) <= RTOL
    assert rel(s, g["sigma"]) <= RTOL
    assert rel(st, g["state"]) <= RTOL
    R = f[right.to(f.device), 0].sum()
    assert abs(float(R.detach()) - float(g["reaction"])) <= RTOL * abs(float(g["reaction"]))
    (gt,) = torch.autograd.grad(R, t)
    assert rel(gt, g["grad_t"]) <= 1e-7


def _hyper(g, E):
    from torchfem_gb300 import Solid
    from torchfem_gb300.materials import Hyperelastic3D, neo_hookean_psi

    nodes = torch.tensor(g["nodes"])
    el = torch.tensor(g["elements"])
    nu = 0.45
    mu = E / (2.0 * (1.0 + nu))
    lbd = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    m = Solid(nodes, el, Hyperelastic3D(neo_hookean_psi, torch.stack([mu, lbd], dim=-1)))
    right = nodes[:, 0] == 3.0
    m.constraints[nodes[:, 0] == 0.0, :] = True
    m.constraints[right, 0] = True
    m.displacements[right, 0] = 0.5
    return m, right


@pytest.mark.parametrize("precision,precond", [("fp64", None), ("mixed", "amg")])
def test_config4_problem_increments_like_the_reference(cuda, golden, precision, precond):
    """Config 4's problem (Neo-Hookean Tetra2 box pulled to +0.5, nlgeom) at
    half the resolution, where the reference's direct solve is affordable
    (hyper_tet2_15x5x5.npz, 11,163 DOF): with the 10 load increments the
    configuration states, the reference's own solve raises (its warm start,
    the previous substep's increment, overshoots after a cutback); the GPU
    path raises with the same message.  With 20 increments both complete:
    u, f, sigma and the tip reaction to 1e-8, d(reaction)/dE_e to 1e-7."""
    g = golden("hyper_tet2_15x5x5.npz")
    E0 = torch.tensor(g["E"])
    m, right = _hyper(g, E0)
    with pytest.raises(RuntimeError, match="increment 9 after 10 cutbacks"):
        m.solve(increments=torch.linspace(0.0, 1.0, 11), nlgeom=True, rtol=1e-10, atol=1e-10, max_iter=20,
                stol=1e-12, precision=precision, preconditioner=precond)
    assert str(g["inc10_error"]).endswith("increment 9 after 10 cutbacks.")
    E = E0.clone().requires_grad_(True)
    m, right = _hyper(g, E)
    u, f, s, _, _ = m.solve(increments=torch.linspace(0.0, 1.0, int(g["increments"]) + 1), nlgeom=True, rtol=1e-10,
                            atol=1e-10, max_iter=20, stol=1e-12, precision=precision, preconditioner=precond,
                            differentiable_parameters=E)

    def rel(a, b):
        return float(np.abs(a.detach().cpu().numpy() - b).max() / np.abs(b).max())

    assert rel(u, g["u"]) <= RTOL
    assert rel(f, g["f"]) <= RTOL
    assert rel(s, g["sigma"]) <= RTOL
    R = f[right.to(f.device), 0].sum()
    assert abs(float(R.detach()) - float(g["reaction"])) <= RTOL * abs(float(g["reaction"]))
    (gE,) = torch.autograd.grad(R, E)
    assert rel(gE, g["grad_E"]) <= 1e-7
