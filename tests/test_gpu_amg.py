"""GPU tests of the smoothed-aggregation multigrid preconditioner (fem_amg_*).

Hierarchy parity against the CPU restatement in oracle/amg_oracle.py:
aggregation and every sparsity pattern bit for bit; the tentative
prolongator, smoothed prolongator and coarse operator to FP32 tolerance
(1e-5 / 1e-4 relative: the GPU builds them in FP32 from the FP32 matrix, the
oracle in FP64); the spectral estimate between 0.95 and 1 times the exact
largest eigenvalue of D^-1 A.  Solutions and gradients of the
multigrid-preconditioned mixed path against the reference's golden vectors
to 1e-8 relative, as for the block-Jacobi path.
"""

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch

from oracle import amg_oracle as AO
from oracle import fem_oracle as O
from torchfem_gb300 import Planar, Solid, _lib, mesh
from torchfem_gb300.materials import IsotropicElasticity3D, IsotropicElasticityPlaneStress

pytestmark = pytest.mark.gpu

RTOL = 1e-8


def rel(a, b):
    a = a.detach().cpu().double().numpy() if torch.is_tensor(a) else np.asarray(a)
    b = b.detach().cpu().double().numpy() if torch.is_tensor(b) else np.asarray(b)
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def fetch(lib, address, count, dtype):
    """Copies `count` elements at a handle-owned device address to numpy."""
    t = torch.empty(max(int(count), 1), dtype=dtype, device="cuda")
    if count:
        _lib.check(lib.fem_copy_device(t.data_ptr(), address, int(count) * t.element_size(),
                                       torch.cuda.current_stream().cuda_stream), "fem_copy_device")
    torch.cuda.synchronize()
    return t.cpu().numpy()[: int(count)]


def jittered_cube(n, seed=0, amp=0.1):
    nodes, el = mesh.cube_hexa(n + 1, n + 1, n + 1)
    h = 1.0 / n
    gen = torch.Generator().manual_seed(seed)
    inner = ((nodes > 0) & (nodes < 1)).all(1)
    jit = (torch.rand(nodes.shape, generator=gen, dtype=torch.float64) * 2 - 1) * amp * h
    return nodes + inner[:, None] * jit, el


def cube_problem(n):
    nodes, el = jittered_cube(n)
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    # partially constrained nodes: the x = 1 face may only slide in y and z
    m.constraints[nodes[:, 0] == 1.0, 0] = True
    m.forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    return m, nodes, el


def test_amg_hierarchy_matches_oracle(cuda):
    m, nodes, el = cube_problem(12)
    u, f, s, _, _ = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")
    sysm = m.last_solve.system
    amg = sysm.amg
    assert amg is not None
    lib = amg.lib
    levels = amg.levels()
    dm = m.device_mesh

    # the solution itself, against the oracle's direct solve
    om = O.LinearModel(nodes.numpy(), el.numpy(), O.elastic_c("3d", 1000.0, 0.3, len(el)))
    con = m.constraints.cpu().numpy()
    uo, fo, so = om.solve(m.forces.cpu().numpy(), con)
    assert rel(u, uo) <= RTOL and rel(s, so) <= RTOL
    assert m.last_solve.iterations[0] <= 40

    K = om.matrix(np.nonzero(con.ravel())[0]).tocsr()
    n = len(nodes)
    ptr = dm.nbr_ptr.cpu().numpy()
    idx = dm.nbr.cpu().numpy().astype(np.int64)
    active = ~np.all(con, axis=1)

    # level 0: aggregation bit for bit
    L0 = levels[0]
    agg = fetch(lib, L0.agg, n, torch.int32)
    agg_o, na_o = AO.aggregate(ptr, idx, active)
    assert L0.n_agg == na_o
    assert np.array_equal(agg, agg_o)

    # tentative prolongator
    T_o, Bc_o = AO.tentative(agg_o, na_o, 3, 6, coords=nodes.numpy(), con=con.ravel())
    T = fetch(lib, L0.tval, n * 18, torch.float32).reshape(n, 3, 6)
    assert np.abs(T - T_o).max() <= 1e-5 * np.abs(T_o).max()

    # smoothed prolongator: pattern exact, values with the GPU's spectral estimate
    p_ptr = fetch(lib, L0.p_ptr, n + 1, torch.int64)
    p_col = fetch(lib, L0.p_col, L0.p_nnz, torch.int32)
    for i in range(n):
        row = sorted({int(agg_o[j]) for j in idx[ptr[i]:ptr[i + 1]] if agg_o[j] >= 0}) if active[i] else []
        assert list(p_col[p_ptr[i]:p_ptr[i + 1]]) == row
    Dinv = AO.bsr_blockdiag(AO.block_diag_inv(K, 3))
    Ts = AO.to_sparse_T(T_o, agg_o, 6)
    P_o = (Ts - (AO.OMEGA / L0.rho) * (Dinv @ (K @ Ts))).toarray()
    p_val = fetch(lib, L0.p_val, L0.p_nnz * 18, torch.float32).reshape(-1, 3, 6)
    P = np.zeros_like(P_o)
    for i in range(n):
        for e in range(p_ptr[i], p_ptr[i + 1]):
            J = p_col[e]
            P[3 * i:3 * i + 3, 6 * J:6 * J + 6] = p_val[e]
    assert np.abs(P - P_o).max() <= 1e-4 * np.abs(P_o).max()

    # spectral estimate of D^-1 A: below and close to the exact largest eigenvalue
    Db = sp.bsr_matrix((np.linalg.inv(AO.block_diag_inv(K, 3)), np.arange(n), np.arange(n + 1)),
                       shape=K.shape).tocsr()
    lam = float(spla.eigsh(K, k=1, M=Db, which="LA", return_eigenvectors=False)[0])
    assert 0.95 * lam <= L0.rho <= lam * (1.0 + 1e-4), (L0.rho, lam)

    # level 1: the Galerkin operator
    L1 = levels[1]
    a_ptr = fetch(lib, L1.a_ptr, L1.n + 1, torch.int64)
    a_col = fetch(lib, L1.a_col, L1.a_nnz, torch.int32)
    a_val = fetch(lib, L1.a_val, L1.a_nnz * 36, torch.float32).reshape(-1, 6, 6)
    Ac = sp.bsr_matrix((a_val, a_col, a_ptr), shape=(6 * L1.n, 6 * L1.n)).toarray()
    Ac_o = P_o.T @ K.toarray() @ P_o
    zero = np.diag(Ac_o) == 0.0
    Ac_o[np.diag_indices_from(Ac_o)] += zero
    assert np.abs(Ac - Ac_o).max() <= 1e-4 * np.abs(Ac_o).max()
    assert np.abs(Ac - Ac.T).max() <= 1e-5 * np.abs(Ac).max()

    # the whole hierarchy: level sizes of the oracle with the GPU's estimates
    rhos = [lv.rho for lv in levels[:-1]]
    lo = AO.hierarchy(K, nodes.numpy(), con.ravel(), 3, rhos=rhos)
    assert [lv.n for lv in levels] == [x.A.shape[0] // x.b for x in lo]


def test_amg_c1_forward_and_adjoint(cuda, golden):
    """Config 1 through the multigrid-preconditioned mixed path: u, f, sigma
    and d(sum u)/d(forces) against the reference."""
    g = golden("c1_cube10.npz")
    nodes, el = mesh.cube_hexa(11, 11, 11)
    m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    forces = torch.zeros_like(nodes)
    forces[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    forces.requires_grad_(True)
    m.forces = forces
    u, f, s, _, _ = m.solve(stol=1e-12, precision="mixed", preconditioner="amg", differentiable_parameters=forces)
    assert rel(u, g["u"]) <= RTOL
    assert rel(f, g["f"]) <= RTOL
    assert rel(s, g["sigma"]) <= RTOL
    (gf,) = torch.autograd.grad(u.sum(), forces)
    assert rel(gf, g["grad_forces"]) <= RTOL
    assert max(m.last_solve.iterations) <= 40


def test_amg_jittered_cube_gradients(cuda, golden):
    g = golden("hexa_jitter3.npz")
    E = torch.tensor(g["E"], requires_grad=True)
    m = Solid(torch.tensor(g["nodes"]), torch.tensor(g["elements"]), IsotropicElasticity3D(E, 0.3))
    m.constraints = torch.tensor(g["constraints"])
    forces = torch.tensor(g["forces"]).requires_grad_(True)
    m.forces = forces
    u, f, s, gr, _ = m.solve(stol=1e-12, precision="mixed", preconditioner="amg",
                             differentiable_parameters=(forces, E))
    assert rel(u, g["u"]) <= RTOL
    assert rel(s, g["sigma"]) <= RTOL
    (gf,) = torch.autograd.grad(u.sum(), forces, retain_graph=True)
    assert rel(gf, g["grad_forces"]) <= RTOL
    L = torch.inner(f.ravel(), u.ravel())
    (gE,) = torch.autograd.grad(L, E)
    assert rel(gE, g["grad_E"]) <= RTOL


def test_amg_planar_matches_oracle(cuda):
    """2D (Quad1 plane stress): 3 rigid-body modes per aggregate."""
    nodes, el = mesh.rect_quad(61, 31, 2.0, 1.0)
    m = Planar(nodes, el, IsotropicElasticityPlaneStress(1000.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    tip = torch.argmin(((nodes - torch.tensor([2.0, 0.5])) ** 2).sum(1))
    m.forces[tip, 1] = -1.0
    u, f, s, _, _ = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")
    om = O.LinearModel(nodes.numpy(), el.numpy(), O.elastic_c("plane_stress", 1000.0, 0.3, len(el)))
    uo, fo, so = om.solve(m.forces.cpu().numpy(), m.constraints.cpu().numpy())
    assert rel(u, uo) <= RTOL
    assert rel(s, so) <= RTOL
    assert max(m.last_solve.iterations) <= 60
    levels = m.last_solve.system.amg.levels()
    assert levels[0].block == 2 and levels[1].block == 3


def test_amg_neo_hookean_tetra2_vs_reference(cuda, golden):
    """Config 4 at small size with multigrid-preconditioned Newton solves."""
    from test_gpu_parity import _hyper_model

    g = golden("hyper_tet2_6x2x2.npz")
    m, E, right = _hyper_model(g)
    u, f, s, F, _ = m.solve(increments=torch.linspace(0.0, 1.0, 11), nlgeom=True, rtol=1e-10, atol=1e-10,
                            max_iter=20, stol=1e-13, precision="mixed", preconditioner="amg",
                            differentiable_parameters=E)
    assert rel(u, g["u"]) <= 1e-8
    assert rel(s, g["sigma"]) <= 1e-8
    R = f[right, 0].sum()
    (gE,) = torch.autograd.grad(R, E)
    assert rel(gE, g["grad_E"]) <= 1e-7


def test_amg_plane_strain_plasticity_vs_reference(cuda, golden):
    """Config 5 at small size (2D, J2 plasticity) with the multigrid path."""
    from test_gpu_parity import _plastic_model

    g = golden("plastic_ogrid_32x8.npz")
    m, t, right = _plastic_model(g)
    u, f, s, _, st = m.solve(increments=torch.linspace(0.0, 1.0, 21), rtol=1e-12, atol=1e-12, max_iter=80,
                             stol=1e-13, precision="mixed", preconditioner="amg", differentiable_parameters=t)
    assert rel(u, g["u"]) <= 1e-8
    assert rel(st, g["state"]) <= 1e-8
    R = f[right, 0].sum()
    (gt,) = torch.autograd.grad(R, t)
    assert rel(gt, g["grad_t"]) <= 1e-7


def test_amg_deterministic(cuda):
    m, _, _ = cube_problem(10)
    u1 = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")[0].clone()
    u2 = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")[0]
    assert torch.equal(u1, u2)


def test_amg_fp64_request_rejected(cuda):
    m, _, _ = cube_problem(4)
    with pytest.raises(ValueError):
        m.solve(precision="fp64", preconditioner="amg")


@pytest.fixture
def half_smoother():
    """Restores the default (FP16 level-0 smoothing copy) after a test."""
    lib = _lib.load()
    yield lib
    lib.fem_amg_set_half_smoother(1)


def _its(m):
    it = m.last_solve.iterations
    return sum(it) if isinstance(it, (list, tuple)) else it


@pytest.mark.parametrize("kind", ["elastic", "heat"])
def test_amg_half_smoother_matches_fp32_smoother(cuda, half_smoother, kind):
    """The FP16 copy of the level-0 matrix in the four smoothing passes
    changes the preconditioner, not the system: the solutions agree with the
    FP32-smoothed V-cycle to 1e-8 (both refine to stol in FP64), and CG needs
    at most 15 % more iterations."""
    lib = half_smoother
    if kind == "elastic":
        m, _, _ = cube_problem(20)
    else:
        from torchfem_gb300 import SolidHeat
        from torchfem_gb300.materials import IsotropicConductivity3D

        nodes, el = jittered_cube(20)
        kappa = 1.0 + torch.rand(len(el), generator=torch.Generator().manual_seed(3), dtype=torch.float64)
        m = SolidHeat(nodes.to(cuda), el.to(cuda), IsotropicConductivity3D(kappa.to(cuda)))
        m.constraints[(nodes[:, 0] == 0.0).to(cuda)] = True
        m.heat_flux[:] = 1.0 / len(nodes)
    out, its = {}, {}
    for half in (0, 1):
        lib.fem_amg_set_half_smoother(half)
        out[half] = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")[0].clone()
        assert m.last_solve.system.amg is not None
        its[half] = _its(m)
    assert rel(out[1], out[0]) <= RTOL
    assert its[1] <= 1.15 * its[0] + 1, its


@pytest.mark.parametrize("kind", ["elastic", "planar", "heat"])
def test_amg_fused_coarse_cycle_matches_per_level_kernels(cuda, half_smoother, kind):
    """The coarse levels of the V-cycle as one cooperative launch (grid
    barriers between phases) against one launch per level operation: the
    same preconditioner up to the order of partial row sums, so the solutions
    agree to 1e-8, CG iteration counts within one, and repeated fused solves
    are bitwise identical."""
    lib = half_smoother
    if kind == "elastic":
        m, _, _ = cube_problem(16)
    elif kind == "planar":
        nodes, el = mesh.rect_quad(41, 21, 2.0, 1.0)
        m = Planar(nodes.to(cuda), el.to(cuda), IsotropicElasticityPlaneStress(1000.0, 0.3))
        m.constraints[(nodes[:, 0] == 0.0).to(cuda), :] = True
        m.forces[(nodes[:, 0] == 2.0).to(cuda), 1] = -1.0
    else:
        from torchfem_gb300 import SolidHeat
        from torchfem_gb300.materials import IsotropicConductivity3D

        nodes, el = jittered_cube(24)
        m = SolidHeat(nodes.to(cuda), el.to(cuda), IsotropicConductivity3D(1.0))
        m.constraints[(nodes[:, 0] == 0.0).to(cuda)] = True
        m.heat_flux[:] = 1.0 / len(nodes)
    out, its = {}, {}
    try:
        for fused in (0, 1):
            lib.fem_amg_set_fused_cycle(fused)
            out[fused] = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")[0].clone()
            assert m.last_solve.system.amg is not None
            assert len(m.last_solve.system.amg.levels()) >= 3
            its[fused] = list(m.last_solve.iterations)
        again = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")[0]
    finally:
        lib.fem_amg_set_fused_cycle(1)
    assert torch.equal(again, out[1])
    assert rel(out[1], out[0]) <= RTOL
    assert all(abs(a - b) <= 1 for a, b in zip(its[0], its[1])), its


@pytest.mark.parametrize("kind", ["elastic", "planar", "heat"])
def test_amg_level0_bulk_copies_match_direct_loads(cuda, half_smoother, kind):
    """Level-0 SpMVs with each slice streamed into shared memory by bulk
    copies (fem_amg_set_level0_tma) against direct loads: the same sums in
    the same order, so the solutions are bitwise identical (3x3 and 2x2
    blocks, and scalar rows)."""
    lib = half_smoother
    if kind == "elastic":
        m, _, _ = cube_problem(16)
    elif kind == "heat":
        from torchfem_gb300 import SolidHeat
        from torchfem_gb300.materials import IsotropicConductivity3D

        nodes, el = jittered_cube(24)
        m = SolidHeat(nodes.to(cuda), el.to(cuda), IsotropicConductivity3D(1.0))
        m.constraints[(nodes[:, 0] == 0.0).to(cuda)] = True
        m.heat_flux[:] = 1.0 / len(nodes)
    else:
        nodes, el = mesh.rect_quad(41, 21, 2.0, 1.0)
        m = Planar(nodes.to(cuda), el.to(cuda), IsotropicElasticityPlaneStress(1000.0, 0.3))
        m.constraints[(nodes[:, 0] == 0.0).to(cuda), :] = True
        m.forces[(nodes[:, 0] == 2.0).to(cuda), 1] = -1.0
    out = {}
    try:
        for tma in (0, 1):
            lib.fem_amg_set_level0_tma(tma)
            out[tma] = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")[0].clone()
    finally:
        lib.fem_amg_set_level0_tma(1)
    assert torch.equal(out[1], out[0])


@pytest.mark.parametrize("kind", ["elastic", "heat"])
def test_amg_programmatic_dependent_launch_is_bitwise_neutral(cuda, half_smoother, kind):
    """The CG iteration's kernels launched with programmatic dependent launch
    (fem_amg_set_pdl) do the same work in the same order: bitwise the same
    solution as ordinary launches."""
    lib = half_smoother
    if kind == "elastic":
        m, _, _ = cube_problem(16)
    else:
        from torchfem_gb300 import SolidHeat
        from torchfem_gb300.materials import IsotropicConductivity3D

        nodes, el = jittered_cube(24)
        m = SolidHeat(nodes.to(cuda), el.to(cuda), IsotropicConductivity3D(1.0))
        m.constraints[(nodes[:, 0] == 0.0).to(cuda)] = True
        m.heat_flux[:] = 1.0 / len(nodes)
    out = {}
    try:
        for pdl in (0, 1):
            lib.fem_amg_set_pdl(pdl)
            out[pdl] = m.solve(stol=1e-12, precision="mixed", preconditioner="amg")[0].clone()
    finally:
        lib.fem_amg_set_pdl(1)
    assert torch.equal(out[1], out[0])


def test_amg_rebind_keeps_the_preconditioner_and_solves_the_new_matrix(cuda, half_smoother):
    """fem_amg_rebind: the hierarchy set up for one stiffness preconditions a
    changed one (a stiffer half of the cube); CG on the new matrix with FP64
    refinement reaches the same solution as a fresh setup to 1e-8, in more
    iterations at most 2x, and the set-up matrix solves bitwise as before."""
    from torchfem_gb300.materials import IsotropicElasticity3D as Iso

    m, nodes, el = cube_problem(12)
    dm = m.device_mesh
    con_cpu = m.constraints.reshape(-1).cpu()
    con = con_cpu.to(torch.uint8).to(dm.device).contiguous()
    f = m.forces.reshape(-1).cpu()
    b = torch.where(con_cpu, torch.zeros_like(f), f).to(dm.device)

    def system(scale, reuse):
        E = torch.full((len(el),), 1000.0, dtype=torch.float64)
        E[nodes[el].mean(1)[:, 0] > 0.5] *= scale
        kind, data = Iso(E, 0.3).kernel_data(len(el))
        data = data.to(dm.device, torch.float64).contiguous()
        mesh = dm.make_mesh(None)
        mat = _lib.FemMaterial(kind, data.data_ptr())
        sysm = dm.build_system(mesh, mat, con, "mixed", keep_refs=(data, mesh, mat), precond="amg", amg_reuse=reuse)
        return sysm

    s1 = system(1.0, False)
    x1 = dm.solve(s1, b.contiguous(), 1e-12, None, 1e-4)
    fresh = system(3.0, False)
    x_fresh = dm.solve(fresh, b.contiguous(), 1e-12, None, 1e-4)
    it_fresh = fresh.stats.iterations
    s1 = system(1.0, False)
    lag = system(3.0, True)
    assert lag.amg_fresh is False
    x_lag = dm.solve(lag, b.contiguous(), 1e-12, None, 1e-4)
    assert rel(x_lag, x_fresh) <= RTOL
    assert lag.stats.iterations <= 2 * it_fresh + 2
    again = system(1.0, False)
    assert torch.equal(dm.solve(again, b.contiguous(), 1e-12, None, 1e-4), x1)
    # without the FP16 smoothing copy the V-cycle would smooth on the new matrix
    lib = half_smoother
    lib.fem_amg_set_half_smoother(0)
    try:
        with pytest.raises(ValueError, match="FP16 smoothing copy"):
            system(3.0, True)
    finally:
        lib.fem_amg_set_half_smoother(1)


def test_config2_full_size_amg_iterations(cuda, half_smoother):
    """Config 2 at full size (70^3 jittered Hexa1, 1,073,733 DOF): the
    V-cycle CG iteration counts of solve + adjoint stay flat (tens, against
    about 1,200 with block Jacobi), with the FP16 smoothing copy as with the
    FP32 matrix.  Accuracy against the reference at this size is
    tests/test_gpu_fullsize.py."""
    import bench

    lib = half_smoother
    m, forces = bench.cube_workload(70, cuda)
    its = {}
    for half in (0, 1):
        lib.fem_amg_set_half_smoother(half)
        bench.step(m, forces, "mixed", 1e-10, precond="amg")
        its[half] = list(m.last_solve.iterations)
    assert max(its[0] + its[1]) <= 60, its
    assert sum(its[1]) <= 1.15 * sum(its[0]) + 2, its
