"""The CPU oracle against golden vectors produced by the reference itself."""

import numpy as np
import pytest

from oracle import fem_oracle as O


def test_pattern_hexa(golden):
    g = golden("hexa_jitter3.npz")
    gi, km, dm, _ = O.pattern(g["elements"], len(g["nodes"]), 3)
    assert np.array_equal(gi, g["glob_idx"])
    assert np.array_equal(km, g["k_map"])
    assert np.array_equal(dm, g["diag_map"])


@pytest.mark.parametrize("which", ["tet2", "orphan"])
def test_pattern_tet2_and_orphan(golden, which):
    g = golden("patterns.npz")
    nodes, el = g[f"{which}_nodes"], g[f"{which}_elements"]
    gi, km, dm, _ = O.pattern(el, len(nodes), nodes.shape[1])
    assert np.array_equal(gi, g[f"{which}_glob_idx"])
    assert np.array_equal(km, g[f"{which}_k_map"])
    assert np.array_equal(dm, g[f"{which}_diag_map"])


def test_element_matrices_and_assembly(golden):
    g = golden("hexa_jitter3.npz")
    m = O.LinearModel(g["nodes"], g["elements"], O.elastic_c("3d", 1000.0, 0.3, len(g["elements"])))
    k = m.stiffness()
    assert np.abs(k - g["ke"]).max() <= 1e-13 * np.abs(g["ke"]).max()
    con = np.nonzero(g["constraints"].ravel())[0]
    val = O.assemble_matrix(g["ke"], m.k_map, m.glob_idx.shape[1], m.glob_idx, m.diag_map, con)
    assert np.array_equal(val, g["kval"])  # serial order: bit-identical


def test_c1_solution(golden):
    g = golden("c1_cube10.npz")
    nodes, el = O.cube_hexa(11, 11, 11)
    m = O.LinearModel(nodes, el, O.elastic_c("3d", 1000.0, 0.3, len(el)))
    con = np.zeros_like(nodes, dtype=bool)
    con[nodes[:, 0] == 0.0, :] = True
    F = np.zeros_like(nodes)
    F[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    u, f, s = m.solve(F, con)
    for a, b in ((u, g["u"]), (f, g["f"]), (s, g["sigma"])):
        assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max()
    gf = m.grad_forces(np.ones(m.n_dofs))
    assert np.abs(gf - g["grad_forces"]).max() <= 1e-10 * np.abs(g["grad_forces"]).max()
    # the oracle's element matrices and serial-order assembly against the
    # reference's k0 and assemble_matrix at config 1 (268,119 values)
    assert np.abs(m.stiffness() - g["ke"]).max() <= 1e-13 * np.abs(g["ke"]).max()
    val = O.assemble_matrix(g["ke"], m.k_map, m.glob_idx.shape[1], m.glob_idx, m.diag_map, np.flatnonzero(con))
    assert np.array_equal(val, g["kval"])  # bit for bit


def test_c2_route_reproduces_direct_solve(golden):
    """The reference's CG route that generated the config-2 fixture (Jacobi
    CG to 1e-13) agrees with its direct solve on the 20^3 and 30^3 cubes of
    the same kind far below the 1e-8 target."""
    g = golden("c2_route_crosscheck.npz")
    for n in g["sizes"]:
        for key in ("u", "sigma", "grad"):
            assert float(g[f"n{n}_{key}"]) < 1e-12, (n, key)


def test_hexa_jitter_gradients(golden):
    g = golden("hexa_jitter3.npz")
    el = g["elements"]
    C = O.elastic_c("3d", g["E"], 0.3, len(el))
    m = O.LinearModel(g["nodes"], el, C)
    u, f, s = m.solve(g["forces"], g["constraints"])
    assert np.abs(u - g["u"]).max() <= 1e-10 * np.abs(g["u"]).max()
    # dL/dE for L = f.u: C is linear in E, dC/dE = C/E
    gC = m.compliance_grad_c(u.ravel())
    gE = (gC * C).sum(axis=(1, 2, 3, 4)) / g["E"]
    assert np.abs(gE - g["grad_E"]).max() <= 1e-9 * np.abs(g["grad_E"]).max()


def test_simp_small(golden):
    g = golden("simp_20x10.npz")
    nodes, el = O.rect_quad(21, 11, 2.0, 1.0)
    rho = g["rho"]
    C = O.elastic_c("plane_stress", rho**3, 0.3, len(el))
    m = O.LinearModel(nodes, el, C, thickness=np.ones(len(el)))
    con = np.zeros_like(nodes, dtype=bool)
    con[nodes[:, 0] == 0.0, :] = True
    F = np.zeros_like(nodes)
    F[int(g["tip"]), 1] = -1.0
    u, f, s = m.solve(F, con)
    L = float(np.dot(f.ravel(), u.ravel()))
    assert abs(L - float(g["compliance"])) <= 1e-10 * abs(float(g["compliance"]))
    gC = m.compliance_grad_c(u.ravel())
    grho = (gC * C).sum(axis=(1, 2, 3, 4)) * 3.0 / rho  # E = rho^3
    assert np.abs(grho - g["grad_rho"]).max() <= 1e-9 * np.abs(g["grad_rho"]).max()


def test_material_points(golden):
    """Neo-Hookean stress/tangent and plane-strain J2 return mapping of the
    oracle against the reference's Material.step outputs."""
    g = golden("material_points.npz")
    P, A = O.neo_hookean_point(g["F"], g["mu"], g["lam"])
    assert np.abs(P - g["P"]).max() <= 1e-11 * np.abs(g["P"]).max()
    assert np.abs(A - g["A"]).max() <= 1e-11 * np.abs(g["A"]).max()
    s, st, D = O.j2_plane_strain_point(g["H"], g["stress"], g["state"], 1000.0, 0.3, 1.0, 100.0)
    assert np.abs(s - g["stress_new"]).max() <= 1e-12 * np.abs(g["stress_new"]).max()
    assert np.abs(st - g["state_new"]).max() <= 1e-12 * max(np.abs(g["state_new"]).max(), 1e-12)
    assert np.abs(D - g["ddsdde"]).max() <= 1e-12 * np.abs(g["ddsdde"]).max()
    assert (st[:, 0] > g["state"][:, 0]).any()  # some points yield


def test_shell_roof(golden):
    """Tria1 flat-facet shell: element matrices against the reference's k0(),
    assembly bit-exact given them, and the linear solution, forces and
    station stresses of the cylindrical-roof fixture."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spla

    g = golden("shell_roof_9x7.npz")
    nodes, el, E, h = g["nodes"], g["elements"], g["E"], g["t"]
    nu = 0.3
    Cv = O.plane_stress_voigt(E, nu)
    Gs = np.stack([E / (2 * (1 + nu))] * 2, axis=1)
    ke = O.shell_stiffness(nodes, el, Cv, Gs, h)
    assert np.abs(ke - g["ke"]).max() <= 1e-13 * np.abs(g["ke"]).max()
    glob_idx, k_map, diag_map, _ = O.pattern(el, len(nodes), 6)
    assert np.array_equal(glob_idx, g["glob_idx"]) and np.array_equal(k_map, g["k_map"])
    n_dofs = 6 * len(nodes)
    y0, y1 = nodes[:, 1] == 0.0, nodes[:, 1] == 2.0
    con = np.zeros((len(nodes), 6), dtype=bool)
    con[y0, :] = True
    con[y1, :3] = True
    DU = np.zeros((len(nodes), 6))
    DU[y1, 1] = 1e-3
    F = np.zeros((len(nodes), 6))
    F[:, 2] = -1.0 / len(nodes)
    F[np.abs(nodes[:, 0] - nodes[:, 0].min()) < 1e-12, 3] = 2e-3
    cidx = np.nonzero(con.ravel())[0]
    val = O.assemble_matrix(g["ke"], k_map, glob_idx.shape[1], glob_idx, diag_map, cidx)
    K = sp.csr_matrix((val, (glob_idx[0], glob_idx[1])), shape=(n_dofs, n_dofs))
    assert np.array_equal(K.toarray(), g["K"])
    valf = np.zeros(glob_idx.shape[1])
    np.add.at(valf, k_map, ke.ravel())
    Kf = sp.csr_matrix((valf, (glob_idx[0], glob_idx[1])), shape=(n_dofs, n_dofs))
    Kc = sp.csr_matrix((O.assemble_matrix(ke, k_map, glob_idx.shape[1], glob_idx, diag_map, cidx),
                        (glob_idx[0], glob_idx[1])), shape=(n_dofs, n_dofs))
    u = np.zeros(n_dofs)
    u[cidx] = DU.ravel()[cidx]
    res = Kf @ u - F.ravel()
    res[cidx] = 0.0
    u = u - spla.spsolve(Kc.tocsc(), res)
    u[cidx] = DU.ravel()[cidx]
    rel = lambda a, b: np.abs(a - b).max() / np.abs(b).max()  # noqa: E731
    assert rel(u.reshape(-1, 6), g["u"]) <= 1e-10
    assert rel((Kf @ u).reshape(-1, 6), g["f"]) <= 1e-10
    s = O.shell_station_stress(nodes, el, Cv, h, u.reshape(-1, 6))
    assert rel(s, g["sigma_ip"]) <= 1e-10
    assert rel(s.mean(0), g["sigma"]) <= 1e-10


def test_hexa2(golden):
    """Hexa2 (20-node serendipity): pattern, element matrices against the
    reference's k0() and the linear solution of a jittered cube."""
    g = golden("hexa2_jitter2.npz")
    nodes, el = g["nodes"], g["elements"]
    m = O.LinearModel(nodes, el, O.elastic_c("3d", 1000.0, 0.3, len(el)))
    assert np.array_equal(m.glob_idx, g["glob_idx"]) and np.array_equal(m.k_map, g["k_map"])
    k = m.stiffness()
    assert np.abs(k - g["ke"]).max() <= 1e-13 * np.abs(g["ke"]).max()
    con = np.zeros(nodes.shape, dtype=bool)
    con[nodes[:, 0] == 0.0, :] = True
    F = np.zeros(nodes.shape)
    F[nodes[:, 0] == 1.0, 2] = -1.0 / len(nodes)
    u, f, s = m.solve(F, con)
    rel = lambda a, b: np.abs(a - b).max() / np.abs(b).max()  # noqa: E731
    assert rel(u, g["u"]) <= 1e-10 and rel(f, g["f"]) <= 1e-10 and rel(s, g["sigma"]) <= 1e-10


# ------------------------------------------------------ multigrid oracle ---
def _amg_cube(n=8, seed=0):
    nodes, el = O.cube_hexa(n + 1, n + 1, n + 1)
    rng = np.random.default_rng(seed)
    inner = np.all((nodes > 0) & (nodes < 1), axis=1)
    nodes = nodes.copy()
    nodes[inner] += rng.uniform(-0.1 / n, 0.1 / n, size=(inner.sum(), 3))
    model = O.LinearModel(nodes, el, O.elastic_c("3d", 1000.0, 0.3, len(el)))
    con = np.zeros((len(nodes), 3), bool)
    con[nodes[:, 0] == 0.0] = True
    con[nodes[:, 0] == 1.0, 0] = True
    K = model.matrix(np.nonzero(con.ravel())[0]).tocsr()
    return nodes, K, con


def test_amg_oracle_aggregation_invariants():
    from oracle import amg_oracle as AO

    nodes, K, con = _amg_cube()
    ptr, idx, _ = AO.block_pattern(K, 3)
    n = len(nodes)
    active = ~np.all(con, axis=1)
    agg, na = AO.aggregate(ptr, idx, active)
    assert np.all(agg[active] >= 0) and np.all(agg[~active] == -1)
    assert set(np.unique(agg[active])) == set(range(na))
    adj = [set(idx[ptr[i]:ptr[i + 1]]) for i in range(n)]
    for a in range(na):  # every aggregate is connected in the node graph
        mem = set(np.nonzero(agg == a)[0])
        seen, todo = set(), [min(mem)]
        while todo:
            v = todo.pop()
            if v in seen:
                continue
            seen.add(v)
            todo.extend((adj[v] & mem) - seen)
        assert seen == mem


def test_amg_oracle_tentative_reproduces_rigid_modes():
    from oracle import amg_oracle as AO

    nodes, K, con = _amg_cube()
    ptr, idx, _ = AO.block_pattern(K, 3)
    active = ~np.all(con, axis=1)
    agg, na = AO.aggregate(ptr, idx, active)
    T, Bc = AO.tentative(agg, na, 3, 6, coords=nodes, con=con.ravel())
    Ts = AO.to_sparse_T(T, agg, 6)
    assert np.abs((Ts.T @ Ts).toarray() - np.eye(6 * na)).max() <= 1e-12
    # on each aggregate, T Bc reproduces the rigid-body rows about the global centroid
    B = AO.null_rows(nodes, con.ravel(), 3, 6, nodes.mean(axis=0)).reshape(-1, 6)
    rows = np.repeat(agg, 3)
    got = np.zeros_like(B)
    for a in range(na):
        sel = rows == a
        got[sel] = Ts[sel][:, 6 * a:6 * a + 6] @ Bc[a]
    assert np.abs(got - B).max() <= 1e-10 * np.abs(B).max()


def test_amg_oracle_vcycle_symmetric_and_converges():
    from oracle import amg_oracle as AO

    nodes, K, con = _amg_cube()
    levels = AO.hierarchy(K, nodes, con.ravel(), 3)
    rng = np.random.default_rng(1)
    u, v = rng.standard_normal(K.shape[0]), rng.standard_normal(K.shape[0])
    a, b = u @ AO.vcycle(levels, v), v @ AO.vcycle(levels, u)
    assert abs(a - b) <= 1e-10 * abs(a)
    rhs = rng.standard_normal(K.shape[0])
    x, it = AO.pcg(K, rhs, levels, rtol=1e-10)
    assert np.linalg.norm(rhs - K @ x) <= 1e-10 * np.linalg.norm(rhs)
    assert it <= 25


# ------------------------------------------------------------ heat conduction --
def _heat_rel(a, b):
    return float(np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300))


def test_heat_oracle_steady(golden):
    """Conductivity matrices, temperatures, heat fluxes and compliance
    gradients of the heat oracle against the reference (heat_cases.npz)."""
    from oracle import heat_oracle as H

    g = golden("heat_cases.npz")
    m = H.HeatModel(g["solid_nodes"], g["solid_elements"], g["solid_kappa"][:, None, None] * np.eye(3))
    assert _heat_rel(m.conductivity(), g["solid_k0"]) < 1e-13
    T, f, flux, gr = m.solve(g["solid_q"], g["solid_con"], g["solid_temp"])
    for a, b in ((T, g["solid_T"]), (f, g["solid_f"]), (flux.mean(0), g["solid_flux"]), (gr.mean(0), g["solid_grad"])):
        assert _heat_rel(a, b.reshape(a.shape)) < 1e-11
    gk, _, gq = m.compliance_grads(T, f)
    assert _heat_rel(np.einsum("Eaa->E", gk), g["solid_g_kappa"]) < 1e-9
    assert _heat_rel(gq, g["solid_g_q"].ravel()) < 1e-11

    rho = g["planar_rho"]
    m = H.HeatModel(g["planar_nodes"], g["planar_elements"], 400.0 * np.eye(2), thickness=rho**3)
    T, f, flux, _ = m.solve(g["planar_q"], g["planar_con"])
    assert _heat_rel(T, g["planar_T"].ravel()) < 1e-12
    assert _heat_rel(flux.mean(0), g["planar_flux"]) < 1e-12
    _, gt, _ = m.compliance_grads(T, f)
    assert _heat_rel(gt * 3 * rho**2, g["planar_g_rho"]) < 1e-11

    m = H.HeatModel(g["planar_nodes"], g["planar_elements"], g["ortho_kappa"], thickness=0.1)
    assert _heat_rel(m.conductivity(), g["ortho_k0"]) < 1e-13
    T, f, flux, gr = m.solve(np.zeros(m.n_nod), g["ortho_con"], g["ortho_temp"])
    assert _heat_rel(T, g["ortho_T"].ravel()) < 1e-12
    assert _heat_rel(f, g["ortho_f"].ravel()) < 1e-12


def test_heat_oracle_transient(golden):
    """Capacity matrices and Crank-Nicolson time integration of the heat
    oracle against the reference's heated plate."""
    from oracle import heat_oracle as H

    g = golden("heat_cases.npz")
    nodes, el = O.rect_quad(5, 5, 1.0, 1.0)
    m = H.HeatModel(nodes, el, 400.0 * np.eye(2), rho=1e5)
    assert _heat_rel(m.capacity(), g["plate_mass"]) < 1e-13
    w, e = np.isclose(nodes[:, 0], 0.0), np.isclose(nodes[:, 0], 1.0)
    temp = np.where(w, 5.0, np.where(e, 20.0, 0.0))
    T, f, flux, gr = H.time_integration(m, w | e, temp, np.zeros(len(nodes)), g["plate_t"], 1.0)
    assert _heat_rel(T, g["plate_temp"][..., 0]) < 1e-12
    assert _heat_rel(f, g["plate_f"][..., 0]) < 1e-12
    assert _heat_rel(flux.mean(1), g["plate_flux"]) < 1e-12
    times, rows = H.time_grid(g["late_t"], 0.5)
    assert times[0] == 0.0 and list(rows) == [5, 10]
    T, f, flux, gr = H.time_integration(m, w | e, temp, np.zeros(len(nodes)), g["late_t"], 0.5)
    assert _heat_rel(T, g["late_temp"][..., 0]) < 1e-12
    assert _heat_rel(flux, g["late_flux"]) < 1e-12


def test_heat_oracle_transient_adjoint(golden):
    """The discrete adjoint of the Crank-Nicolson steps against the
    reference's autograd through time_integration (unequal steps, per-element
    conductivity and density, nodal sources)."""
    from oracle import heat_oracle as H

    g = golden("heat_transient_grad.npz")
    m = H.HeatModel(g["nodes"], g["elements"], g["kappa"][:, None, None] * np.eye(2), rho=g["rho"])
    L, gk, gr, gq = H.time_integration_adjoint(m, g["con"], g["temp_bc"], g["q"], g["t_out"], float(g["delta_t"]),
                                               g["c"])
    assert abs(L - float(g["L"])) <= 1e-13 * abs(float(g["L"]))
    assert _heat_rel(np.einsum("Eaa->E", gk), g["g_kappa"]) < 1e-12
    assert _heat_rel(gr, g["g_rho"]) < 1e-12
    assert _heat_rel(gq, g["g_q"].ravel()) < 1e-12


def test_modal_oracle(golden):
    """FEM.solve_modes: the lowest squared angular frequencies, mode shapes
    (up to sign) and d(sum omega^2)/d(E, rho) against the reference."""
    from oracle import modal_oracle as MO

    g = golden("modes_hexa_jitter3.npz")
    lam, modes, gE, gr = MO.solve_modes(g["nodes"], g["elements"], g["E"], 0.3, g["rho"], g["con"], 6)
    assert _heat_rel(lam, g["omega_sq"]) < 1e-12
    sign = np.sign(np.einsum("mnd,mnd->m", modes, g["modes"]))
    assert _heat_rel(modes * sign[:, None, None], g["modes"]) < 1e-10
    assert _heat_rel(gE, g["g_E"]) < 1e-12
    assert _heat_rel(gr, g["g_rho"]) < 1e-12


def test_assembly_oracle(golden):
    """The assembly oracle (oracle/assembly_oracle.py) against the reference's
    own coupled solves: a cube turned by a 3D reference point, a Quad1 plate
    turned by a 2D point, a conducting cube held by a thermal point."""
    from oracle import assembly_oracle as A
    from oracle import heat_oracle as H

    g = golden("assembly_cases.npz")

    def rel(a, b):
        return float(np.abs(np.asarray(a) - b).max() / max(np.abs(b).max(), 1e-300))

    nodes, el = O.cube_hexa(3, 3, 3)
    solid = A.ModelPart(O.LinearModel(nodes, el, O.elastic_c("3d", 1000.0, 0.3, len(el))), 3)
    solid.constraints[nodes[:, 2] == 0.0] = True
    point = A.PointPart([0.5, 0.5, 2.0])
    point.forces[0, 3] = 50.0
    point.forces[0, 1] = 7.0
    asm = A.AssemblyOracle([solid, point])
    asm.coupling(0, nodes[:, 2] == nodes[:, 2].max(), 1)
    u, f = asm.solve()
    assert rel(u[0], g["rp_u0"]) < 1e-10 and rel(u[1], g["rp_u1"]) < 1e-10
    assert rel(f[0], g["rp_f0"]) < 1e-10 and rel(f[1], g["rp_f1"]) < 1e-10

    nodes, el = O.rect_quad(5, 5)
    plate = A.ModelPart(O.LinearModel(nodes, el, O.elastic_c("plane_stress", 1000.0, 0.3, len(el))), 2)
    plate.constraints[nodes[:, 1] == 0.0] = True
    p2 = A.PointPart([0.5, 1.5])
    p2.forces[0, 2] = 20.0
    p2.forces[0, 0] = 3.0
    asm = A.AssemblyOracle([plate, p2])
    asm.coupling(0, nodes[:, 1] == 1.0, 1)
    u, f = asm.solve(method="cg")
    assert rel(u[0], g["planar_u0"]) < 1e-9 and rel(u[1], g["planar_u1"]) < 1e-9
    assert rel(f[1], g["planar_f1"]) < 1e-9

    nodes, el = O.cube_hexa(4, 4, 4)
    heat = A.ModelPart(H.HeatModel(nodes, el, np.eye(3)), 1)
    heat.constraints[nodes[:, 2] == 0.0] = True
    heat.forces[nodes[:, 0] == 0.0, 0] = 0.1
    hp = A.PointPart([0.5, 0.5, 1.5], heat=True)
    hp.forces[0, 0] = 4.0
    asm = A.AssemblyOracle([heat, hp])
    asm.coupling(0, nodes[:, 2] == 1.0, 1)
    T, q = asm.solve()
    assert rel(T[0], g["heat_T0"]) < 1e-10 and rel(T[1], g["heat_T1"]) < 1e-10
    assert rel(q[0], g["heat_q0"]) < 1e-10 and rel(q[1], g["heat_q1"]) < 1e-10
