"""Host side of Assembly (no GPU): the reference's construction and coupling
checks with their messages (tests/test_assembly.py of torch-fem), the
elimination map u = T q, and the symbolic phase of K_r = T^T K T (pattern,
contribution lists, condensation flags) against a scipy product of the same
matrices with random values.
"""

import numpy as np
import pytest
import scipy.sparse as sp
import torch

from torchfem_gb300 import Assembly, Planar, ReferencePoint, Shell, Solid, SolidHeat, mesh
from torchfem_gb300.assembly import _csr, coupled_pattern
from torchfem_gb300.materials import (IsotropicConductivity3D, IsotropicElasticity3D,
                                      IsotropicElasticityPlaneStrain, IsotropicElasticityPlaneStress)

SOLID = IsotropicElasticity3D(1000.0, 0.3)
PLANE = IsotropicElasticityPlaneStress(1000.0, 0.3)


def _block(z0, z1):
    nodes = torch.tensor([[x, y, z] for z in (z0, z1) for y in (0.0, 1.0) for x in (0.0, 1.0)],
                         dtype=torch.float64)
    return nodes, torch.tensor([[0, 1, 3, 2, 4, 5, 7, 6]])


def _two_blocks():
    n_a, e_a = _block(0.0, 1.0)
    n_b, e_b = _block(1.0, 2.0)
    return Solid(n_a, e_a, SOLID), Solid(n_b, e_b, SOLID), n_a, n_b


def test_a_part_cannot_appear_twice():
    a, _, _, _ = _two_blocks()
    with pytest.raises(ValueError, match="only once"):
        Assembly([a, a])


def test_one_physics_and_one_dimension():
    nodes, elements = mesh.cube_hexa(2, 2, 2)
    solid = Solid(nodes, elements, SOLID)
    heat = SolidHeat(nodes, elements, IsotropicConductivity3D(1.0))
    with pytest.raises(ValueError, match="mechanical or thermal"):
        Assembly([solid, heat])
    with pytest.raises(ValueError, match="mechanical or thermal"):
        Assembly([heat, ReferencePoint([0.0, 0.0, 1.0])])
    planar = Planar(*mesh.rect_quad(3, 3), IsotropicElasticityPlaneStrain(1000.0, 0.3))
    with pytest.raises(ValueError, match="one spatial dimension"):
        Assembly([planar, solid])
    with pytest.raises(ValueError, match="one spatial dimension"):
        Assembly([planar, ReferencePoint([0.0, 0.0, 0.0])])


def test_coupling_checks():
    a, b, n_a, n_b = _two_blocks()
    with pytest.raises(ValueError, match="must belong to this assembly"):
        Assembly([a]).coupling(a, n_a[:, 2] == 1.0, b)
    asm = Assembly([a, b])
    with pytest.raises(ValueError, match=r"indices in \[0, 3\)"):
        asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0, dofs=[5])
    nodes, elements = mesh.strip_tria(5, 3, 10.0, 1.0)
    shell = Shell(nodes, elements, PLANE, thickness=0.4)
    asm = Assembly([a, shell])
    with pytest.raises(ValueError, match="primary part that has none"):
        asm.coupling(shell, nodes[:, 0] == 0.0, a, n_a[:, 2] == 1.0, dofs=[3])


def test_elimination_checks_run_before_the_gpu():
    a, b, n_a, n_b = _two_blocks()
    asm = Assembly([a, b])
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    with pytest.raises(ValueError, match="more than one constraint"):
        asm.solve()
    a, b, n_a, n_b = _two_blocks()
    point = ReferencePoint([0.5, 0.5, 1.0])
    asm = Assembly([a, b, point])
    asm.coupling(a, n_a[:, 2] == 1.0, point)
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    with pytest.raises(ValueError, match="both eliminated and used as a primary"):
        asm.solve()
    a, b, n_a, n_b = _two_blocks()
    b.constraints[n_b[:, 2] == 1.0] = True
    asm = Assembly([a, b])
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    with pytest.raises(ValueError, match="constrained DOF is eliminated"):
        asm.solve()


def test_reference_point_dofs():
    assert ReferencePoint([0.5, 1.5]).n_dofs == 3
    assert ReferencePoint([0.5, 1.5, 0.0]).n_dofs == 6


def test_elimination_map_reproduces_rigid_motion():
    """u = T q: coupled nodes follow the point's translation plus theta x r."""
    nodes, elements = mesh.cube_hexa(3, 3, 3)
    solid = Solid(nodes, elements, SOLID)
    point = ReferencePoint([0.5, 0.5, 2.0])
    asm = Assembly([solid, point])
    top = nodes[:, 2] == nodes[:, 2].max()
    asm.coupling(solid, top, point)
    rows, cols, vals, retained = asm._build_T()
    T = sp.csr_matrix((vals, (rows, cols)), shape=(asm.n_dofs, len(retained)))
    rng = np.random.default_rng(0)
    q = rng.standard_normal(len(retained))
    u = T @ q
    up = u[asm.offsets[1]:asm.offsets[1] + 6]
    us = u[: solid.n_dofs].reshape(-1, 3)[top.numpy()]
    r = (nodes[top] - point.nodes[0].to(torch.float64)).numpy()
    assert np.allclose(us, up[:3] + np.cross(np.broadcast_to(up[3:], r.shape), r), atol=1e-14)


@pytest.mark.parametrize("seed", [0, 1])
def test_coupled_pattern_matches_scipy(seed):
    """The symbolic phase plus a host evaluation of the contribution lists
    equals T^T K T with the condensation, for random part values."""
    rng = np.random.default_rng(seed)
    a, b, n_a, n_b = _two_blocks()
    point = ReferencePoint([0.5, 0.5, 3.0])
    asm = Assembly([a, b, point])
    asm.coupling(b, n_b[:, 2] == 1.0, a, n_a[:, 2] == 1.0)
    asm.coupling(b, n_b[:, 2] == 2.0, point, dofs=[0, 2])
    rows, cols, vals, retained = asm._build_T()
    n = len(retained)
    T = _csr(rows, cols, vals, asm.n_dofs)
    patterns, blocks = [], []
    for part, off in zip(asm.parts[:2], asm.offsets[:2]):
        nd = part.n_dofs
        M = sp.random(nd, nd, density=0.4, random_state=rng, format="csr")
        M = (M + M.T + sp.eye(nd)).tocsr()
        M.sort_indices()
        patterns.append((off, M.indptr.astype(np.int64), M.indices.astype(np.int64)))
        blocks.append(M)
    con = np.zeros(n, dtype=bool)
    con[rng.choice(n, 4, replace=False)] = True
    rptr, ccol, cptr, src, coef, fix, diag_map = coupled_pattern(T, patterns, n, con)
    kval = np.concatenate([M.data for M in blocks])
    out = np.array([np.dot(coef[cptr[e]:cptr[e + 1]], kval[src[cptr[e]:cptr[e + 1]]]) for e in range(len(ccol))])
    out[fix == 1] = 0.0
    out[fix == 2] = 1.0
    got = sp.csr_matrix((out, ccol, rptr), shape=(n, n)).toarray()
    Kb = sp.block_diag(blocks + [sp.csr_matrix((point.n_dofs, point.n_dofs))]).tocsr()
    Tm = sp.csr_matrix((vals, (rows, cols)), shape=(asm.n_dofs, n))
    ref = (Tm.T @ Kb @ Tm).toarray()
    ref[con, :] = 0.0
    ref[:, con] = 0.0
    ref[con, con] = 1.0
    assert np.allclose(got, ref, rtol=1e-14, atol=1e-14)
    # an explicit diagonal for every retained DOF
    assert len(diag_map) == n and np.all(ccol[diag_map] == np.arange(n))
    # columns ascend within each row, and each entry's contributions are in
    # source order (the fixed summation order of the GPU values)
    assert all(np.all(np.diff(ccol[rptr[i]:rptr[i + 1]]) > 0) for i in range(n))
    assert all(np.all(np.diff(src[cptr[e]:cptr[e + 1]]) >= 0) for e in range(len(ccol)))


def test_csr_sums_duplicates_and_keeps_empty_rows():
    rows = np.array([2, 0, 2, 2], dtype=np.int64)
    cols = np.array([1, 3, 1, 0], dtype=np.int64)
    vals = np.array([1.0, 2.0, 3.0, 4.0])
    ptr_, col, val = _csr(rows, cols, vals, 4)
    assert ptr_.tolist() == [0, 1, 1, 3, 3]
    assert col.tolist() == [3, 0, 1]
    assert val.tolist() == [2.0, 4.0, 4.0]


def test_coupled_pattern_of_an_uncoupled_point_has_only_its_diagonal():
    """A reference point that no coupling touches keeps an explicit (zero)
    diagonal row, as Assembly._stiffness adds one for every retained DOF."""
    a, _, n_a, _ = _two_blocks()
    point = ReferencePoint([0.5, 0.5, 3.0])
    asm = Assembly([a, point])
    rows, cols, vals, retained = asm._build_T()
    n = len(retained)
    T = _csr(rows, cols, vals, asm.n_dofs)
    M = sp.eye(a.n_dofs, format="csr") * 2.0
    M.sort_indices()
    patterns = [(0, M.indptr.astype(np.int64), M.indices.astype(np.int64))]
    rptr, ccol, cptr, src, coef, fix, diag_map = coupled_pattern(T, patterns, n, np.zeros(n, dtype=bool))
    for i in range(a.n_dofs, n):
        assert rptr[i + 1] - rptr[i] == 1 and ccol[rptr[i]] == i
        e = rptr[i]
        assert np.all(coef[cptr[e]:cptr[e + 1]] == 0.0)
