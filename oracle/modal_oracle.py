"""CPU oracle of torch-fem's modal analysis — TEST INFRASTRUCTURE ONLY.

numpy/scipy restatement of `FEM.solve_modes` (src/torchfem/base.py:1097-1129),
used by `tests/` only.  It covers:
  - the generalized eigenproblem K phi = omega^2 M phi on the free DOFs
    (sparse.py:798-827, which solves the free-DOF block by shift-invert);
  - the eigenvalue sensitivities of sparse.py:930-983:
    d(omega^2)/dK_ij = phi_i phi_j and d(omega^2)/dM_ij = -omega^2 phi_i phi_j,
    with phi normalised so that phi^T M phi = 1.

Parity pin: tests/test_oracle.py checks it against
tests/golden/modes_hexa_jitter3.npz, written by running the reference itself
(tests/golden/make_golden.py, `make_modes`).
"""

from __future__ import annotations

import numpy as np
import scipy.linalg as sla

from .fem_oracle import LinearModel, elastic_c
from .heat_oracle import shape_values


def element_mass(model: LinearModel, rho) -> np.ndarray:
    """m_e = sum_ip w detJ rho N N^T expanded to the DOFs (kron with I_d),
    [n_elem, n_e d, n_e d] (base.py:376-396, solid.py:60-62)."""
    N = shape_values(model.etype)
    rho = np.broadcast_to(np.asarray(rho, float), (model.n_elem,))
    m = np.einsum("iE,iN,iM->ENM", model.w[:, None] * model.detJ * rho[None], N, N)
    d = model.d
    return np.einsum("ENM,ij->ENiMj", m, np.eye(d)).reshape(model.n_elem, model.n_e * d, model.n_e * d)


def solve_modes(nodes, elements, E, nu, rho, constraints, n_modes):
    """(omega^2 [n_modes], modes [n_modes, n_nod, d], d(sum omega^2)/dE [n_elem],
    d(sum omega^2)/drho [n_elem]) for IsotropicElasticity3D with per-element E
    and rho."""
    nodes = np.asarray(nodes, float)
    n_elem = len(elements)
    E = np.broadcast_to(np.asarray(E, float), (n_elem,))
    model = LinearModel(nodes, elements, elastic_c("3d", E, nu, n_elem))
    k = model.stiffness()
    m = element_mass(model, rho)
    none = np.array([], dtype=np.int64)
    K = model.matrix(none, k).toarray()
    M = model.matrix(none, m).toarray()
    free = ~np.asarray(constraints).ravel().astype(bool)
    lam, vec = sla.eigh(K[np.ix_(free, free)], M[np.ix_(free, free)], subset_by_index=[0, n_modes - 1])
    phi = np.zeros((model.n_dofs, n_modes))
    phi[free] = vec  # eigh normalises to phi^T M phi = 1
    idx = model.elements[:, :, None] * model.d + np.arange(model.d)
    pe = phi[idx.reshape(n_elem, -1)]  # [E, n_e d, n_modes]
    # K and M are linear in E_e and rho_e for fixed nu
    g_E = np.einsum("Eam,Eab,Ebm->E", pe, k, pe) / E
    g_rho = -np.einsum("Eam,Eab,Ebm,m->E", pe, m, pe, lam) / np.broadcast_to(np.asarray(rho, float), (n_elem,))
    modes = phi.T.reshape(n_modes, model.n_nod, model.d)
    return lam, modes, g_E, g_rho
