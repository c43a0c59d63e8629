"""CPU oracle of torch-fem's forward + adjoint path — TEST INFRASTRUCTURE ONLY.

This module restates, in numpy/scipy, the arithmetic of the reference's hot
path so that the GPU library can be checked against it.  Only `tests/`,
`__graft_entry__.smoke()` and the `cpu_baseline` leg of `bench.py` may import
it; the product (`torch-fem_gb300/`) never does.

Parity pin: every function here is checked against golden vectors generated
by running the reference itself (tests/golden/make_golden.py, committed with
its outputs) — pattern, k_map, element matrices, assembled values, solutions
and adjoint gradients.

Restated reference code (paths relative to the torch-fem repository):
  pattern              src/torchfem/base.py:72-122
  shape gradients      src/torchfem/base.py:293-314, elements.py (tables)
  integrate_material   src/torchfem/base.py:982-1092 (+ solid.py:52-58,
                       planar.py:86-92, materials/elasticity.py:44-241)
  assemble_matrix      src/torchfem/base.py:398-426 (serial index_add_ order)
  assemble_rhs         src/torchfem/base.py:428-445
  solve (linear)       src/torchfem/base.py:597-923 with sparse.py:271-514
  adjoint              src/torchfem/sparse.py:641-724
  Neo-Hookean point    materials/hyperelasticity.py:117-123 with the energy of
                       benchmarks/hyperelasticity.py:24-30
  J2 plane strain      materials/plasticity.py:504-590
  Tria1 flat shell     src/torchfem/shell.py:48-177 (section), :263-356
                       (strain operators), :358-387 (frames), :416-603
                       (stiffness, forces, station stresses)
"""

from __future__ import annotations

from math import sqrt
import time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

# --------------------------------------------------------------- elements ---
_HEX_SIGNS = np.array(
    [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)],
    dtype=np.float64,
)
_QUAD_SIGNS = np.array([(-1, -1), (1, -1), (1, 1), (-1, 1)], dtype=np.float64)


def _hexa1_dn(xi):
    x = xi[:, None, :]  # [nip, 1, 3]
    s = _HEX_SIGNS[None]  # [1, 8, 3]
    f = 1.0 + s * x  # [nip, 8, 3]
    d0 = s[..., 0] * f[..., 1] * f[..., 2]
    d1 = s[..., 1] * f[..., 0] * f[..., 2]
    d2 = s[..., 2] * f[..., 0] * f[..., 1]
    return 0.125 * np.stack([d0, d1, d2], axis=1)  # [nip, 3, 8]


def _quad1_dn(xi):
    x = xi[:, None, :]
    s = _QUAD_SIGNS[None]
    f = 1.0 + s * x
    return 0.25 * np.stack([s[..., 0] * f[..., 1], s[..., 1] * f[..., 0]], axis=1)  # [nip, 2, 4]


def _tetra2_dn(xi):
    x, y, z = xi[:, 0], xi[:, 1], xi[:, 2]
    o = np.zeros_like(x)
    c = 4 * (x + y + z) - 3
    dx = [c, 4 * x - 1, o, o, -4 * (2 * x + y + z - 1), 4 * y, -4 * y, -4 * z, 4 * z, o]
    dy = [c, o, 4 * y - 1, o, -4 * x, 4 * x, -4 * (x + 2 * y + z - 1), -4 * z, o, 4 * z]
    dz = [c, o, o, 4 * z - 1, -4 * x, o, -4 * y, -4 * (x + y + 2 * z - 1), 4 * x, 4 * y]
    return np.stack([np.stack(dx, -1), np.stack(dy, -1), np.stack(dz, -1)], axis=1)


def _tetra1_dn(xi):
    b = np.array([[-1.0, 1.0, 0.0, 0.0], [-1.0, 0.0, 1.0, 0.0], [-1.0, 0.0, 0.0, 1.0]])
    return np.broadcast_to(b, (xi.shape[0], 3, 4)).copy()


def _tria1_dn(xi):
    b = np.array([[-1.0, 1.0, 0.0], [-1.0, 0.0, 1.0]])
    return np.broadcast_to(b, (xi.shape[0], 2, 3)).copy()


_HEX2_COORDS = np.concatenate([_HEX_SIGNS, np.array(
    [(0, -1, -1), (1, 0, -1), (0, 1, -1), (-1, 0, -1), (0, -1, 1), (1, 0, 1), (0, 1, 1), (-1, 0, 1),
     (-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0)], dtype=np.float64)])


def _hexa2_dn(xi):
    """Serendipity 20-node gradients: corners (1+s.x) products times
    (s.x_sum - 2), mid-edge nodes (1 - t^2) times the two edge-normal factors."""
    out = np.zeros((xi.shape[0], 3, 20))
    for a, s in enumerate(_HEX2_COORDS):
        for k in range(3):  # derivative direction
            val = np.ones(xi.shape[0])
            if np.all(s != 0):
                f = 1.0 + s * xi  # [nip, 3]
                g = (s * xi).sum(1) - 2.0
                others = np.prod(np.delete(f, k, axis=1), axis=1)
                val = 0.125 * s[k] * others * (g + f[:, k])
            else:
                m = int(np.nonzero(s == 0)[0][0])  # coordinate along the edge
                fac = [(1.0 - xi[:, j] ** 2) if j == m else (1.0 + s[j] * xi[:, j]) for j in range(3)]
                dfac = [(-2.0 * xi[:, j]) if j == m else np.full(xi.shape[0], s[j]) for j in range(3)]
                val = 0.25 * np.prod([dfac[j] if j == k else fac[j] for j in range(3)], axis=0)
            out[:, k, a] = val
    return out


_S3 = 1.0 / sqrt(3.0)
ELEMENTS = {
    # name: (nodes, dim, ipoints, weights, dN/dxi)
    "Hexa1": (8, 3, np.array([[a * _S3, b * _S3, c * _S3] for c in (-1.0, 1.0) for b in (-1.0, 1.0) for a in (-1.0, 1.0)]),
              np.ones(8), _hexa1_dn),
    "Quad1": (4, 2, np.array([[a * _S3, b * _S3] for b in (-1, 1) for a in (-1, 1)]), np.ones(4), _quad1_dn),
    "Tetra2": (10, 3, np.array([[0.58541020, 0.13819660, 0.13819660], [0.13819660, 0.58541020, 0.13819660],
                                [0.13819660, 0.13819660, 0.58541020], [0.13819660, 0.13819660, 0.13819660]]),
               np.full(4, 0.041666667), _tetra2_dn),
    "Tetra1": (4, 3, np.array([[0.25, 0.25, 0.25]]), np.array([1.0 / 6.0]), _tetra1_dn),
    "Tria1": (3, 2, np.array([[1.0 / 3.0, 1.0 / 3.0]]), np.array([0.5]), _tria1_dn),
    "Hexa2": (20, 3, np.array([[a * _S3, b * _S3, c * _S3] for c in (-1.0, 1.0) for b in (-1.0, 1.0) for a in (-1.0, 1.0)]),
              np.ones(8), _hexa2_dn),
}


def element_name(n_e: int, dim: int) -> str:
    table = {(8, 3): "Hexa1", (10, 3): "Tetra2", (4, 3): "Tetra1", (4, 2): "Quad1", (3, 2): "Tria1",
             (20, 3): "Hexa2"}
    return table[(n_e, dim)]


# ---------------------------------------------------------------- pattern ---
def pattern(elements: np.ndarray, n_nod: int, d: int):
    """glob_idx [2, nnz], k_map [n_elem (n_e d)^2], diag_map [n_dofs] of the
    reference's precompute (base.py:72-122): unique packed (row << 32 | col)
    keys of all element entries plus the diagonal, then searchsorted."""
    elements = np.asarray(elements, dtype=np.int64)
    n_elem = elements.shape[0]
    idx = (d * elements[..., None] + np.arange(d)).reshape(n_elem, -1)
    keys = ((idx[:, :, None] << 32) | idx[:, None, :]).reshape(-1)
    diag = np.arange(n_nod * d, dtype=np.int64)
    packed = np.unique(np.concatenate([keys, (diag << 32) | diag]))
    k_map = np.searchsorted(packed, keys)
    diag_map = np.searchsorted(packed, (diag << 32) | diag)
    glob_idx = np.stack([packed >> 32, packed & 0xFFFFFFFF])
    return glob_idx, k_map, diag_map, idx


# ----------------------------------------------------------- integration ---
def shape_gradients(nodes: np.ndarray, elements: np.ndarray, etype: str):
    """B [nip, n_elem, dim, n_e] (dN/dx) and detJ [nip, n_elem] (base.py:306-313)."""
    n_e, dim, ip, w, dn = ELEMENTS[etype]
    b = dn(ip)  # [nip, dim, n_e]
    X = nodes[elements]  # [n_elem, n_e, dim]
    J = np.einsum("iaN,ANj->iAaj", b, X)
    detJ = np.linalg.det(J)
    if np.any(detJ <= 0.0):
        raise ValueError("Negative Jacobian. Check element numbering.")
    B = np.einsum("iAaj,ijN->iAaN", np.linalg.inv(J), b)
    return B, detJ, w


def iso_c(lam: np.ndarray, G: np.ndarray, d: int) -> np.ndarray:
    """C = lam I(x)I + G (I4 + I4^T) per element (elasticity.py:58-70)."""
    I = np.eye(d)
    i4 = np.einsum("ij,kl->ijkl", I, I)
    i4s = np.einsum("ik,jl->ijkl", I, I) + np.einsum("il,jk->ijkl", I, I)
    return lam[:, None, None, None, None] * i4 + G[:, None, None, None, None] * i4s


def elastic_c(kind: str, E, nu, n_elem: int) -> np.ndarray:
    """Tangent of IsotropicElasticity3D / PlaneStress / PlaneStrain (elasticity.py:44-241)."""
    E = np.broadcast_to(np.asarray(E, dtype=np.float64), (n_elem,))
    nu = np.broadcast_to(np.asarray(nu, dtype=np.float64), (n_elem,))
    lbd = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    G = E / (2.0 * (1.0 + nu))
    if kind == "3d":
        return iso_c(lbd, G, 3)
    C = np.zeros((n_elem, 2, 2, 2, 2))
    if kind == "plane_stress":
        fac = E / (1.0 - nu**2)
        a, b, s = fac, fac * nu, fac * 0.5 * (1.0 - nu)
    elif kind == "plane_strain":
        a, b, s = 2.0 * G + lbd, lbd, G
    else:
        raise ValueError(kind)
    C[:, 0, 0, 0, 0] = a
    C[:, 1, 1, 1, 1] = a
    C[:, 0, 0, 1, 1] = b
    C[:, 1, 1, 0, 0] = b
    for i, j, k, l in ((0, 1, 0, 1), (0, 1, 1, 0), (1, 0, 0, 1), (1, 0, 1, 0)):
        C[:, i, j, k, l] = s
    return C


def integrate(B, detJ, w, C, du_e, sigma_prev=None, de0=None, thickness=None, need_k=True):
    """Linear-elastic integrate_material (base.py:1020-1092): element forces,
    stiffness, stress and increment gradient.  du_e [n_elem, n_e, d]."""
    nip, n_elem, d, n_e = B.shape
    t = np.ones(n_elem) if thickness is None else thickness
    du = du_e.transpose(0, 2, 1)  # [n_elem, d, n_e]
    f = np.zeros((n_elem, n_e * d))
    k = np.zeros((n_elem, n_e * d, n_e * d)) if need_k else None
    sig = np.zeros((nip, n_elem, d, d))
    H_all = np.zeros((nip, n_elem, d, d))
    e0 = np.zeros((n_elem, d, d)) if de0 is None else de0
    for i in range(nip):
        H = du @ B[i].transpose(0, 2, 1)
        de = 0.5 * (H.transpose(0, 2, 1) + H)
        s = np.einsum("eijkl,ekl->eij", C, de - e0)
        if sigma_prev is not None:
            s = s + sigma_prev[i]
        sig[i] = s
        H_all[i] = H
        fc = np.einsum("e,eiI,eAi->eIA", t * detJ[i], B[i], s)
        f += w[i] * fc.reshape(n_elem, -1)
        if need_k:
            BCB = np.einsum("eJp,eiJkL,eLq->epiqk", B[i], C, B[i]).reshape(n_elem, n_e * d, n_e * d)
            k += (t * detJ[i])[:, None, None] * BCB * w[i]
    return f, k, sig, H_all


def assemble_matrix(k, k_map, nnz, glob_idx, diag_map, con):
    """Serial ascending-order sums (CPU index_add_ order), then condensation."""
    val = np.zeros(nnz)
    np.add.at(val, k_map, k.ravel())
    is_con = np.zeros(diag_map.shape[0], dtype=bool)
    is_con[con] = True
    val[is_con[glob_idx[0]] | is_con[glob_idx[1]]] = 0.0
    val[diag_map[con]] = 1.0
    return val


def assemble_rhs(f, idx, n_dofs):
    F = np.zeros(n_dofs)
    np.add.at(F, idx.ravel(), f.ravel())
    return F


# ------------------------------------------------------------------ model ---
class LinearModel:
    """Linear-elastic model: the reference's single-increment solve
    (increments [0, 1]) and its adjoint, on the CPU."""

    def __init__(self, nodes, elements, C, thickness=None):
        self.nodes = np.asarray(nodes, dtype=np.float64)
        self.elements = np.asarray(elements, dtype=np.int64)
        self.n_nod, self.d = self.nodes.shape
        self.n_elem, self.n_e = self.elements.shape
        self.n_dofs = self.n_nod * self.d
        self.etype = element_name(self.n_e, self.d)
        self.C = np.asarray(C, dtype=np.float64)
        self.thickness = None if thickness is None else np.asarray(thickness, dtype=np.float64)
        self.glob_idx, self.k_map, self.diag_map, self.idx = pattern(self.elements, self.n_nod, self.d)
        self.B, self.detJ, self.w = shape_gradients(self.nodes, self.elements, self.etype)

    def stiffness(self):
        du0 = np.zeros((self.n_elem, self.n_e, self.d))
        _, k, _, _ = integrate(self.B, self.detJ, self.w, self.C, du0, thickness=self.thickness)
        return k

    def matrix(self, con, k=None):
        k = self.stiffness() if k is None else k
        val = assemble_matrix(k, self.k_map, self.glob_idx.shape[1], self.glob_idx, self.diag_map, con)
        return sp.csr_matrix((val, (self.glob_idx[0], self.glob_idx[1])), shape=(self.n_dofs, self.n_dofs))

    def forces_of(self, u):
        du_e = u.reshape(self.n_nod, self.d)[self.elements]
        f, _, sig, H = integrate(self.B, self.detJ, self.w, self.C, du_e, thickness=self.thickness, need_k=False)
        return assemble_rhs(f, self.idx, self.n_dofs), sig, H

    def solve(self, forces, constraints, displacements=None, method="spsolve", rtol=1e-12):
        """u, f, sigma (mean over points) of one linear increment (base.py:704-857)."""
        F_ext = np.asarray(forces, dtype=np.float64).ravel()
        con = np.nonzero(np.asarray(constraints).ravel())[0]
        DU = np.zeros(self.n_dofs) if displacements is None else np.asarray(displacements, dtype=np.float64).ravel()
        du = np.zeros(self.n_dofs)
        du[con] = DU[con]
        F_int, _, _ = self.forces_of(du)
        res = F_int - F_ext
        res[con] = 0.0
        K = self.matrix(con)
        du = du - self.linear_solve(K, res, method, rtol)
        du[con] = DU[con]
        F_int, sig, H = self.forces_of(du)
        self.K, self.con = K, con
        return du.reshape(self.n_nod, self.d), F_int.reshape(self.n_nod, self.d), sig.mean(axis=0)

    cg_iterations: list = []  # iterations of every Jacobi-CG solve (appended per solve)
    cg_seconds: list = []  # wall time of every Jacobi-CG solve

    @staticmethod
    def linear_solve(K, b, method="spsolve", rtol=1e-12):
        if method == "spsolve":
            return spla.spsolve(K.tocsc(), b)
        M = sp.diags(1.0 / K.diagonal())
        count = [0]

        def tick(_):
            count[0] += 1

        t0 = time.perf_counter()
        x, info = spla.cg(K, b, rtol=rtol, atol=0.0, M=M, maxiter=20 * K.shape[0], callback=tick)
        LinearModel.cg_seconds.append(time.perf_counter() - t0)
        LinearModel.cg_iterations.append(count[0])
        if info != 0:
            raise RuntimeError(f"CG failed with exit code {info}")
        return x

    def adjoint(self, g_u, method="spsolve", rtol=1e-12):
        """lambda = K^-1 g on free DOFs (sparse.py:671-680); 0 on constrained."""
        g = np.asarray(g_u, dtype=np.float64).ravel().copy()
        g[self.con] = 0.0
        return self.linear_solve(self.K, g, method, rtol)

    def grad_forces(self, g_u, method="spsolve"):
        """d(L)/d(forces) for a loss with dL/du = g_u: equals lambda."""
        return self.adjoint(g_u, method).reshape(self.n_nod, self.d)

    def compliance_grad_c(self, u):
        """dL/dC_e for L = f.u at equilibrium: -sum_ip w detJ t eps(u):dC:eps(u)
        expressed per entry of C_e: -sum_ip w detJ t eps_ij eps_kl."""
        du_e = u.reshape(self.n_nod, self.d)[self.elements].transpose(0, 2, 1)
        t = np.ones(self.n_elem) if self.thickness is None else self.thickness
        g = np.zeros_like(self.C)
        for i in range(self.B.shape[0]):
            H = du_e @ self.B[i].transpose(0, 2, 1)
            eps = 0.5 * (H + H.transpose(0, 2, 1))
            g -= (self.w[i] * self.detJ[i] * t)[:, None, None, None, None] * np.einsum("eij,ekl->eijkl", eps, eps)
        return g


# ------------------------------------------------------------------ shell ---
def simpson_stations(n: int):
    """Normalised through-thickness stations in [-1/2, 1/2] and Simpson
    weights summing to one (shell.py:136-144)."""
    z = np.linspace(-0.5, 0.5, n)
    w = np.ones(n)
    w[1:-1:2] = 4.0
    w[2:-2:2] = 2.0
    return z, w / (3.0 * (n - 1))


def shell_frames(nodes, elements, orientation=None):
    """Element frames (rows: material axis 1, axis 2, normal) and the nodes'
    in-plane coordinates relative to node 0 (shell.py:358-380)."""
    X = np.asarray(nodes, dtype=np.float64)[np.asarray(elements)]
    n = np.cross(X[:, 1] - X[:, 0], X[:, 2] - X[:, 1])
    n /= np.linalg.norm(n, axis=1, keepdims=True)
    o = np.broadcast_to(np.asarray([1.0, 0.0, 0.0] if orientation is None else orientation, dtype=np.float64),
                        n.shape)
    proj = o - (o * n).sum(1, keepdims=True) * n
    degenerate = np.linalg.norm(proj, axis=1, keepdims=True) < 1e-8
    a1 = np.where(degenerate, X[:, 1] - X[:, 0], proj)
    a1 /= np.linalg.norm(a1, axis=1, keepdims=True)
    a2 = np.cross(n, a1)
    a2 /= np.linalg.norm(a2, axis=1, keepdims=True)
    t = np.stack([a1, a2, n], axis=1)
    loc = np.einsum("eij,eaj->eai", t[:, :2], X - X[:, :1])
    return t, loc


def shell_operators(loc):
    """Per element: area A, in-plane shape gradients B [2, 3] and the
    generalised strain operators on the 18 local DOFs (u, v, w, rx, ry, rz
    per node): membrane Dm [3, 18], curvature Db [3, 18] and the averaged
    transverse shear Ds [2, 18] (shell.py:263-356)."""
    dn = np.array([[-1.0, 1.0, 0.0], [-1.0, 0.0, 1.0]])
    J = np.einsum("iN,eNj->eij", dn, loc)
    detJ = np.linalg.det(J)
    if np.any(detJ <= 0.0):
        raise ValueError("Negative Jacobian")
    B = np.linalg.inv(J) @ dn
    E = loc.shape[0]
    A = detJ / 2.0
    Dm = np.zeros((E, 3, 18))
    Db = np.zeros((E, 3, 18))
    for a in range(3):
        bx, by = B[:, 0, a], B[:, 1, a]
        Dm[:, 0, 6 * a] = bx
        Dm[:, 1, 6 * a + 1] = by
        Dm[:, 2, 6 * a] = by
        Dm[:, 2, 6 * a + 1] = bx
        Db[:, 0, 6 * a + 4] = bx
        Db[:, 1, 6 * a + 3] = -by
        Db[:, 2, 6 * a + 3] = -bx
        Db[:, 2, 6 * a + 4] = by
    Ds = np.zeros((E, 2, 18))
    for p0, p1, p2 in ((0, 1, 2), (1, 2, 0), (2, 0, 1)):
        a = loc[:, p1, 0] - loc[:, p0, 0]
        b = loc[:, p1, 1] - loc[:, p0, 1]
        c = loc[:, p2, 0] - loc[:, p0, 0]
        d = loc[:, p2, 1] - loc[:, p0, 1]
        Ds[:, 0, 6 * p0 + 2] += b - d
        Ds[:, 0, 6 * p0 + 4] += A
        Ds[:, 1, 6 * p0 + 2] += c - a
        Ds[:, 1, 6 * p0 + 3] += -A
        Ds[:, 0, 6 * p1 + 2] += d
        Ds[:, 0, 6 * p1 + 3] += -b * d / 2.0
        Ds[:, 0, 6 * p1 + 4] += a * d / 2.0
        Ds[:, 1, 6 * p1 + 2] += -c
        Ds[:, 1, 6 * p1 + 3] += b * c / 2.0
        Ds[:, 1, 6 * p1 + 4] += -a * c / 2.0
        Ds[:, 0, 6 * p2 + 2] += -b
        Ds[:, 0, 6 * p2 + 3] += b * d / 2.0
        Ds[:, 0, 6 * p2 + 4] += -b * c / 2.0
        Ds[:, 1, 6 * p2 + 2] += a
        Ds[:, 1, 6 * p2 + 3] += -a * d / 2.0
        Ds[:, 1, 6 * p2 + 4] += a * c / 2.0
    Ds /= (3.0 * 2.0 * A)[:, None, None]
    return A, B, detJ, Dm, Db, Ds


def shell_rotation(t):
    """Block-diagonal [18, 18] map from global to local DOFs (six copies of t)."""
    T = np.zeros((t.shape[0], 18, 18))
    for k in range(6):
        T[:, 3 * k:3 * k + 3, 3 * k:3 * k + 3] = t
    return T


def plane_stress_voigt(E, nu):
    """Voigt [3, 3] of the isotropic plane-stress tensor (elasticity.py:130-182)."""
    E = np.asarray(E, dtype=np.float64)
    f = E / (1.0 - nu**2)
    C = np.zeros(E.shape + (3, 3))
    C[..., 0, 0] = C[..., 1, 1] = f
    C[..., 0, 1] = C[..., 1, 0] = f * nu
    C[..., 2, 2] = f * (1.0 - nu) / 2.0
    return C


def shell_stiffness(nodes, elements, Cv, Gs, h, kappa=5.0 / 6.0, nu_t=0.5, drill=1.0, n_simpson=3,
                    orientation=None):
    """Global element matrices [E, 18, 18] of the homogeneous Tria1 shell:
    T^T (km + kb + kc + ks + kd) T with ABD from Simpson stations, transverse
    shear scaled by psi = kappa h^2 / (h^2 + alpha he^2) (shell.py:416-586)."""
    t, loc = shell_frames(nodes, elements, orientation)
    A, _, detJ, Dm, Db, Ds = shell_operators(loc)
    h = np.asarray(h, dtype=np.float64)
    zh, wh = simpson_stations(n_simpson)
    Am = np.zeros_like(Cv)
    Bm = np.zeros_like(Cv)
    Dmat = np.zeros_like(Cv)
    for z, w in zip(zh, wh):
        zz, ww = (z * h)[:, None, None], (w * h)[:, None, None]
        Am += Cv * ww
        Bm += Cv * ww * zz
        Dmat += Cv * ww * zz**2
    wd = (0.5 * detJ)[:, None, None]  # Tria1 weight 1/2 times detJ
    km = wd * np.einsum("eji,ejk,ekl->eil", Dm, Am, Dm)
    kb = wd * np.einsum("eji,ejk,ekl->eil", Db, Dmat, Db)
    kc = wd * (np.einsum("eji,ejk,ekl->eil", Dm, Bm, Db) + np.einsum("eji,ejk,ekl->eil", Db, Bm, Dm))
    he = np.sqrt(2.0) * np.sqrt(A)
    alpha = kappa / (2.0 * (1.0 + nu_t))
    psi = kappa * h**2 / (h**2 + alpha * he**2)
    As = np.zeros((len(h), 2, 2))
    As[:, 0, 0] = h * Gs[:, 0]
    As[:, 1, 1] = h * Gs[:, 1]
    ks = wd * np.einsum("eji,ejk,ekl->eil", Ds, psi[:, None, None] * As, Ds)
    kl = km + kb + kc + ks
    for a in range(3):
        kl[:, 6 * a + 5, 6 * a + 5] += drill
    T = shell_rotation(t)
    return np.einsum("eji,ejk,ekl->eil", T, kl, T)


def shell_station_stress(nodes, elements, Cv, h, u, n_simpson=3, orientation=None):
    """Cauchy stresses [n_stations, E, 2, 2] of the total displacements u
    [n_nod, 6] from zero prestress: C (eps_m + z kappa) at each station
    (shell.py:474-504)."""
    t, loc = shell_frames(nodes, elements, orientation)
    _, _, _, Dm, Db, _ = shell_operators(loc)
    ue = np.asarray(u, dtype=np.float64)[np.asarray(elements)].reshape(len(elements), 18)
    ul = np.einsum("eij,ej->ei", shell_rotation(t), ue)
    em = np.einsum("eij,ej->ei", Dm, ul)
    kb = np.einsum("eij,ej->ei", Db, ul)
    zh, _ = simpson_stations(n_simpson)
    out = []
    for z in zh:
        ev = em + (z * h)[:, None] * kb
        sv = np.einsum("eij,ej->ei", Cv, ev)
        out.append(np.stack([np.stack([sv[:, 0], sv[:, 2]], -1), np.stack([sv[:, 2], sv[:, 1]], -1)], -2))
    return np.stack(out)


# ------------------------------------------------------------- workloads ---
def cube_hexa(Nx, Ny, Nz, Lx=1.0, Ly=1.0, Lz=1.0):
    """Node/element numbering of the reference's cube_hexa (mesh.py:8-46)."""
    X, Y, Z = np.linspace(0, Lx, Nx), np.linspace(0, Ly, Ny), np.linspace(0, Lz, Nz)
    x, y, z = np.meshgrid(X, Y, Z, indexing="ij")
    nodes = np.stack([x.ravel(), y.ravel(), z.ravel()], axis=1)
    ids = np.arange(Nx * Ny * Nz).reshape(Nx, Ny, Nz)
    c = lambda i, j, k: ids[i : Nx - 1 + i, j : Ny - 1 + j, k : Nz - 1 + k].ravel()  # noqa: E731
    el = np.stack([c(0, 0, 0), c(1, 0, 0), c(1, 1, 0), c(0, 1, 0), c(0, 0, 1), c(1, 0, 1), c(1, 1, 1), c(0, 1, 1)], 1)
    return nodes, el


def rect_quad(Nx, Ny, Lx=1.0, Ly=1.0):
    """Node/element numbering of the reference's rect_quad (mesh.py:103-135)."""
    X, Y = np.linspace(0, Lx, Nx), np.linspace(0, Ly, Ny)
    x, y = np.meshgrid(X, Y, indexing="ij")
    nodes = np.stack([x.ravel(), y.ravel()], axis=1)
    ids = np.arange(Nx * Ny).reshape(Nx, Ny)
    c = lambda i, j: ids[i : Nx - 1 + i, j : Ny - 1 + j].ravel()  # noqa: E731
    return nodes, np.stack([c(0, 0), c(1, 0), c(1, 1), c(0, 1)], 1)


# ------------------------------------------------------- nonlinear points ---
def neo_hookean_point(F, mu, lam):
    """First Piola stress and tangent of the Neo-Hookean energy
    psi = mu/2 (tr C - 3) - mu ln J + lam/2 (ln J)^2 (the energy of
    benchmarks/hyperelasticity.py:24-30, differentiated by jacrev in
    materials/hyperelasticity.py:117-123).  F [n, 3, 3]; mu, lam [n]."""
    Fi = np.linalg.inv(F)
    lnJ = np.log(np.linalg.det(F))
    P = mu[:, None, None] * F + (lam * lnJ - mu)[:, None, None] * Fi.transpose(0, 2, 1)
    I = np.eye(3)
    A = (mu[:, None, None, None, None] * np.einsum("ik,JL->iJkL", I, I)
         + lam[:, None, None, None, None] * np.einsum("nJi,nLk->niJkL", Fi, Fi)
         + (mu - lam * lnJ)[:, None, None, None, None] * np.einsum("nJk,nLi->niJkL", Fi, Fi))
    return P, A


def j2_plane_strain_point(H_inc, stress, state, E, nu, sigma_y, hard, de0=None, tol=1e-5, max_iter=10):
    """Return mapping of IsotropicPlasticityPlaneStrain.step
    (materials/plasticity.py:504-590) with linear hardening
    sigma_f(q) = sigma_y + hard q.  H_inc, stress [n, 2, 2]; state [n, 2]
    = (q, eps_z^p).  Returns stress_new, state_new, ddsdde [n, 2, 2, 2, 2]."""
    n = H_inc.shape[0]
    lbd = E * nu / ((1.0 + nu) * (1.0 - 2.0 * nu))
    G = E / (2.0 * (1.0 + nu))
    C = elastic_c("plane_strain", E, nu, n)
    de = 0.5 * (H_inc.transpose(0, 2, 1) + H_inc) - (0.0 if de0 is None else de0)
    q = state[:, 0].copy()
    ez = state[:, 1].copy()
    s2 = stress + np.einsum("nijkl,nkl->nij", C, de)
    s3 = np.zeros((n, 3, 3))
    s3[:, :2, :2] = s2
    s3[:, 2, 2] = nu * (s2[:, 0, 0] + s2[:, 1, 1]) - E * ez
    dev = s3 - np.trace(s3, axis1=1, axis2=2)[:, None, None] / 3.0 * np.eye(3)
    nrm = np.linalg.norm(dev, axis=(1, 2))
    c = np.sqrt(2.0 / 3.0)
    fm = nrm - c * (sigma_y + hard * q) > 0
    stress_new = s2.copy()
    ddsdde = C.copy()
    if fm.any():
        nn = dev[fm] / nrm[fm][:, None, None]
        Gf = np.broadcast_to(G, (n,))[fm]
        dG = np.zeros(fm.sum())
        qf = q[fm]
        for _ in range(max_iter):
            res = nrm[fm] - 2.0 * Gf * dG - c * (sigma_y + hard * qf)
            dd = res / (2.0 * Gf + 2.0 / 3.0 * hard)
            dG = dG + dd
            qf = qf + c * dd
            if (np.abs(res) < tol).all():
                break
        stress_new[fm] = (s3[fm] - (2.0 * Gf * dG)[:, None, None] * nn)[:, :2, :2]
        q[fm] = qf
        ez[fm] = ez[fm] + dG * nn[:, 2, 2]
        A = 2.0 * Gf / (1.0 + hard / (3.0 * Gf))
        B = 4.0 * Gf**2 * dG / nrm[fm]
        n00, n11, n01, n10 = nn[:, 0, 0], nn[:, 1, 1], nn[:, 0, 1], nn[:, 1, 0]
        d = ddsdde[fm]
        d[:, 0, 0, 0, 0] += -A * n00**2 - B * (2 / 3 - n00**2)
        d[:, 1, 1, 1, 1] += -A * n11**2 - B * (2 / 3 - n11**2)
        d[:, 0, 0, 1, 1] += -A * n00 * n11 - B * (-1 / 3 - n00 * n11)
        d[:, 1, 1, 0, 0] += -A * n00 * n11 - B * (-1 / 3 - n00 * n11)
        d[:, 0, 1, 0, 1] += -A * n01**2 - B * (1 / 2 - n01**2)
        d[:, 0, 1, 1, 0] += -A * n01**2 - B * (1 / 2 - n10**2)
        d[:, 1, 0, 0, 1] += -A * n10**2 - B * (1 / 2 - n01**2)
        d[:, 1, 0, 1, 0] += -A * n10**2 - B * (1 / 2 - n10**2)
        ddsdde[fm] = d
    return stress_new, np.stack([q, ez], axis=-1), ddsdde
