"""CPU restatement of the library's smoothed-aggregation multigrid (test
infrastructure: only tests/ use it, as the checker of the GPU hierarchy).

The reference preconditions its iterative solves with smoothed-aggregation
AMG: on the CPU pyamg.smoothed_aggregation_solver(A, B, smooth="jacobi")
(src/torchfem/sparse.py:495-507; pyamg is not vendored in the reference and
not installed here) with B = FEM.compute_B() (src/torchfem/base.py:316-344),
on the GPU AmgX aggregation AMG (src/torchfem/amgx.py:62-91).  The library
builds the same kind of hierarchy with GPU-parallel choices, restated here
step by step so that its arrays can be compared:

- aggregation: roots = a distance-2 maximal independent set under the fixed
  priorities (state, lowbias32(i) >> 2, i); then two passes attach each
  unassigned node to the aggregate of its assigned neighbour of largest
  (lowbias32(j) >> 2, j) (Bell, Dalton & Olson, SIAM J. Sci. Comput. 34
  (2012) C123);
- tentative prolongator: per aggregate, Cholesky of the Gram matrix of the
  near-null rows with rank drop (pivot <= 1e-10 of the diagonal), Q = rows of
  B R^-1, coarse near-null space R (rows about the aggregate centroid on the
  finest level, carried to the global centroid) (Vanek, Mandel & Brezina
  1996);
- P = (I - w D^-1 A) T with w = 4 / (3 rho), D the block diagonal;
- A_c = P^T A P, with a unit diagonal for a dropped (zero) coarse DOF;
- Chebyshev degree 2 on [0.1, 1.1] rho, V(2,2) cycle, dense coarsest solve.
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp

COARSE_MAX_DOF = 96
DROP_TOL = 1e-10
OMEGA = 4.0 / 3.0
CHEB_LO, CHEB_HI = 0.1, 1.1


def lowbias32(x):
    """The integer hash behind the aggregation priorities (C. Wellons)."""
    x = np.asarray(x, dtype=np.uint64) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(16)
    x = (x * np.uint64(0x7FEB352D)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(15)
    x = (x * np.uint64(0x846CA68B)) & np.uint64(0xFFFFFFFF)
    x ^= x >> np.uint64(16)
    return x


def _keys(state, n):
    i = np.arange(n, dtype=np.uint64)
    k = (state.astype(np.uint64) << np.uint64(62)) | ((lowbias32(i) >> np.uint64(2)) << np.uint64(32)) | i
    k[state == 0] = 0
    return k


def aggregate(ptr, idx, active):
    """(agg [n] int32 with -1 for inactive nodes, n_agg)."""
    n = len(ptr) - 1
    rows = np.repeat(np.arange(n), np.diff(ptr))
    ok = active[rows] & active[idx]
    r, c = rows[ok], idx[ok]
    state = np.where(active, 1, 0).astype(np.int64)
    while np.any(state == 1):
        k0 = _keys(state, n)
        k1 = np.zeros(n, np.uint64)
        np.maximum.at(k1, r, k0[c])
        k2 = np.zeros(n, np.uint64)
        np.maximum.at(k2, r, k1[c])
        und = state == 1
        own = _keys(np.ones(n, np.int64), n)
        win = und & (k2 == own)
        lose = und & ~win & ((k2 >> np.uint64(62)) == 2)
        state = state.copy()
        state[win] = 2
        state[lose] = 0
    roots = state == 2
    agg = np.where(roots, np.cumsum(roots) - 1, -1).astype(np.int64)
    jk = (np.uint64(1) << np.uint64(63)) | ((lowbias32(np.arange(n)) >> np.uint64(2)) << np.uint64(32)) | np.arange(
        n, dtype=np.uint64)
    rows_all = np.repeat(np.arange(n), np.diff(ptr))
    for _ in range(2):
        cand = np.where(agg[idx] >= 0, jk[idx], np.uint64(0))
        best = np.zeros(n, np.uint64)
        np.maximum.at(best, rows_all, cand)
        new = agg.copy()
        sel = (agg < 0) & active & (best > 0)
        j = (best[sel] & np.uint64(0xFFFFFFFF)).astype(np.int64)
        new[sel] = agg[j]
        agg = new
    if np.any(agg[active] < 0):
        raise RuntimeError("aggregation left nodes unassigned")
    return agg.astype(np.int32), int(roots.sum())


def null_rows(coords, con, b, K, center):
    """Near-null rows [n, b, K] about `center` (FEM.compute_B's modes; the
    constant field for one DOF per node)."""
    n = coords.shape[0]
    B = np.zeros((n, b, K))
    for r in range(b):
        B[:, r, r] = 1.0
    p = coords - center
    if b == 3:
        x, y, z = p[:, 0], p[:, 1], p[:, 2]
        B[:, 0, 4], B[:, 0, 5] = z, -y
        B[:, 1, 3], B[:, 1, 5] = -z, x
        B[:, 2, 3], B[:, 2, 4] = y, -x
    elif b == 2:
        B[:, 0, 2], B[:, 1, 2] = p[:, 1], -p[:, 0]
    if con is not None:
        B[con.reshape(n, b)] = 0.0
    return B


def tentative(agg, n_agg, b, K, coords=None, con=None, bn=None):
    """T [n, b, K] (rows of Q) and the coarse near-null rows [n_agg, K, K]."""
    n = agg.shape[0]
    T = np.zeros((n, b, K))
    Bc = np.zeros((n_agg, K, K))
    origin = coords.mean(axis=0) if bn is None else None
    for a in range(n_agg):
        mem = np.nonzero(agg == a)[0]
        if bn is None:
            c = coords[mem].mean(axis=0)
            M = null_rows(coords[mem], None if con is None else con.reshape(n, b)[mem], b, K, c)
        else:
            M = bn[mem]
        M = M.reshape(-1, K)
        G = M.T @ M
        R = np.zeros((K, K))
        keep = np.zeros(K, bool)
        for j in range(K):
            d = G[j, j] - np.sum(R[:j, j] ** 2)
            keep[j] = G[j, j] > 0.0 and d > DROP_TOL * G[j, j]
            if not keep[j]:
                continue
            R[j, j] = np.sqrt(d)
            for q in range(j + 1, K):
                R[j, q] = (G[j, q] - R[:j, j] @ R[:j, q]) / R[j, j]
        Q = np.zeros_like(M)
        for k in range(K):
            if keep[k]:
                Q[:, k] = (M[:, k] - Q[:, :k] @ R[:k, k]) / R[k, k]
        T[mem] = Q.reshape(len(mem), b, K)
        S = np.eye(K)
        if bn is None and b > 1:
            cx, cy = c[0] - origin[0], c[1] - origin[1]
            if b == 3:
                cz = c[2] - origin[2]
                S[1, 3], S[2, 3], S[0, 4], S[2, 4], S[0, 5], S[1, 5] = -cz, cy, cz, -cx, -cy, cx
            else:
                S[0, 2], S[1, 2] = cy, -cx
        Bc[a] = R @ S
    return T, Bc


def block_pattern(A, b):
    """Row pointers and sorted block columns of the b x b block pattern of A."""
    Ab = sp.bsr_matrix(A, blocksize=(b, b))
    Ab.sort_indices()
    return Ab.indptr.astype(np.int64), Ab.indices.astype(np.int64), Ab


def block_diag_inv(A, b):
    n = A.shape[0] // b
    D = np.zeros((n, b, b))
    A = A.tocsr()
    for r in range(b):
        for c in range(b):
            rows = np.arange(n) * b + r
            D[:, r, c] = np.asarray(A[rows, np.arange(n) * b + c]).ravel()
    return np.linalg.inv(D)


def bsr_blockdiag(Dinv):
    n, b, _ = Dinv.shape
    return sp.bsr_matrix((Dinv, np.arange(n), np.arange(n + 1)), shape=(n * b, n * b)).tocsr()


def lam_max(A, Dinv_op, iters=60, seed=3):
    """Largest eigenvalue of D^-1 A (power iteration, for the checks)."""
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(A.shape[0])
    lam = 0.0
    for _ in range(iters):
        w = Dinv_op @ (A @ v)
        lam = np.linalg.norm(w) / np.linalg.norm(v)
        v = w / np.linalg.norm(w)
    return lam


def to_sparse_T(T, agg, K):
    n, b, _ = T.shape
    rows, cols, vals = [], [], []
    for i in np.nonzero(agg >= 0)[0]:
        for r in range(b):
            for k in range(K):
                rows.append(i * b + r)
                cols.append(agg[i] * K + k)
                vals.append(T[i, r, k])
    n_agg = int(agg.max()) + 1 if np.any(agg >= 0) else 0
    return sp.csr_matrix((vals, (rows, cols)), shape=(n * b, n_agg * K))


class Level:
    pass


def hierarchy(A, coords, con, dim, rhos=None):
    """Levels of the multigrid hierarchy of the condensed matrix A (scipy,
    FP64).  rhos: spectral estimates per level (default: power iteration)."""
    K = 6 if dim == 3 else (3 if dim == 2 else 1)
    b = dim
    n = A.shape[0] // b
    ptr, idx, _ = block_pattern(A, b)
    active = ~np.all(con.reshape(n, b), axis=1) if con is not None else np.ones(n, bool)
    levels = []
    bn = None
    level = 0
    while True:
        L = Level()
        L.A, L.b = A.tocsr(), b
        L.Dinv = block_diag_inv(A, b)
        levels.append(L)
        if level >= 1 and A.shape[0] <= COARSE_MAX_DOF:
            L.dense_inv = np.linalg.inv(A.toarray())
            break
        L.rho = rhos[level] if rhos is not None else lam_max(A, bsr_blockdiag(L.Dinv))
        L.agg, L.n_agg = aggregate(ptr, idx, active)
        if level == 0:
            L.T, Bc = tentative(L.agg, L.n_agg, b, K, coords=coords, con=con)
        else:
            L.T, Bc = tentative(L.agg, L.n_agg, b, K, bn=bn)
        Ts = to_sparse_T(L.T, L.agg, K)
        omega = OMEGA / L.rho
        P = (Ts - omega * (bsr_blockdiag(L.Dinv) @ (L.A @ Ts))).tocsr()
        L.P = P
        Ac = (P.T @ L.A @ P).tocsr()
        d = Ac.diagonal()
        zero = d == 0.0
        if zero.any():
            Ac = (Ac + sp.diags(zero.astype(float))).tocsr()
        A, b, bn = Ac, K, Bc
        ptr, idx, _ = block_pattern(A, b)
        active = np.ones(A.shape[0] // b, bool)
        level += 1
    return levels


def chebyshev(L, f, x):
    lo, hi = CHEB_LO * L.rho, CHEB_HI * L.rho
    theta, delta = 0.5 * (hi + lo), 0.5 * (hi - lo)
    sigma = theta / delta
    rho0 = 1.0 / sigma
    rho1 = 1.0 / (2.0 * sigma - rho0)
    D = bsr_blockdiag(L.Dinv)
    r = f - L.A @ x if x is not None else f.copy()
    x = np.zeros_like(f) if x is None else x.copy()
    d = (D @ r) / theta
    x = x + d
    r = r - L.A @ d
    d = rho1 * rho0 * d + (2.0 * rho1 / delta) * (D @ r)
    return x + d


def vcycle(levels, f, level=0):
    L = levels[level]
    if hasattr(L, "dense_inv"):
        return L.dense_inv @ f
    x = chebyshev(L, f, None)
    r = f - L.A @ x
    x = x + L.P @ vcycle(levels, L.P.T @ r, level + 1)
    return chebyshev(L, f, x)


def pcg(A, b, levels, rtol=1e-10, max_iter=500):
    """CG preconditioned by one V-cycle; returns (x, iterations)."""
    x = np.zeros_like(b)
    r = b.copy()
    bn = np.linalg.norm(b)
    p = None
    rz = None
    for it in range(1, max_iter + 1):
        z = vcycle(levels, r)
        rz_new = r @ z
        p = z if p is None else z + (rz_new / rz) * p
        rz = rz_new
        q = A @ p
        alpha = rz / (p @ q)
        x += alpha * p
        r -= alpha * q
        if np.linalg.norm(r) <= rtol * bn:
            return x, it
    return x, max_iter
