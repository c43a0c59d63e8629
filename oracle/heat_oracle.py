"""CPU oracle of torch-fem's heat-conduction path — TEST INFRASTRUCTURE ONLY.

numpy/scipy restatement of the reference's steady and transient heat
conduction, used by `tests/` to check the GPU library.  The product
(`torch-fem_gb300/`) never imports it.

Parity pin: tests/test_oracle.py checks every function here against
tests/golden/heat_cases.npz, generated by running the reference itself
(tests/golden/make_golden.py, `make_heat`).

Restated reference code (paths relative to the torch-fem repository):
  Heat.integrate_material  src/torchfem/base.py:1177-1286 with compute_k /
                           compute_f (solid.py:52-58, planar.py:86-92) and the
                           Fourier law of materials/conductivity.py:80-99
  integrate_mass           src/torchfem/base.py:376-396 with compute_m
                           (solid.py:60-62, planar.py:94-96)
  solve (linear)           src/torchfem/base.py:597-923
  adjoint                  src/torchfem/sparse.py:641-724
  time_integration         src/torchfem/base.py:1288-1553 (Crank-Nicolson)
  its gradients            the reverse sweep of those steps, pinned to the
                           reference's autograd (heat_transient_grad.npz)
"""

from __future__ import annotations

import math
import time

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla

from .fem_oracle import ELEMENTS, assemble_matrix, assemble_rhs, element_name, pattern, shape_gradients

_HEX_SIGNS = np.array(
    [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1), (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)],
    dtype=np.float64,
)
_QUAD_SIGNS = np.array([(-1, -1), (1, -1), (1, 1), (-1, 1)], dtype=np.float64)


def shape_values(etype: str) -> np.ndarray:
    """N at the integration points [nip, n_e] (elements.py Quad1 / Hexa1)."""
    _, dim, ip, _, _ = ELEMENTS[etype]
    signs = {"Quad1": _QUAD_SIGNS, "Hexa1": _HEX_SIGNS}[etype]
    return np.prod(1.0 + signs[None] * ip[:, None, :], axis=-1) / 2.0**dim


class HeatModel:
    """Linear heat conduction on one mesh: kappa [n_elem, dim, dim] (or
    [dim, dim]), thickness per element for planar meshes."""

    def __init__(self, nodes, elements, kappa, thickness=None, rho=None):
        self.nodes = np.asarray(nodes, dtype=np.float64)
        self.elements = np.asarray(elements, dtype=np.int64)
        self.n_elem, self.n_e = self.elements.shape
        self.dim = self.nodes.shape[1]
        self.n_nod = self.nodes.shape[0]
        self.etype = element_name(self.n_e, self.dim)
        kappa = np.asarray(kappa, dtype=np.float64)
        self.kappa = np.broadcast_to(kappa, (self.n_elem, self.dim, self.dim))
        self.t = np.ones(self.n_elem) if thickness is None else np.broadcast_to(np.asarray(thickness, float), (self.n_elem,))
        self.rho = None if rho is None else np.broadcast_to(np.asarray(rho, float), (self.n_elem,))
        self.B, self.detJ, self.w = shape_gradients(self.nodes, self.elements, self.etype)  # B [nip, E, dim, n_e]
        self.glob_idx, self.k_map, self.diag_map, self.idx = pattern(self.elements, self.n_nod, 1)
        self.nnz = self.glob_idx.shape[1]

    # -------------------------------------------------------- element level --
    def conductivity(self):
        """k_e = sum_ip w detJ t B^T kappa B (base.py:1264-1273)."""
        wj = self.w[:, None] * self.detJ * self.t[None]
        return np.einsum("iE,iEaN,Eab,iEbM->ENM", wj, self.B, self.kappa, self.B)

    def capacity(self):
        """m_e = sum_ip w detJ t rho N N^T (base.py:376-396)."""
        N = shape_values(self.etype)
        wj = self.w[:, None] * self.detJ * (self.t * self.rho)[None]
        return np.einsum("iE,iN,iM->ENM", wj, N, N)

    def integrate(self, dT, flux_prev=None):
        """(f_e [E, n_e], flux [nip, E, dim], grad_inc [nip, E, dim]) of a
        temperature increment (base.py:1236-1262)."""
        g = np.einsum("iEaN,EN->iEa", self.B, dT[self.elements])
        flux = np.einsum("Eab,iEb->iEa", self.kappa, g)
        if flux_prev is not None:
            flux = flux + flux_prev
        wj = self.w[:, None] * self.detJ * self.t[None]
        f = np.einsum("iE,iEaN,iEa->EN", wj, self.B, flux)
        return f, flux, g

    # --------------------------------------------------------------- global --
    def matrix(self, con, k=None):
        k = self.conductivity() if k is None else k
        val = assemble_matrix(k, self.k_map, self.nnz, self.glob_idx, self.diag_map, con)
        return sp.csr_matrix((val, (self.glob_idx[0], self.glob_idx[1])), shape=(self.n_nod, self.n_nod))

    def internal(self, T, flux_prev=None):
        f, flux, g = self.integrate(T, flux_prev)
        return assemble_rhs(f, self.idx, self.n_nod), flux, g

    cg_iterations: list = []  # iterations of every Jacobi-CG solve (appended per solve)
    cg_seconds: list = []  # wall time of every Jacobi-CG solve

    @staticmethod
    def linear_solve(K, b, method="spsolve", rtol=1e-12):
        """spsolve, or Jacobi-preconditioned CG to ||r|| <= rtol ||b||."""
        if method == "spsolve":
            return spla.spsolve(K.tocsc(), b)
        dinv = 1.0 / K.diagonal()
        count = [0]

        def tick(_):
            count[0] += 1

        t0 = time.perf_counter()
        x, info = spla.cg(K.tocsr(), b, rtol=rtol, atol=0.0, maxiter=10 * K.shape[0],
                          M=spla.LinearOperator(K.shape, matvec=lambda v: dinv * v), callback=tick)
        HeatModel.cg_seconds.append(time.perf_counter() - t0)
        HeatModel.cg_iterations.append(count[0])
        if info != 0:
            raise RuntimeError(f"CG did not converge ({info})")
        return x

    def solve(self, q, constraints, temperatures=None, method="spsolve", rtol=1e-12):
        """One load increment of the linear solve (base.py:704-857):
        K dT = q - f_int(T_bc) on the free DOFs, T = T_bc on the constrained."""
        con = np.nonzero(np.asarray(constraints).ravel())[0]
        Tbc = np.zeros(self.n_nod)
        if temperatures is not None:
            Tbc[con] = np.asarray(temperatures).ravel()[con]
        K = self.matrix(con).tocsc()
        f0, _, _ = self.internal(Tbc)
        res = f0 - np.asarray(q).ravel()
        res[con] = 0.0
        T = Tbc - self.linear_solve(K, res, method, rtol)
        self.K, self.con = K, con
        f, flux, g = self.internal(T)
        return T, f, flux, g

    def adjoint(self, g_T, method="spsolve", rtol=1e-12):
        """lambda with K^T lambda = g_T, lambda = 0 on constrained DOFs
        (sparse.py:671-680)."""
        g = np.array(g_T, dtype=np.float64).ravel()
        g[self.con] = 0.0
        return self.linear_solve(self.K.T, g, method, rtol)

    def compliance_grads(self, T, f):
        """d(f.T)/d(kappa_e) [E, dim, dim], d(f.T)/d(t_e) [E] and d(f.T)/dq
        for the converged state.  f = K T on all DOFs (the internal heat
        flux), so L = T^T K_full T with T = T(q, kappa); dL = 2 T^T dK T
        - lambda^T dR with dR = dK T - dq on the free DOFs; with lambda solved
        from K lambda = 2 K_full T restricted to the free DOFs."""
        con = self.con
        free = np.ones(self.n_nod, dtype=bool)
        free[con] = False
        kfull = self.conductivity()
        Kf = self.matrix(np.array([], dtype=np.int64), kfull)
        g_T = (Kf @ T) + (Kf.T @ T)  # dL/dT through f(T) and T
        lam = self.adjoint(g_T)
        Te = T[self.elements]
        le = lam[self.elements]
        # dL/dk_e = T_e T_e^T - lambda_e T_e^T (the residual R = f_int - q)
        dk = np.einsum("EN,EM->ENM", Te, Te) - np.einsum("EN,EM->ENM", le * free[self.elements], Te)
        wj = self.w[:, None] * self.detJ * self.t[None]
        g_kappa = np.einsum("ENM,iE,iEaN,iEbM->Eab", dk, wj, self.B, self.B)
        wj0 = self.w[:, None] * self.detJ
        k_unit = np.einsum("iE,iEaN,Eab,iEbM->ENM", wj0, self.B, self.kappa, self.B)
        g_t = np.einsum("ENM,ENM->E", dk, k_unit)
        g_q = lam
        return g_kappa, g_t, g_q


def time_grid(t_output, delta_t):
    """Internal times and the rows of the outputs (base.py:1387-1411)."""
    t_output = np.asarray(t_output, dtype=np.float64)
    knots = t_output if t_output[0] <= 0.0 else np.concatenate([[0.0], t_output])
    chunks = [knots[:1]]
    rows = [] if t_output[0] > 0.0 else [0]
    row = 0
    for a, b in zip(knots[:-1], knots[1:]):
        ratio = (b - a) / delta_t
        n_sub = max(1, math.ceil(ratio - 1e-9 * max(1.0, ratio)))
        sub = np.linspace(a, b, n_sub + 1)[1:]
        sub[-1] = b
        chunks.append(sub)
        row += n_sub
        rows.append(row)
    return np.concatenate(chunks), np.array(rows)


def time_integration(model: HeatModel, constraints, temperatures, q, t_output, delta_t, rtol=1e-8, atol=1e-6,
                     max_iter=100):
    """Crank-Nicolson integration (base.py:1288-1553): equilibrium at t = 0
    with every temperature prescribed, then per step Newton on
    r = M du + dt/2 (f_old + f_int + f_ext), r = 0 on constrained DOFs, solved
    with (M + dt/2 K) du = -r.  The first step's f_old is zero, as in the
    reference.  Returns (T [n_out, n_nod], f [n_out, n_nod],
    flux [n_out, nip, E, dim], grad [n_out, nip, E, dim])."""
    n = model.n_nod
    temperatures = np.asarray(temperatures, float).ravel()
    q = np.asarray(q, float).ravel()
    T0, _, flux0, g0 = model.solve(np.zeros(n), np.ones(n, dtype=bool), temperatures)
    times, rows = time_grid(t_output, delta_t)
    con = np.nonzero(np.asarray(constraints).ravel())[0]
    K = model.matrix(con)
    M = model.matrix(con, model.capacity())
    nip = model.B.shape[0]
    T = np.zeros((len(times), n))
    f = np.zeros((len(times), n))
    flux = np.zeros((len(times), nip, model.n_elem, model.dim))
    grad = np.zeros_like(flux)
    T[0], flux[0], grad[0] = T0, flux0, g0
    T[0][con] = temperatures[con]
    for k in range(1, len(times)):
        dt = times[k] - times[k - 1]
        guess = T[k - 1].copy()
        res0 = None
        for it in range(max_iter):
            du = guess - T[k - 1]
            fe, flux_k, g = model.integrate(du, flux[k - 1])
            f_int = assemble_rhs(fe, model.idx, n)
            flux[k], grad[k] = flux_k, grad[k - 1] + g
            r = M @ du + 0.5 * dt * (f[k - 1] + f_int + q)
            r[con] = 0.0
            rn = np.linalg.norm(r)
            if it == 0:
                res0 = rn
            if rn < rtol * res0 or rn < atol:
                break
            guess = guess + spla.spsolve((M + 0.5 * dt * K).tocsc(), -r)
        T[k], f[k] = guess, f_int
    return T[rows], f[rows], flux[rows], grad[rows]


def time_integration_adjoint(model: HeatModel, constraints, temperatures, q, t_output, delta_t, c):
    """Gradients of L = sum_k c_k . T(t_k) through the Crank-Nicolson
    integration of `time_integration` (base.py:1288-1553) for a linear
    conductivity, by reverse sweep of the discrete steps.

    With g_n the assembled B^T flux_n (g_0 = K u_0, u_0 the prescribed
    temperatures), h = dt_n / 2, P the projection on the free DOFs and
    A_n = P (M + h K) P, each step is one Newton correction (exact solve):
        s_n  = g_0 + q (n = 1; the reference's f_old of the first step is 0)
             = 2 g_{n-1} + q (n > 1; f_old = f_int of the previous step = g_{n-1})
        du_n = -A_n^-1 P h s_n,   g_n = g_{n-1} + K du_n,   u_n = u_{n-1} + du_n.
    Returns (L, dL/dkappa [E, dim, dim], dL/drho [E], dL/dq [n])."""
    n = model.n_nod
    con = np.asarray(constraints).ravel().astype(bool)
    free = ~con
    u0 = np.asarray(temperatures, float).ravel().copy()
    q = np.asarray(q, float).ravel()
    times, rows = time_grid(t_output, delta_t)
    c = np.asarray(c, float).reshape(len(rows), n)
    kel = model.conductivity()
    mel = model.capacity()
    K = model.matrix(np.array([], dtype=np.int64), kel).toarray()
    M = model.matrix(np.array([], dtype=np.int64), mel).toarray()
    Kff, Mff = K[np.ix_(free, free)], M[np.ix_(free, free)]
    # forward
    us, dus, gs, hs = [u0], [], [K @ u0], []
    for k in range(1, len(times)):
        h = 0.5 * (times[k] - times[k - 1])
        s = (gs[0] if k == 1 else 2.0 * gs[-1]) + q
        du = np.zeros(n)
        du[free] = -np.linalg.solve(Mff + h * Kff, h * s[free])
        dus.append(du)
        hs.append(h)
        gs.append(gs[-1] + K @ du)
        us.append(us[-1] + du)
    L = float(sum(c[j] @ us[r] for j, r in enumerate(rows)))
    # reverse
    cbar = np.zeros((len(times), n))
    for j, r in enumerate(rows):
        cbar[r] += c[j]
    ubar = cbar[-1].copy()
    gbar = np.zeros(n)
    Kbar = np.zeros((n, n))
    Mbar = np.zeros((n, n))
    qbar = np.zeros(n)
    for k in range(len(times) - 1, 0, -1):
        du, h = dus[k - 1], hs[k - 1]
        dubar = ubar.copy()
        # g_k = g_{k-1} + K du
        dubar += K.T @ gbar
        Kbar += np.outer(gbar, du)
        # du = -A^-1 P h s
        lam = np.zeros(n)
        lam[free] = np.linalg.solve((Mff + h * Kff).T, dubar[free])
        Af = np.outer(lam[free], du[free])
        Mbar[np.ix_(free, free)] -= Af
        Kbar[np.ix_(free, free)] -= h * Af
        sbar = -h * lam
        qbar += sbar
        if k == 1:
            gbar = gbar + sbar  # s_1 = g_0 + q
        else:
            gbar = gbar + 2.0 * sbar
        ubar = ubar + cbar[k - 1]
    # g_0 = K u_0 (u_0 prescribed, not a parameter)
    Kbar += np.outer(gbar, u0)
    # element parameters: K = sum_e kappa-contractions, M = sum_e rho_e m_e
    el = model.elements
    Kb_e = Kbar[el[:, :, None], el[:, None, :]]
    Mb_e = Mbar[el[:, :, None], el[:, None, :]]
    wj = model.w[:, None] * model.detJ * model.t[None]
    g_kappa = np.einsum("ENM,iE,iEaN,iEbM->Eab", Kb_e, wj, model.B, model.B)
    g_rho = np.einsum("ENM,ENM->E", Mb_e, mel / model.rho[:, None, None])
    return L, g_kappa, g_rho, qbar
