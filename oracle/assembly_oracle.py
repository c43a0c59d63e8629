"""CPU oracle of torch-fem's Assembly.solve for linear parts — TEST INFRASTRUCTURE ONLY.

numpy/scipy restatement of the reference's coupled solve, used by `tests/`
to pin the GPU library's assemblies and by `bench.py`'s CPU baseline of the
assembly workload.  The product (`torch-fem_gb300/`) never imports it.

Restated reference code (paths relative to the torch-fem repository):
  coupling rows        src/torchfem/assembly.py:180-257 (nearest primary node,
                       u_s = u_p + theta_p x (x_s - x_p), theta_s = theta_p)
  elimination map T    src/torchfem/assembly.py:258-294
  reduced stiffness    src/torchfem/assembly.py:295-334 (T^T K T, explicit
                       diagonal, Dirichlet condensation)
  solve                src/torchfem/assembly.py:378-608, one linear load step:
                       res = T^T (F_int(T q) - F_ext), q -= K_r^-1 res, and
                       the retained DOFs' forces T^T F_int

Parity pin: tests/test_oracle.py checks it against the reference's own
results in tests/golden/assembly_cases.npz (make_golden.py assembly).
"""

from __future__ import annotations

import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla


class PointPart:
    """A reference point: rigid-body DOFs (3 + 3 in 3D, 2 + 1 in 2D) or one
    temperature (heat), no stiffness (assembly.py:39-106)."""

    def __init__(self, position, heat: bool = False):
        self.nodes = np.asarray(position, dtype=np.float64).reshape(1, -1)
        dim = self.nodes.shape[1]
        self.d = 1 if heat else dim + (3 if dim == 3 else 1)
        self.n_nod = 1
        self.n_dofs = self.d
        self.forces = np.zeros((1, self.d))
        self.constraints = np.zeros((1, self.d), dtype=bool)
        self.displacements = np.zeros((1, self.d))


class ModelPart:
    """A model part: an oracle model with `matrix(con)` and `n_dofs` (the
    fem_oracle LinearModel or the heat_oracle HeatModel) and its loads."""

    def __init__(self, model, d: int):
        self.model = model
        self.nodes = model.nodes
        self.n_nod = model.nodes.shape[0]
        self.d = d
        self.n_dofs = self.n_nod * d
        self.forces = np.zeros((self.n_nod, d))
        self.constraints = np.zeros((self.n_nod, d), dtype=bool)
        self.displacements = np.zeros((self.n_nod, d))

    def stiffness(self):
        return self.model.matrix(np.zeros(0, dtype=np.int64)).tocsr()


class AssemblyOracle:
    def __init__(self, parts):
        self.parts = list(parts)
        self.dim = self.parts[0].nodes.shape[1]
        sizes = [p.n_dofs for p in self.parts]
        self.offsets = [int(sum(sizes[:i])) for i in range(len(sizes))]
        self.n_dofs = int(sum(sizes))
        self.eliminated: list[np.ndarray] = []
        self.rows: list[tuple[np.ndarray, np.ndarray, np.ndarray]] = []

    def _skew(self, r):
        r = np.concatenate([r, np.zeros((len(r), 3 - self.dim))], axis=1)
        out = np.zeros((len(r), 3, 3))
        for b in range(3):
            e = np.zeros(3)
            e[b] = 1.0
            out[:, :, b] = np.cross(np.broadcast_to(e, r.shape), r)
        return out  # out[:, dof, axis] = (e_axis x r)[dof]

    def coupling(self, si: int, mask, pi: int, primary_mask=None, dofs=None):
        sec, pri = self.parts[si], self.parts[pi]
        dofs = list(range(sec.d)) if dofs is None else list(dofs)
        s_nodes = np.nonzero(np.asarray(mask))[0]
        p_cand = np.arange(pri.n_nod) if primary_mask is None else np.nonzero(np.asarray(primary_mask))[0]
        xs = sec.nodes[s_nodes]
        dist = np.linalg.norm(xs[:, None, :] - pri.nodes[p_cand][None, :, :], axis=2)
        p_nodes = p_cand[np.argmin(dist, axis=1)]
        sb = self.offsets[si] + s_nodes * sec.d
        pb = self.offsets[pi] + p_nodes * pri.d
        skew = self._skew(xs - pri.nodes[p_nodes])
        axes = (0, 1, 2) if self.dim == 3 else (2,)
        for dof in dofs:
            self.eliminated.append(sb + dof)
            self.rows.append((sb + dof, pb + dof, np.ones(len(sb))))
            if dof < self.dim and pri.d > self.dim:
                for b, axis in enumerate(axes):
                    self.rows.append((sb + dof, pb + self.dim + b, skew[:, dof, axis]))

    def elimination(self):
        eliminated = np.concatenate(self.eliminated) if self.eliminated else np.zeros(0, np.int64)
        keep = np.ones(self.n_dofs, dtype=bool)
        keep[eliminated] = False
        retained = np.nonzero(keep)[0]
        column = np.full(self.n_dofs, -1, dtype=np.int64)
        column[retained] = np.arange(len(retained))
        rows = [retained] + [r[0] for r in self.rows]
        cols = [column[retained]] + [column[r[1]] for r in self.rows]
        vals = [np.ones(len(retained))] + [r[2] for r in self.rows]
        T = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                          shape=(self.n_dofs, len(retained)))
        return T, retained

    def solve(self, method: str = "spsolve", rtol: float = 1e-12):
        """One linear load step [0, 1]: per part u and f."""
        T, retained = self.elimination()
        n = len(retained)
        blocks = [p.stiffness() if isinstance(p, ModelPart) else sp.csr_matrix((p.n_dofs, p.n_dofs))
                  for p in self.parts]
        K = sp.block_diag(blocks, format="csr")
        neumann = np.concatenate([p.forces.ravel() for p in self.parts])
        dirichlet = np.concatenate([p.displacements.ravel() for p in self.parts])
        constrained = np.concatenate([p.constraints.ravel() for p in self.parts])
        con = np.nonzero(constrained[retained])[0]
        free = np.ones(n)
        free[con] = 0.0
        Fr = sp.diags(free)
        Kr = (Fr @ (T.T @ K @ T) @ Fr + sp.diags(1.0 - free)).tocsr()
        DU = dirichlet[retained]
        q = np.zeros(n)
        q[con] = DU[con]
        res = T.T @ (K @ (T @ q) - neumann)
        res[con] = 0.0
        if method == "spsolve":
            dq = spla.spsolve(Kr.tocsc(), res)
        else:
            dinv = 1.0 / Kr.diagonal()
            self.cg_iterations = 0

            def tick(_):
                self.cg_iterations += 1

            dq, info = spla.cg(Kr, res, rtol=rtol, atol=0.0, maxiter=10 * n,
                               M=spla.LinearOperator(Kr.shape, matvec=lambda v: dinv * v), callback=tick)
            if info != 0:
                raise RuntimeError(f"CG did not converge ({info})")
        q = q - dq
        q[con] = DU[con]
        u = T @ q
        F_int = K @ u
        f = F_int.copy()
        f[retained] = T.T @ F_int
        out_u, out_f = [], []
        for p, off in zip(self.parts, self.offsets):
            out_u.append(u[off:off + p.n_dofs].reshape(p.n_nod, p.d))
            out_f.append(f[off:off + p.n_dofs].reshape(p.n_nod, p.d))
        return out_u, out_f
