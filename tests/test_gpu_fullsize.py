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
