"""The allocation-free CG entry point, fem_pcg_static.

Some callers cannot allocate device memory where they solve (a host behind
an FFI with no CUDA allocator binding, or a control loop that cannot accept
cudaMalloc's implicit synchronisation or its failure under memory pressure).
fem_pcg_static serves them from a static device array.  This test calls it
through the C ABI twice in a row and checks each result against fem_pcg,
which uses a caller-provided workspace, on the same assembled system.  The
file name makes pytest collect it last.
"""

import ctypes as C

import pytest
import torch

from torchfem_gb300 import Planar, Solid, _lib, mesh
from torchfem_gb300.materials import IsotropicElasticity3D, IsotropicElasticityPlaneStress

pytestmark = pytest.mark.gpu


def _system(cuda, kind="fp64"):
    """An assembled system through the public model API: the FP64 CSR matrix
    with Jacobi ("fp64"), or the FP32 sliced block matrix with its
    block-Jacobi inverse in 3D ("fp32-3d", block 3) and in plane stress
    ("fp32-2d", block 2)."""
    if kind == "fp32-2d":
        nodes, el = mesh.rect_quad(41, 21, 2.0, 1.0)
        m = Planar(nodes, el, IsotropicElasticityPlaneStress(1000.0, 0.3))
    else:
        nodes, el = mesh.cube_hexa(9, 9, 9)
        gen = torch.Generator().manual_seed(0)
        inner = ((nodes > 0) & (nodes < 1)).all(1)
        nodes = nodes + inner[:, None] * (torch.rand(nodes.shape, generator=gen) * 2 - 1) * 0.01
        m = Solid(nodes, el, IsotropicElasticity3D(1000.0, 0.3))
    m.constraints[nodes[:, 0] == 0.0, :] = True
    dm = m.device_mesh
    mkind, data = m.material.kernel_data(m.n_elem)
    data = data.to(cuda).contiguous()
    th = m._thickness()
    th = None if th is None else th.to(cuda, torch.float64).contiguous()
    mesh_s = dm.make_mesh(th)
    mat = _lib.FemMaterial(mkind, data.data_ptr())
    con = m.constraints.reshape(-1).to(cuda, torch.uint8).contiguous()
    precision = "fp64" if kind == "fp64" else "mixed"
    sysm = dm.build_system(mesh_s, mat, con, precision, keep_refs=(data, mesh_s, mat, th), precond="jacobi")
    return dm, sysm, con


def _solve_existing(dm, sysm, b, rtol):
    x = torch.empty_like(b)
    info = _lib.FemSolveInfo()
    ws = torch.empty(dm.lib.fem_pcg_workspace_bytes(C.byref(sysm.matrix)), dtype=torch.uint8, device=b.device)
    rc = dm.lib.fem_pcg(C.byref(sysm.matrix), b.data_ptr(), x.data_ptr(), rtol, 10 * b.numel(),
                        ws.data_ptr(), ws.numel(), C.byref(info), dm.stream)
    assert rc == 0, dm.lib.fem_last_error()
    return x, info


def _solve_static(dm, sysm, b, rtol):
    x = torch.full_like(b, float("nan"))
    info = _lib.FemSolveInfo()
    rc = dm.lib.fem_pcg_static(C.byref(sysm.matrix), b.data_ptr(), x.data_ptr(), rtol, 10 * b.numel(),
                               C.byref(info), dm.stream)
    assert rc == 0, dm.lib.fem_last_error()
    return x, info


@pytest.mark.parametrize("kind", ["fp64", "fp32-3d", "fp32-2d"])
def test_static_workspace_solve_matches_workspace_solve_twice(cuda, kind):
    """Both entry points run the same iteration on the same system, so the
    iteration counts are equal and the solutions agree to 1e-12 relative,
    on two calls in a row (the second reuses the array the first left).
    The FP32 sliced formats exercise the array's FP32 vectors and the
    unit-norm scaling of the right-hand side."""
    dm, sysm, con = _system(cuda, kind)
    assert dm.n_dofs <= dm.lib.fem_pcg_static_max_unknowns()
    rtol = 1e-12 if kind == "fp64" else 1e-6
    gen = torch.Generator(device=cuda).manual_seed(1)
    for call in range(2):
        b = torch.randn(dm.n_dofs, dtype=torch.float64, device=cuda, generator=gen)
        b[con.bool()] = 0.0
        x_ref, info_ref = _solve_existing(dm, sysm, b, rtol)
        x, info = _solve_static(dm, sysm, b, rtol)
        torch.cuda.synchronize()
        assert info.iterations == info_ref.iterations > 0, call
        err = float((x - x_ref).abs().max() / x_ref.abs().max())
        assert err <= 1e-12, (call, err)


def test_static_workspace_rejects_oversized_systems(cuda):
    dm, sysm, con = _system(cuda)
    big = _lib.FemMatrix(sysm.matrix.format, sysm.matrix.block, dm.lib.fem_pcg_static_max_unknowns() + 1,
                         dm.lib.fem_pcg_static_max_unknowns() + 1, sysm.matrix.row_ptr, sysm.matrix.col,
                         sysm.matrix.val, sysm.matrix.precond)
    info = _lib.FemSolveInfo()
    rc = dm.lib.fem_pcg_static(C.byref(big), None, None, 1e-12, 10, C.byref(info), dm.stream)
    assert rc == _lib.FEM_BOUNDS
    assert b"unknowns exceed the static workspace limit" in dm.lib.fem_last_error()
