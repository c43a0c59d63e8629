"""Structured mesh generators.

`cube_hexa`, `rect_quad`, `cube_tetra` and `linear_to_quadratic` produce the
same node and element numbering as the reference (src/torchfem/mesh.py:8-135,
elements.py:1438-1494), because the numbering fixes the DOF numbering and so
the sparsity pattern.  `box_tetra6` (hexahedra split into six tetrahedra
around the main diagonal) and `plate_hole_ogrid` (an O-grid around a circular
hole) build the meshes of the hyperelastic and plasticity workloads; the
reference has no generator for either.
"""

from __future__ import annotations

import itertools
import math

import numpy as np
import torch
from torch import Tensor


def cube_hexa(Nx: int, Ny: int, Nz: int, Lx: float = 1.0, Ly: float = 1.0, Lz: float = 1.0):
    """Hexa1 grid with Nx x Ny x Nz nodes, x-major numbering (mesh.py:8-46)."""
    X = torch.linspace(0, Lx, Nx, dtype=torch.float64)
    Y = torch.linspace(0, Ly, Ny, dtype=torch.float64)
    Z = torch.linspace(0, Lz, Nz, dtype=torch.float64)
    x, y, z = torch.meshgrid(X, Y, Z, indexing="ij")
    nodes = torch.stack([x.ravel(), y.ravel(), z.ravel()], dim=1)
    ids = torch.arange(Nx * Ny * Nz).reshape(Nx, Ny, Nz)
    c = lambda i, j, k: ids[i : Nx - 1 + i, j : Ny - 1 + j, k : Nz - 1 + k].ravel()  # noqa: E731
    # reference node order of Hexa1: (000)(100)(110)(010)(001)(101)(111)(011)
    elements = torch.stack(
        [c(0, 0, 0), c(1, 0, 0), c(1, 1, 0), c(0, 1, 0), c(0, 0, 1), c(1, 0, 1), c(1, 1, 1), c(0, 1, 1)],
        dim=1,
    )
    return nodes, elements


def rect_quad(Nx: int, Ny: int, Lx: float = 1.0, Ly: float = 1.0):
    """Quad1 grid with Nx x Ny nodes (mesh.py:103-135)."""
    X = torch.linspace(0, Lx, Nx, dtype=torch.float64)
    Y = torch.linspace(0, Ly, Ny, dtype=torch.float64)
    x, y = torch.meshgrid(X, Y, indexing="ij")
    nodes = torch.stack([x.ravel(), y.ravel()], dim=1)
    ids = torch.arange(Nx * Ny).reshape(Nx, Ny)
    c = lambda i, j: ids[i : Nx - 1 + i, j : Ny - 1 + j].ravel()  # noqa: E731
    elements = torch.stack([c(0, 0), c(1, 0), c(1, 1), c(0, 1)], dim=1)
    return nodes, elements


def cube_tetra(Nx: int, Ny: int, Nz: int, Lx: float = 1.0, Ly: float = 1.0, Lz: float = 1.0):
    """Hexahedra split into five tetrahedra, alternating in a checkerboard
    (mesh.py:49-100): all even cells first, then all odd cells."""
    nodes, hexa = cube_hexa(Nx, Ny, Nz, Lx, Ly, Lz)
    I, J, K = torch.meshgrid(torch.arange(Nx - 1), torch.arange(Ny - 1), torch.arange(Nz - 1), indexing="ij")
    even = ((I + J + K) % 2 == 0).ravel()
    t_even = torch.tensor([[0, 1, 3, 4], [1, 2, 3, 6], [1, 3, 4, 6], [1, 4, 5, 6], [3, 4, 6, 7]])
    t_odd = torch.tensor([[4, 5, 0, 7], [5, 6, 2, 7], [5, 7, 2, 0], [5, 0, 2, 1], [7, 0, 3, 2]])
    tets = torch.cat([hexa[even][:, t_even].reshape(-1, 4), hexa[~even][:, t_odd].reshape(-1, 4)])
    return nodes, tets


_EDGES = {
    (3, 2): [[0, 1], [1, 2], [2, 0]],  # Tria1
    (4, 2): [[0, 1], [1, 2], [2, 3], [3, 0]],  # Quad1
    (4, 3): [[0, 1], [1, 2], [0, 2], [3, 0], [1, 3], [2, 3]],  # Tetra1
    (8, 3): [[0, 1], [1, 2], [2, 3], [3, 0], [4, 5], [5, 6], [6, 7], [7, 4],
             [0, 4], [1, 5], [2, 6], [3, 7]],  # Hexa1
}


def linear_to_quadratic(nodes: Tensor, elements: Tensor):
    """Mid-edge nodes appended to `nodes` (elements.py:1438-1494).

    Edges are (min, max) node pairs; distinct edges are numbered in the order
    of numpy's unique over their raw int64 bytes — the order of the
    reference's CPU branch — so mid-node ids match it node for node.
    """
    key = (elements.shape[1], nodes.shape[1])
    if key not in _EDGES:
        raise ValueError("The element type is not supported. Maybe the element is already quadratic?")
    edges = torch.tensor(_EDGES[key])
    pairs = elements[:, edges].reshape(-1, 2).to(torch.int64)
    pairs, _ = torch.sort(pairs, dim=1)
    raw = np.ascontiguousarray(pairs.cpu().numpy())
    as_bytes = raw.view(np.dtype((np.void, 16))).ravel()
    _, first, inverse = np.unique(as_bytes, return_index=True, return_inverse=True)
    uniq = pairs[torch.as_tensor(first)]
    mids = (nodes[uniq[:, 0]] + nodes[uniq[:, 1]]) / 2.0
    new_nodes = torch.cat([nodes, mids], dim=0)
    new_elements = torch.cat(
        [elements, torch.as_tensor(inverse.reshape(elements.shape[0], -1)) + nodes.shape[0]], dim=1
    )
    return new_nodes, new_elements


def box_tetra6(Nx: int, Ny: int, Nz: int, Lx: float = 1.0, Ly: float = 1.0, Lz: float = 1.0):
    """Each hexahedron of `cube_hexa` split into six tetrahedra sharing its
    main diagonal (local node 0 to node 6), one per ordering of the axes.
    Every tetrahedron is oriented so that its Jacobian is positive."""
    nodes, hexa = cube_hexa(Nx, Ny, Nz, Lx, Ly, Lz)
    corner = {(0, 0, 0): 0, (1, 0, 0): 1, (1, 1, 0): 2, (0, 1, 0): 3,
              (0, 0, 1): 4, (1, 0, 1): 5, (1, 1, 1): 6, (0, 1, 1): 7}
    tets = []
    for perm in itertools.permutations(range(3)):
        p = [0, 0, 0]
        path = [corner[tuple(p)]]
        for ax in perm:
            p[ax] = 1
            path.append(corner[tuple(p)])
        sign = np.linalg.det(np.eye(3)[list(perm)])
        if sign < 0:
            path[1], path[2] = path[2], path[1]
        tets.append(path)
    tets = torch.tensor(tets)
    return nodes, hexa[:, tets].reshape(-1, 4)


def plate_hole_ogrid(n_theta: int, n_rad: int, Lx: float = 2.0, Ly: float = 1.0, radius: float = 0.25):
    """Quad1 O-grid of a Lx x Ly plate with a centred circular hole.

    Angular index i in [0, n_theta) (periodic), radial index j in [0, n_rad]:
    node (i, j) lies on the segment from the hole point at angle
    theta_i = 2 pi i / n_theta to the point where the ray from the centre
    leaves the rectangle, at fraction j / n_rad.  Node id = i (n_rad + 1) + j.
    """
    cx, cy = Lx / 2.0, Ly / 2.0
    th = torch.arange(n_theta, dtype=torch.float64) * (2.0 * math.pi / n_theta)
    c, s = torch.cos(th), torch.sin(th)
    inner = torch.stack([cx + radius * c, cy + radius * s], dim=1)
    with torch.no_grad():
        tx = torch.where(c.abs() > 1e-15, (Lx / 2.0) / c.abs().clamp_min(1e-300), torch.full_like(c, math.inf))
        ty = torch.where(s.abs() > 1e-15, (Ly / 2.0) / s.abs().clamp_min(1e-300), torch.full_like(s, math.inf))
        t = torch.minimum(tx, ty)
    outer = torch.stack([cx + t * c, cy + t * s], dim=1)
    # snap the outer points onto the rectangle exactly
    outer[:, 0] = outer[:, 0].clamp(0.0, Lx)
    outer[:, 1] = outer[:, 1].clamp(0.0, Ly)
    outer[(tx <= ty), 0] = torch.where(c[(tx <= ty)] > 0, torch.tensor(Lx, dtype=torch.float64), torch.tensor(0.0, dtype=torch.float64))
    outer[(ty <= tx), 1] = torch.where(s[(ty <= tx)] > 0, torch.tensor(Ly, dtype=torch.float64), torch.tensor(0.0, dtype=torch.float64))
    f = torch.arange(n_rad + 1, dtype=torch.float64) / n_rad
    nodes = inner[:, None, :] * (1.0 - f)[None, :, None] + outer[:, None, :] * f[None, :, None]
    nodes = nodes.reshape(-1, 2)
    ids = torch.arange(n_theta * (n_rad + 1)).reshape(n_theta, n_rad + 1)
    nxt = torch.roll(ids, -1, dims=0)
    # counter-clockwise: (i, j) -> (i, j+1) -> (i+1, j+1) -> (i+1, j)
    elements = torch.stack(
        [ids[:, :-1], ids[:, 1:], nxt[:, 1:], nxt[:, :-1]], dim=-1
    ).reshape(-1, 4)
    return nodes, elements


def strip_tria(Nx: int, Ny: int, Lx: float = 1.0, Ly: float = 1.0):
    """Flat Tria1 strip in the z = 0 plane: an Nx x Ny node grid, each cell
    split along alternating diagonals.  Shell meshes (3D nodes)."""
    X = torch.linspace(0, Lx, Nx, dtype=torch.float64)
    Y = torch.linspace(0, Ly, Ny, dtype=torch.float64)
    x, y = torch.meshgrid(X, Y, indexing="ij")
    nodes = torch.stack([x.ravel(), y.ravel(), torch.zeros(Nx * Ny, dtype=torch.float64)], dim=1)
    return nodes, _grid_triangles(Nx, Ny)


def cylinder_patch_tria(n_arc: int, n_len: int, radius: float = 1.0, length: float = 2.0,
                        angle: float = 80.0):
    """Tria1 mesh of a cylindrical roof: the cylinder's axis is y, the arc
    spans +-angle/2 degrees about the z axis (apex at z = radius), n_arc x
    n_len nodes, each cell split along alternating diagonals."""
    half = math.radians(angle) / 2.0
    th = torch.linspace(-half, half, n_arc, dtype=torch.float64)
    Y = torch.linspace(0.0, length, n_len, dtype=torch.float64)
    t, y = torch.meshgrid(th, Y, indexing="ij")
    nodes = torch.stack([radius * torch.sin(t).ravel(), y.ravel(), radius * torch.cos(t).ravel()], dim=1)
    return nodes, _grid_triangles(n_arc, n_len)


def _grid_triangles(Nx: int, Ny: int) -> Tensor:
    """Counter-clockwise triangles of an Nx x Ny node grid (node i * Ny + j)."""
    tris = []
    for i in range(Nx - 1):
        for j in range(Ny - 1):
            a, b, c, d = i * Ny + j, (i + 1) * Ny + j, (i + 1) * Ny + j + 1, i * Ny + j + 1
            if (i + j) % 2 == 0:
                tris += [(a, b, c), (a, c, d)]
            else:
                tris += [(a, b, d), (b, c, d)]
    return torch.tensor(tris, dtype=torch.int64)
