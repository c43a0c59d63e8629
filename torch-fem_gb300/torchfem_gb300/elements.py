"""Isoparametric element tables (src/torchfem/elements.py).

Each element type provides its shape functions ``N(xi)``, their reference
gradients ``B(xi)`` with shape ``[..., iso_dim, nodes]``, integration points
and weights, exactly as the reference defines them (same constants, including
Tetra2's 8-digit points and ``0.041666667`` weights, elements.py:920-933, and
Quad1's integer weights, elements.py:555-557).  The GPU kernels receive the
gradient table ``B(ipoints)`` and the weights; they do not hard-code a rule.
"""

from __future__ import annotations

from math import sqrt

import torch
from torch import Tensor

from . import _lib


def _f64(rows) -> Tensor:
    return torch.tensor(rows, dtype=torch.float64)


class Element:
    """Base class: subclasses set the tables below."""

    nodes: int
    iso_dim: int
    etype_id: int

    @classmethod
    def N(cls, xi: Tensor) -> Tensor:
        raise NotImplementedError

    @classmethod
    def B(cls, xi: Tensor) -> Tensor:
        raise NotImplementedError

    @classmethod
    def ipoints(cls) -> Tensor:
        raise NotImplementedError

    @classmethod
    def iweights(cls) -> Tensor:
        raise NotImplementedError

    @classmethod
    def gradient_table(cls) -> Tensor:
        """``B`` at every integration point, float64 ``[nip, iso_dim, nodes]``."""
        return cls.B(cls.ipoints().to(torch.float64)).to(torch.float64).reshape(
            -1, cls.iso_dim, cls.nodes
        )


class Quad1(Element):
    """Four-node bilinear quadrilateral (elements.py:491-567)."""

    nodes, iso_dim, etype_id = 4, 2, _lib.FEM_QUAD1

    @classmethod
    def N(cls, xi):
        x, y = xi[..., 0], xi[..., 1]
        return 0.25 * torch.stack(
            [(1.0 - x) * (1.0 - y), (1.0 + x) * (1.0 - y), (1.0 + x) * (1.0 + y), (1.0 - x) * (1.0 + y)],
            dim=-1,
        )

    @classmethod
    def B(cls, xi):
        x, y = xi[..., 0], xi[..., 1]
        dx = torch.stack([-(1 - y), (1 - y), (1.0 + y), -(1.0 + y)], dim=-1)
        dy = torch.stack([-(1 - x), -(1 + x), (1.0 + x), (1.0 - x)], dim=-1)
        return 0.25 * torch.stack([dx, dy], dim=-2)

    @classmethod
    def ipoints(cls):
        s = 1.0 / sqrt(3.0)
        return _f64([[a * s, b * s] for b in (-1, 1) for a in (-1, 1)])

    @classmethod
    def iweights(cls):
        return torch.tensor([1, 1, 1, 1])


class Quad2(Quad1):
    """Eight-node serendipity quadrilateral with a 2x2 rule (elements.py:570-724)."""

    nodes, etype_id = 8, _lib.FEM_QUAD2

    @classmethod
    def N(cls, xi):
        x, y = xi[..., 0], xi[..., 1]
        return 0.25 * torch.stack(
            [
                -(1 - x) * (1 - y) * (1 + x + y),
                -(1 + x) * (1 - y) * (1 - x + y),
                -(1 + x) * (1 + y) * (1 - x - y),
                -(1 - x) * (1 + y) * (1 + x - y),
                2 * (1 - x) * (1 - y) * (1 + x),
                2 * (1 + x) * (1 - y) * (1 + y),
                2 * (1 - x) * (1 + y) * (1 + x),
                2 * (1 - x) * (1 - y) * (1 + y),
            ],
            dim=-1,
        )

    @classmethod
    def B(cls, xi):
        x, y = xi[..., 0], xi[..., 1]
        dx = torch.stack(
            [
                -(y - 1) * (2 * x + y),
                -(y - 1) * (2 * x - y),
                +(y + 1) * (2 * x + y),
                +(y + 1) * (2 * x - y),
                +4 * x * (y - 1),
                +2 - 2 * y**2,
                -4 * x * (y + 1),
                -2 + 2 * y**2,
            ],
            dim=-1,
        )
        dy = torch.stack(
            [
                -(x - 1) * (x + 2 * y),
                -(x + 1) * (x - 2 * y),
                +(x + 1) * (x + 2 * y),
                +(x - 1) * (x - 2 * y),
                -2 + 2 * x**2,
                -4 * y * (x + 1),
                +2 - 2 * x**2,
                +4 * (x - 1) * y,
            ],
            dim=-1,
        )
        return 0.25 * torch.stack([dx, dy], dim=-2)


class Tria1(Element):
    """Three-node linear triangle (elements.py:309-382)."""

    nodes, iso_dim, etype_id = 3, 2, _lib.FEM_TRIA1

    @classmethod
    def N(cls, xi):
        x, y = xi[..., 0], xi[..., 1]
        return torch.stack([1.0 - x - y, x, y], dim=-1)

    @classmethod
    def B(cls, xi):
        base = _f64([[-1.0, 1.0, 0.0], [-1.0, 0.0, 1.0]])
        return base.expand(*xi.shape[:-1], 2, 3).clone()

    @classmethod
    def ipoints(cls):
        return _f64([[1.0 / 3.0, 1.0 / 3.0]])

    @classmethod
    def iweights(cls):
        return _f64([0.5])


class Tria2(Tria1):
    """Six-node quadratic triangle (elements.py:385-488)."""

    nodes, etype_id = 6, _lib.FEM_TRIA2

    @classmethod
    def N(cls, xi):
        x, y = xi[..., 0], xi[..., 1]
        return torch.stack(
            [
                (1 - x - y) * (1 - 2 * x - 2 * y),
                x * (2 * x - 1),
                y * (2 * y - 1),
                4 * x * (1 - x - y),
                4 * x * y,
                4 * y * (1 - x - y),
            ],
            dim=-1,
        )

    @classmethod
    def B(cls, xi):
        x, y = xi[..., 0], xi[..., 1]
        z = torch.zeros_like(x)
        dx = torch.stack([4 * x + 4 * y - 3, 4 * x - 1, z, -4 * (2 * x + y - 1), 4 * y, -4 * y], dim=-1)
        dy = torch.stack([4 * x + 4 * y - 3, z, 4 * y - 1, -4 * x, 4 * x, -4 * (x + 2 * y - 1)], dim=-1)
        return torch.stack([dx, dy], dim=-2)

    @classmethod
    def ipoints(cls):
        return _f64([[0.5, 0.5], [0.5, 0.0], [0.0, 0.5]])

    @classmethod
    def iweights(cls):
        return _f64([1.0 / 6.0, 1.0 / 6.0, 1.0 / 6.0])


class Tetra1(Element):
    """Four-node linear tetrahedron (elements.py:727-790)."""

    nodes, iso_dim, etype_id = 4, 3, _lib.FEM_TETRA1

    @classmethod
    def N(cls, xi):
        x, y, z = xi[..., 0], xi[..., 1], xi[..., 2]
        return torch.stack([1.0 - x - y - z, x, y, z], dim=-1)

    @classmethod
    def B(cls, xi):
        base = _f64([[-1.0, 1.0, 0.0, 0.0], [-1.0, 0.0, 1.0, 0.0], [-1.0, 0.0, 0.0, 1.0]])
        return base.expand(*xi.shape[:-1], 3, 4).clone()

    @classmethod
    def ipoints(cls):
        return _f64([[0.25, 0.25, 0.25]])

    @classmethod
    def iweights(cls):
        return _f64([1.0 / 6.0])


class Tetra2(Tetra1):
    """Ten-node quadratic tetrahedron (elements.py:793-933)."""

    nodes, etype_id = 10, _lib.FEM_TETRA2

    @classmethod
    def N(cls, xi):
        x, y, z = xi[..., 0], xi[..., 1], xi[..., 2]
        w = 1.0 - x - y - z
        return torch.stack(
            [w * (2 * w - 1), x * (2 * x - 1), y * (2 * y - 1), z * (2 * z - 1), 4 * x * w,
             4 * x * y, 4 * y * w, 4 * z * w, 4 * x * z, 4 * y * z],
            dim=-1,
        )

    @classmethod
    def B(cls, xi):
        x, y, z = xi[..., 0], xi[..., 1], xi[..., 2]
        o = torch.zeros_like(x)
        c = 4 * (x + y + z) - 3
        dx = torch.stack([c, 4 * x - 1, o, o, -4 * (2 * x + y + z - 1), 4 * y, -4 * y, -4 * z, 4 * z, o], dim=-1)
        dy = torch.stack([c, o, 4 * y - 1, o, -4 * x, 4 * x, -4 * (x + 2 * y + z - 1), -4 * z, o, 4 * z], dim=-1)
        dz = torch.stack([c, o, o, 4 * z - 1, -4 * x, o, -4 * y, -4 * (x + y + 2 * z - 1), 4 * x, 4 * y], dim=-1)
        return torch.stack([dx, dy, dz], dim=-2)

    @classmethod
    def ipoints(cls):
        return _f64(
            [
                [0.58541020, 0.13819660, 0.13819660],
                [0.13819660, 0.58541020, 0.13819660],
                [0.13819660, 0.13819660, 0.58541020],
                [0.13819660, 0.13819660, 0.13819660],
            ]
        )

    @classmethod
    def iweights(cls):
        return _f64([0.041666667, 0.041666667, 0.041666667, 0.041666667])


class Hexa1(Element):
    """Eight-node trilinear hexahedron (elements.py:936-1075)."""

    nodes, iso_dim, etype_id = 8, 3, _lib.FEM_HEXA1

    # local node signs (xi_1, xi_2, xi_3) in the reference node order
    _SIGNS = ((-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1),
              (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1))

    @classmethod
    def N(cls, xi):
        x, y, z = xi[..., 0], xi[..., 1], xi[..., 2]
        return 0.125 * torch.stack(
            [(1.0 + sx * x) * (1.0 + sy * y) * (1.0 + sz * z) for sx, sy, sz in cls._SIGNS], dim=-1
        )

    @classmethod
    def B(cls, xi):
        x, y, z = xi[..., 0], xi[..., 1], xi[..., 2]
        dx = [sx * (1.0 + sy * y) * (1.0 + sz * z) for sx, sy, sz in cls._SIGNS]
        dy = [sy * (1.0 + sx * x) * (1.0 + sz * z) for sx, sy, sz in cls._SIGNS]
        dz = [sz * (1.0 + sx * x) * (1.0 + sy * y) for sx, sy, sz in cls._SIGNS]
        return 0.125 * torch.stack(
            [torch.stack(dx, dim=-1), torch.stack(dy, dim=-1), torch.stack(dz, dim=-1)], dim=-2
        )

    @classmethod
    def ipoints(cls):
        s = 1.0 / sqrt(3.0)
        return _f64([[a * s, b * s, c * s] for c in (-1.0, 1.0) for b in (-1.0, 1.0) for a in (-1.0, 1.0)])

    @classmethod
    def iweights(cls):
        return _f64([1.0] * 8)


class Hexa2(Element):
    """Twenty-node serendipity hexahedron with the 2 x 2 x 2 rule of Hexa1
    (elements.py:1078-1406): corner functions
    (1 + s1 x)(1 + s2 y)(1 + s3 z)(s1 x + s2 y + s3 z - 2) / 8, mid-edge
    functions (1 - t^2)(1 + s y)(1 + s' z) / 4 with t the coordinate along
    the edge."""

    nodes, iso_dim, etype_id = 20, 3, _lib.FEM_HEXA2

    # iso coordinates of the 8 corners and the 12 mid-edge nodes, reference order
    _COORDS = Hexa1._SIGNS + ((0, -1, -1), (1, 0, -1), (0, 1, -1), (-1, 0, -1),
                              (0, -1, 1), (1, 0, 1), (0, 1, 1), (-1, 0, 1),
                              (-1, -1, 0), (1, -1, 0), (1, 1, 0), (-1, 1, 0))

    @classmethod
    def _terms(cls, xi):
        x, y, z = xi[..., 0], xi[..., 1], xi[..., 2]
        N, dx, dy, dz = [], [], [], []
        for sx, sy, sz in cls._COORDS:
            if sx and sy and sz:
                a, b, c = 1.0 + sx * x, 1.0 + sy * y, 1.0 + sz * z
                g = sx * x + sy * y + sz * z - 2.0
                N.append(0.125 * a * b * c * g)
                dx.append(0.125 * sx * b * c * (g + a))
                dy.append(0.125 * sy * a * c * (g + b))
                dz.append(0.125 * sz * a * b * (g + c))
            elif sx == 0:
                b, c = 1.0 + sy * y, 1.0 + sz * z
                N.append(0.25 * (1.0 - x * x) * b * c)
                dx.append(-0.5 * x * b * c)
                dy.append(0.25 * (1.0 - x * x) * sy * c)
                dz.append(0.25 * (1.0 - x * x) * b * sz)
            elif sy == 0:
                a, c = 1.0 + sx * x, 1.0 + sz * z
                N.append(0.25 * a * (1.0 - y * y) * c)
                dx.append(0.25 * sx * (1.0 - y * y) * c)
                dy.append(-0.5 * y * a * c)
                dz.append(0.25 * a * (1.0 - y * y) * sz)
            else:
                a, b = 1.0 + sx * x, 1.0 + sy * y
                N.append(0.25 * a * b * (1.0 - z * z))
                dx.append(0.25 * sx * b * (1.0 - z * z))
                dy.append(0.25 * a * sy * (1.0 - z * z))
                dz.append(-0.5 * z * a * b)
        return N, dx, dy, dz

    @classmethod
    def N(cls, xi):
        return torch.stack(cls._terms(xi)[0], dim=-1)

    @classmethod
    def B(cls, xi):
        _, dx, dy, dz = cls._terms(xi)
        return torch.stack([torch.stack(dx, dim=-1), torch.stack(dy, dim=-1), torch.stack(dz, dim=-1)], dim=-2)

    @classmethod
    def ipoints(cls):
        return Hexa1.ipoints()

    @classmethod
    def iweights(cls):
        return _f64([1.0] * 8)


SOLID_TYPES = {4: Tetra1, 8: Hexa1, 10: Tetra2, 20: Hexa2}
PLANAR_TYPES = {3: Tria1, 4: Quad1, 6: Tria2, 8: Quad2}
