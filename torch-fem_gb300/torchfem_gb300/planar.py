"""Planar continuum models (src/torchfem/planar.py:17-96, :306-340).

Element forces, stiffness and capacity carry the element thickness t_e as a
factor (planar.py:86-96), which the kernels apply per element.
"""

from __future__ import annotations

import torch
from torch import Tensor

from .base import FEM, Heat, Mechanics
from .elements import PLANAR_TYPES


class PlanarGeometry(FEM):
    """Tria1, Quad1, Tria2 or Quad2 connectivity with a thickness per element."""

    def __init__(self, nodes: Tensor, elements: Tensor, material, thickness: Tensor | float = 1.0):
        super().__init__(nodes, elements, material)
        if isinstance(thickness, float):
            self.thickness = torch.full((self.n_elem,), thickness, dtype=nodes.dtype, device=nodes.device)
        else:
            self.thickness = torch.as_tensor(thickness)

    @property
    def etype(self):
        n = len(self.elements[0])
        if n not in PLANAR_TYPES:
            raise ValueError("Element type not supported.")
        return PLANAR_TYPES[n]

    @property
    def volume_scale(self) -> Tensor:
        return self.thickness

    def _thickness(self) -> Tensor | None:
        t = self.thickness
        if t.dim() == 0:
            t = t.expand(self.n_elem)
        return t


class Planar(PlanarGeometry, Mechanics):
    """Plane-stress / plane-strain model (planar.py:306-322)."""

    @property
    def n_flux(self) -> list[int]:
        return [2, 2]

    def __repr__(self) -> str:
        return f"<torch-fem planar ({self.n_nod} nodes, {self.n_elem} {self.etype.__name__} elements)>"


class PlanarHeat(PlanarGeometry, Heat):
    """Planar heat conduction model: one temperature per node (planar.py:325-339)."""

    def __repr__(self) -> str:
        return f"<torch-fem planar heat ({self.n_nod} nodes, {self.n_elem} {self.etype.__name__} elements)>"
