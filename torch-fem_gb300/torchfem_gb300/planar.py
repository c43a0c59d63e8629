"""Planar continuum model (src/torchfem/planar.py:17-92, :306-322).

Element forces and stiffness carry the element thickness t_e as a factor
(planar.py:86-92), which the kernels apply per element.
"""

from __future__ import annotations

import torch
from torch import Tensor

from .base import Mechanics
from .elements import PLANAR_TYPES


class Planar(Mechanics):
    """Plane-stress / plane-strain model: Tria1, Quad1, Tria2 or Quad2."""

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
    def n_flux(self) -> list[int]:
        return [2, 2]

    @property
    def volume_scale(self) -> Tensor:
        return self.thickness

    def _thickness(self) -> Tensor | None:
        t = self.thickness
        if t.dim() == 0:
            t = t.expand(self.n_elem)
        return t

    def __repr__(self) -> str:
        return f"<torch-fem planar ({self.n_nod} nodes, {self.n_elem} {self.etype.__name__} elements)>"
