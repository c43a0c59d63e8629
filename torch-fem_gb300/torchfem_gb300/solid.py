"""Three-dimensional continuum models (src/torchfem/solid.py:15-62, :240-270)."""

from __future__ import annotations

from .base import FEM, Heat, Mechanics
from .elements import SOLID_TYPES


class SolidGeometry(FEM):
    """Hexa1, Hexa2, Tetra1 or Tetra2 connectivity, picked by the number of
    nodes per element (solid.py:32-44).  Plotting is not part of this
    library."""

    @property
    def etype(self):
        n = len(self.elements[0])
        if n not in SOLID_TYPES:
            raise ValueError("Element type not supported.")
        return SOLID_TYPES[n]


class Solid(SolidGeometry, Mechanics):
    """Solid mechanics model (solid.py:240-255)."""

    @property
    def n_flux(self) -> list[int]:
        return [3, 3]

    def __repr__(self) -> str:
        return f"<torch-fem solid ({self.n_nod} nodes, {self.n_elem} {self.etype.__name__} elements)>"


class SolidHeat(SolidGeometry, Heat):
    """Solid heat conduction model: one temperature per node (solid.py:258-270)."""

    def __repr__(self) -> str:
        return f"<torch-fem solid heat ({self.n_nod} nodes, {self.n_elem} {self.etype.__name__} elements)>"
