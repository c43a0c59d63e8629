"""GB300-native forward + adjoint path of torch-fem.

Drop-in for `Solid(...)` / `Planar(...)` / `Shell(...)` / `SolidHeat(...)` /
`PlanarHeat(...)` / `Assembly(...)` and `model.solve(..., differentiable_parameters=...)` of
torch-fem; the compute runs in hand-written
sm_103a CUDA kernels reached through the C ABI of ``include/torchfem_gb300.h``.
"""

from .assembly import Assembly, ReferencePoint, ReferencePointHeat
from .planar import Planar, PlanarHeat
from .shell import Shell
from .solid import Solid, SolidHeat

__all__ = ["Assembly", "Planar", "PlanarHeat", "ReferencePoint", "ReferencePointHeat", "Shell", "Solid",
           "SolidHeat"]
