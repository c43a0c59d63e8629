"""GB300-native forward + adjoint path of torch-fem.

Drop-in for `Solid(...)` / `Planar(...)` / `Shell(...)` / `SolidHeat(...)` /
`PlanarHeat(...)` and `model.solve(..., differentiable_parameters=...)` of
torch-fem; the compute runs in hand-written
sm_103a CUDA kernels reached through the C ABI of ``include/torchfem_gb300.h``.
"""

from .planar import Planar, PlanarHeat
from .shell import Shell
from .solid import Solid, SolidHeat

__all__ = ["Planar", "PlanarHeat", "Shell", "Solid", "SolidHeat"]
