"""GB300-native forward + adjoint path of torch-fem.

Drop-in for `Solid(...)` / `Planar(...)` / `Shell(...)` and `model.solve(...,
differentiable_parameters=...)` of torch-fem; the compute runs in hand-written
sm_103a CUDA kernels reached through the C ABI of ``include/torchfem_gb300.h``.
"""

from .planar import Planar
from .shell import Shell
from .solid import Solid

__all__ = ["Planar", "Shell", "Solid"]
