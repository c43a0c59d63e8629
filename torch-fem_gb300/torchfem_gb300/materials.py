"""Material models with the reference's interface (src/torchfem/materials).

Each material keeps the reference attributes (``n_state``, ``is_vectorized``,
``rho``, the elastic constants and ``C``), ``vectorize(n_elem)`` and
``step(H_inc, F, stress, state, de0, cl, iter)`` (materials/base.py:10-103).
``step`` is written with torch ops and is the per-point definition of the
material; the GPU kernels do not call it.  They consume the material through
``kernel_data(n_elem)``, which returns the layout code and a per-element
tensor derived from the constants with differentiable torch ops, so the
hand-written adjoint's gradient for that tensor flows back to whatever the
user built the constants from (E, rho, ...).
"""

from __future__ import annotations

import copy

import torch
from torch import Tensor

from . import _lib


class Material:
    """Base class (materials/base.py:10-46)."""

    def __init__(self):
        self.n_state: int = 0
        self.is_vectorized: bool = False
        self.rho: Tensor = torch.tensor(1.0)

    def vectorize(self, n_elem: int) -> "Material":
        """The material batched over `n_elem` elements (base.py:29-46)."""
        if self.is_vectorized:
            return self
        new = copy.copy(self)
        for key, value in list(vars(new).items()):
            if isinstance(value, Tensor):
                setattr(new, key, value.repeat(n_elem, *(value.dim() * [1])))
        new.is_vectorized = True
        return new

    def step(self, H_inc, F, stress, state, de0, cl, iter):
        raise NotImplementedError

    def rotate(self, R: Tensor) -> "Material":
        return self

    def kernel_data(self, n_elem: int) -> tuple[int, Tensor]:
        raise NotImplementedError(f"{type(self).__name__} has no GPU kernel in torchfem_gb300")


def _iso_or_general(C: Tensor, n_elem: int, d: int) -> tuple[int, Tensor]:
    """ISO (lambda, G) per element when C has the isotropic form, else C.

    Both are computed from C by indexing, so autograd links them to C.
    """
    Cb = C if C.dim() > 4 else C.unsqueeze(0)
    lam = Cb[..., 0, 0, 1, 1]
    G = Cb[..., 0, 1, 0, 1]
    with torch.no_grad():
        eye = torch.eye(d, dtype=C.dtype, device=C.device)
        i4 = torch.einsum("ij,kl->ijkl", eye, eye)
        i4s = torch.einsum("ik,jl->ijkl", eye, eye) + torch.einsum("il,jk->ijkl", eye, eye)
        rec = lam[..., None, None, None, None] * i4 + G[..., None, None, None, None] * i4s
        iso = bool(torch.allclose(rec, Cb, rtol=1e-14, atol=0.0))
    if iso:
        data = torch.stack([lam, G], dim=-1).to(torch.float64)
        if data.shape[0] != n_elem:
            data = data.expand(n_elem, 2)
        return _lib.FEM_MAT_ISO, data.contiguous()
    flat = Cb.reshape(Cb.shape[0], d**4).to(torch.float64)
    if flat.shape[0] != n_elem:
        flat = flat.expand(n_elem, d**4)
    return _lib.FEM_MAT_GENERAL, flat.contiguous()


class IsotropicElasticity3D(Material):
    """Isotropic linear elasticity in 3D (materials/elasticity.py:12-127).

    lambda = E nu / ((1 + nu)(1 - 2 nu)), G = E / (2 (1 + nu)),
    C = lambda I (x) I + G (d_ik d_jl + d_il d_jk).
    """

    def __init__(self, E, nu, rho=1.0):
        self.E = torch.as_tensor(E)
        self.nu = torch.as_tensor(nu)
        self.rho = torch.as_tensor(rho)
        self.n_state = 0
        self.is_vectorized = self.E.dim() > 0
        self.lbd = self.E * self.nu / ((1.0 + self.nu) * (1.0 - 2.0 * self.nu))
        self.G = self.E / (2.0 * (1.0 + self.nu))
        eye = torch.eye(3)
        i4 = torch.einsum("ij,kl->ijkl", eye, eye)
        i4s = torch.einsum("ik,jl->ijkl", eye, eye) + torch.einsum("il,jk->ijkl", eye, eye)
        self.C = self.lbd[..., None, None, None, None] * i4 + self.G[..., None, None, None, None] * i4s

    def step(self, H_inc, F, stress, state, de0, cl, iter):
        """sigma_new = sigma + C : (sym(H_inc) - de0); tangent C (elasticity.py:119-127)."""
        de = 0.5 * (H_inc.transpose(-1, -2) + H_inc)
        stress_new = stress + torch.einsum("...ijkl,...kl->...ij", self.C, de - de0)
        return stress_new, state, self.C

    def kernel_data(self, n_elem: int) -> tuple[int, Tensor]:
        return _iso_or_general(self.C, n_elem, self.C.shape[-1])


class IsotropicElasticityPlaneStress(IsotropicElasticity3D):
    """Plane stress (elasticity.py:130-182): C0000 = C1111 = E/(1-nu^2),
    C0011 = C1100 = E nu/(1-nu^2), C0101 = C0110 = C1001 = C1010 = E/(2(1+nu))."""

    def __init__(self, E, nu, rho=1.0):
        super().__init__(E, nu, rho)
        fac = self.E / (1.0 - self.nu**2)
        shear = fac * 0.5 * (1.0 - self.nu)
        self.C = _planar_c(fac, fac * self.nu, shear, self.E)


class IsotropicElasticityPlaneStrain(IsotropicElasticity3D):
    """Plane strain (elasticity.py:185-241): C0000 = C1111 = 2G + lambda,
    C0011 = C1100 = lambda, shear terms G."""

    def __init__(self, E, nu, rho=1.0):
        super().__init__(E, nu, rho)
        self.C = _planar_c(2.0 * self.G + self.lbd, self.lbd, self.G, self.E)


def _planar_c(c_diag: Tensor, c_off: Tensor, c_shear: Tensor, E: Tensor) -> Tensor:
    """2x2x2x2 tensor from its three distinct entries (differentiable)."""
    z = torch.zeros_like(c_diag)
    rows = [
        # (0,0,0,0) (0,0,0,1) (0,0,1,0) (0,0,1,1)
        c_diag, z, z, c_off,
        # (0,1,0,0) (0,1,0,1) (0,1,1,0) (0,1,1,1)
        z, c_shear, c_shear, z,
        # (1,0,0,0) (1,0,0,1) (1,0,1,0) (1,0,1,1)
        z, c_shear, c_shear, z,
        # (1,1,0,0) (1,1,0,1) (1,1,1,0) (1,1,1,1)
        c_off, z, z, c_diag,
    ]
    return torch.stack(rows, dim=-1).reshape(*E.shape, 2, 2, 2, 2)
