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
from collections import OrderedDict

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


# isotropy decisions per stiffness tensor, valid while the tensor is unchanged
# (same object, same in-place version counter); the tensor is held so that
# its id cannot be reused by another tensor while the entry lives
_ISO_CACHE: "OrderedDict[int, tuple[Tensor, int, bool]]" = OrderedDict()
_ISO_CACHE_SIZE = 8


def _is_isotropic(Cb: Tensor, lam: Tensor, G: Tensor, d: int) -> bool:
    hit = _ISO_CACHE.get(id(Cb))
    if hit is not None and hit[0] is Cb and hit[1] == Cb._version:
        _ISO_CACHE.move_to_end(id(Cb))
        return hit[2]
    with torch.no_grad():
        eye = torch.eye(d, dtype=Cb.dtype, device=Cb.device)
        i4 = torch.einsum("ij,kl->ijkl", eye, eye)
        i4s = torch.einsum("ik,jl->ijkl", eye, eye) + torch.einsum("il,jk->ijkl", eye, eye)
        rec = lam[..., None, None, None, None] * i4 + G[..., None, None, None, None] * i4s
        iso = bool(torch.allclose(rec, Cb, rtol=1e-14, atol=0.0))
    _ISO_CACHE[id(Cb)] = (Cb, Cb._version, iso)
    if len(_ISO_CACHE) > _ISO_CACHE_SIZE:
        _ISO_CACHE.popitem(last=False)
    return iso


def _is_isotropic_small(Cb: Tensor, lam: Tensor, G: Tensor, d: int) -> bool:
    with torch.no_grad():
        eye = torch.eye(d, dtype=Cb.dtype, device=Cb.device)
        i4 = torch.einsum("ij,kl->ijkl", eye, eye)
        i4s = torch.einsum("ik,jl->ijkl", eye, eye) + torch.einsum("il,jk->ijkl", eye, eye)
        rec = lam[..., None, None, None, None] * i4 + G[..., None, None, None, None] * i4s
        return bool(torch.allclose(rec, Cb, rtol=1e-14, atol=0.0))


def _iso_or_general(C: Tensor, n_elem: int, d: int) -> tuple[int, Tensor]:
    """ISO (lambda, G) per element when C has the isotropic form, else C.

    Both are computed from C by indexing, so autograd links them to C.  The
    isotropy test (a full comparison of C) runs once per stiffness tensor and
    is reused while the tensor is not modified.
    """
    Cb = C if C.dim() > 4 else C.unsqueeze(0)
    lam = Cb[..., 0, 0, 1, 1]
    G = Cb[..., 0, 1, 0, 1]
    iso = _is_isotropic(C, lam, G, d) if C.dim() > 4 else _is_isotropic_small(Cb, lam, G, d)
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
        self.nu = torch.as_tensor(nu, device=self.E.device)
        self.rho = torch.as_tensor(rho)
        self.n_state = 0
        self.is_vectorized = self.E.dim() > 0
        self.lbd = self.E * self.nu / ((1.0 + self.nu) * (1.0 - 2.0 * self.nu))
        self.G = self.E / (2.0 * (1.0 + self.nu))
        eye = torch.eye(3, dtype=self.lbd.dtype, device=self.lbd.device)
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


# ------------------------------------------------------------ finite strain ---
def neo_hookean_psi(F: Tensor, params: Tensor) -> Tensor:
    """Neo-Hookean energy with params = (mu, lambda):
    psi = mu/2 (tr C - 3) - mu ln J + lambda/2 (ln J)^2, C = F^T F."""
    mu, lbd = params[0], params[1]
    C = F.transpose(-1, -2) @ F
    log_j = 0.5 * torch.logdet(C)
    return mu / 2 * (torch.trace(C) - 3.0) - mu * log_j + lbd / 2 * log_j**2


def _neo_hookean_stress(F: Tensor, mu: Tensor, lbd: Tensor) -> Tensor:
    Fit = torch.linalg.inv(F).transpose(-1, -2)
    log_j = torch.log(torch.det(F))
    return mu[..., None, None] * F + (lbd * log_j - mu)[..., None, None] * Fit


class Hyperelastic3D(Material):
    """Hyperelastic material defined by an energy psi(F, params)
    (materials/hyperelasticity.py:12-127).

    `step` differentiates psi with torch.func like the reference.  The GPU
    kernels implement the Neo-Hookean energy in closed form; a psi is accepted
    for them if it is `neo_hookean_psi` or agrees with it (stress to 1e-10 on
    sample deformations), with params = (mu, lambda) per element.
    """

    def __init__(self, psi, params, rho=1.0):
        self.psi = psi
        self.params = torch.as_tensor(params)
        self.n_state = 0
        self.rho = torch.as_tensor(rho)
        self.is_vectorized = self.params.dim() > 1

    def step(self, H_inc, F, stress, state, de0, cl, iter):
        from torch.func import jacrev, vmap

        params = self.params if self.params.dim() > 1 else self.params.expand(H_inc.shape[0], -1)
        with torch.enable_grad():
            F_new = (F + H_inc).requires_grad_(True)
            P_new = vmap(jacrev(self.psi))(F_new, params)
            ddsdde = vmap(jacrev(jacrev(self.psi)))(F_new, params)
        return P_new, state, ddsdde

    def _is_neo_hookean(self) -> bool:
        if self.psi is neo_hookean_psi or getattr(self.psi, "gpu_model", None) == "neo_hookean":
            return True
        from torch.func import jacrev

        p = self.params.detach().reshape(-1, self.params.shape[-1])[0].to(torch.float64)
        if p.numel() != 2:
            return False
        gen = torch.Generator().manual_seed(0)
        for _ in range(3):
            F = torch.eye(3, dtype=torch.float64) + 0.2 * torch.rand(3, 3, generator=gen, dtype=torch.float64)
            try:
                P = jacrev(self.psi)(F, p)
            except Exception:  # noqa: BLE001 - any failure means "not the known energy"
                return False
            ref = _neo_hookean_stress(F, p[0], p[1])
            if not torch.allclose(P.to(torch.float64), ref, rtol=1e-10, atol=1e-10 * float(ref.abs().max())):
                return False
        return True

    def kernel_data(self, n_elem: int):
        if not self._is_neo_hookean():
            raise NotImplementedError(
                "Hyperelastic3D runs on the GPU for the Neo-Hookean energy only (params = (mu, lambda))"
            )
        data = self.params.to(torch.float64)
        if data.dim() == 1:
            data = data.expand(n_elem, 2)
        return "neo_hookean", data.contiguous()


# --------------------------------------------------------------- plasticity ---
class IsotropicPlasticityPlaneStrain(IsotropicElasticityPlaneStrain):
    """J2 plasticity in plane strain (materials/plasticity.py:430-590), with
    state (q, eps_z^p).  The GPU kernels implement linear hardening
    sigma_f(q) = sigma_y + H q; other hardening laws raise on solve."""

    def __init__(self, E, nu, sigma_f, sigma_f_prime, tolerance=1e-5, max_iter=10, rho=1.0):
        super().__init__(E, nu, rho)
        self.sigma_f = sigma_f
        self.sigma_f_prime = sigma_f_prime
        self.n_state = 2
        self.tolerance = tolerance
        self.max_iter = max_iter

    def _linear_hardening(self):
        q = torch.tensor([0.0, 0.1, 1.0, 10.0], dtype=torch.float64)
        sf = torch.as_tensor(self.sigma_f(q), dtype=torch.float64)
        sfp = torch.as_tensor(self.sigma_f_prime(q), dtype=torch.float64)
        if sf.shape != q.shape:
            sf = sf.expand(q.shape)
        if sfp.shape != q.shape:
            sfp = sfp.expand(q.shape)
        sy, H = float(sf[0]), float(sfp[0])
        ok = torch.allclose(sf, sy + H * q, rtol=1e-12, atol=1e-12) and torch.allclose(
            sfp, torch.full_like(q, H), rtol=1e-12, atol=1e-12
        )
        if not ok:
            raise NotImplementedError(
                "IsotropicPlasticityPlaneStrain runs on the GPU for linear hardening "
                "sigma_f(q) = sigma_y + H q only"
            )
        return sy, H

    def kernel_data(self, n_elem: int):
        sy, H = self._linear_hardening()
        E = torch.as_tensor(self.E, dtype=torch.float64).expand(n_elem)
        nu = torch.as_tensor(self.nu, dtype=torch.float64).expand(n_elem)
        data = torch.stack([E, nu, torch.full_like(E, sy), torch.full_like(E, H)], dim=-1)
        return "j2_plane_strain", data.contiguous()

    def step(self, H_inc, F, stress, state, de0, cl, iter):
        """Return mapping of plasticity.py:504-590 written with torch ops."""
        from math import sqrt

        de = 0.5 * (H_inc.transpose(-1, -2) + H_inc)
        C = self.C if self.C.dim() > 4 else self.C.expand(H_inc.shape[0], 2, 2, 2, 2)
        E = torch.as_tensor(self.E).expand(H_inc.shape[0])
        nu = torch.as_tensor(self.nu).expand(H_inc.shape[0])
        G = torch.as_tensor(self.G).expand(H_inc.shape[0])
        q, ez = state[..., 0].clone(), state[..., 1].clone()
        s2 = stress + torch.einsum("...ijkl,...kl->...ij", C, de - de0)
        s3 = torch.zeros(stress.shape[0], 3, 3, dtype=stress.dtype)
        s3[..., :2, :2] = s2
        s3[..., 2, 2] = nu * (s2[..., 0, 0] + s2[..., 1, 1]) - E * ez
        dev = s3 - torch.einsum("...ii->...", s3)[..., None, None] / 3 * torch.eye(3, dtype=s3.dtype)
        nrm = torch.linalg.norm(dev, dim=(-1, -2))
        f = nrm - sqrt(2.0 / 3.0) * self.sigma_f(q)
        fm = f > 0
        stress_new = s2.clone()
        ddsdde = C.clone()
        if fm.any():
            n = dev[fm] / nrm[fm][:, None, None]
            dG = torch.zeros_like(f[fm])
            qf = q[fm]
            for _ in range(self.max_iter):
                res = nrm[fm] - 2.0 * G[fm] * dG - sqrt(2.0 / 3.0) * self.sigma_f(qf)
                dd = res / (2.0 * G[fm] + 2.0 / 3.0 * self.sigma_f_prime(qf))
                dG = dG + dd
                qf = qf + sqrt(2.0 / 3.0) * dd
                if (res.abs() < self.tolerance).all():
                    break
            stress_new[fm] = (s3[fm] - (2.0 * G[fm] * dG)[:, None, None] * n)[..., :2, :2]
            q[fm] = qf
            ez[fm] = ez[fm] + dG * n[:, 2, 2]
            Gf = G[fm]
            A = 2.0 * Gf / (1.0 + self.sigma_f_prime(qf) / (3.0 * Gf))
            B = 4.0 * Gf**2 * dG / nrm[fm]
            n00, n11, n01, n10 = n[:, 0, 0], n[:, 1, 1], n[:, 0, 1], n[:, 1, 0]
            d = ddsdde[fm]
            d[:, 0, 0, 0, 0] += -A * n00**2 - B * (2 / 3 - n00**2)
            d[:, 1, 1, 1, 1] += -A * n11**2 - B * (2 / 3 - n11**2)
            d[:, 0, 0, 1, 1] += -A * n00 * n11 - B * (-1 / 3 - n00 * n11)
            d[:, 1, 1, 0, 0] += -A * n00 * n11 - B * (-1 / 3 - n00 * n11)
            d[:, 0, 1, 0, 1] += -A * n01**2 - B * (1 / 2 - n01**2)
            d[:, 0, 1, 1, 0] += -A * n01**2 - B * (1 / 2 - n10**2)
            d[:, 1, 0, 0, 1] += -A * n10**2 - B * (1 / 2 - n01**2)
            d[:, 1, 0, 1, 0] += -A * n10**2 - B * (1 / 2 - n10**2)
            ddsdde[fm] = d
        state_new = torch.stack([q, ez], dim=-1)
        return stress_new, state_new, ddsdde


# ------------------------------------------------------------ heat conduction ---
class IsotropicConductivity3D(Material):
    """Fourier heat conduction in 3D (materials/conductivity.py:11-99):
    conductivity tensor KAPPA = kappa I, heat flux update
    q_new = q + KAPPA (grad_inc - de0), tangent KAPPA.  The GPU kernels take
    KAPPA per element, so any symmetric or rotated tensor is exact."""

    dim = 3

    def __init__(self, kappa, rho=1.0):
        self.kappa = torch.as_tensor(kappa)
        self.rho = torch.as_tensor(rho)
        self.n_state = 0
        self.is_vectorized = self.kappa.dim() > 0
        self.KAPPA = self.kappa[..., None, None] * torch.eye(3, device=self.kappa.device)

    def step(self, H_inc, F, stress, state, de0, cl, iter):
        """q_new = q + KAPPA (grad_inc - de0) (conductivity.py:80-99)."""
        flux = stress + torch.einsum("...ij,...kj->...ki", self.KAPPA, H_inc - de0)
        return flux, state, self.KAPPA

    def kernel_data(self, n_elem: int) -> tuple[int, Tensor]:
        d = self.KAPPA.shape[-1]
        k = self.KAPPA.reshape(-1, d * d).to(torch.float64)
        if k.shape[0] != n_elem:
            k = k.expand(n_elem, d * d)
        return _lib.FEM_MAT_CONDUCTIVITY, k.contiguous()


class IsotropicConductivity2D(IsotropicConductivity3D):
    """In-plane 2x2 block of the 3D conductivity (conductivity.py:102-121)."""

    dim = 2

    def __init__(self, kappa, rho=1.0):
        super().__init__(kappa, rho)
        self.KAPPA = self.KAPPA[..., :2, :2]


class IsotropicConductivity1D(IsotropicConductivity2D):
    """Scalar 1x1 conductivity (conductivity.py:124-142); no 1D element is part
    of the GPU path, so it is kept for the material interface only."""

    dim = 1

    def __init__(self, kappa, rho=1.0):
        super().__init__(kappa, rho)
        self.KAPPA = self.KAPPA[..., :1, :1]


class OrthotropicConductivity3D(IsotropicConductivity3D):
    """Principal conductivities along the material axes, rotated into the
    global frame by `rotate` (conductivity.py:145-191)."""

    def __init__(self, kappa_1, kappa_2, kappa_3, rho=1.0):
        self.kappa_1 = torch.as_tensor(kappa_1)
        self.kappa_2 = torch.as_tensor(kappa_2)
        self.kappa_3 = torch.as_tensor(kappa_3)
        self.rho = torch.as_tensor(rho)
        self.n_state = 0
        self.is_vectorized = self.kappa_1.dim() > 0
        e = torch.eye(3, device=self.kappa_1.device)
        self.KAPPA = sum(k[..., None, None] * torch.outer(e[i], e[i])
                         for i, k in enumerate((self.kappa_1, self.kappa_2, self.kappa_3)))

    def rotate(self, R: Tensor) -> "OrthotropicConductivity3D":
        if R.shape[-2] != 3 or R.shape[-1] != 3:
            raise ValueError("Rotation matrix must be a 3x3 tensor.")
        new = copy.copy(self)
        new.KAPPA = torch.einsum("...ik,...jl,...kl->...ij", R, R, self.KAPPA)
        return new


class OrthotropicConductivity2D(IsotropicConductivity2D):
    """Two principal in-plane conductivities (conductivity.py:194-237)."""

    def __init__(self, kappa_1, kappa_2, rho=1.0):
        self.kappa_1 = torch.as_tensor(kappa_1)
        self.kappa_2 = torch.as_tensor(kappa_2)
        self.rho = torch.as_tensor(rho)
        self.n_state = 0
        self.is_vectorized = self.kappa_1.dim() > 0
        e = torch.eye(2, device=self.kappa_1.device)
        self.KAPPA = (self.kappa_1[..., None, None] * torch.outer(e[0], e[0])
                      + self.kappa_2[..., None, None] * torch.outer(e[1], e[1]))

    def rotate(self, R: Tensor) -> "OrthotropicConductivity2D":
        if R.shape[-2] != 2 or R.shape[-1] != 2:
            raise ValueError("Rotation matrix must be a 2x2 tensor.")
        new = copy.copy(self)
        new.KAPPA = torch.einsum("...ik,...jl,...kl->...ij", R, R, self.KAPPA)
        return new
