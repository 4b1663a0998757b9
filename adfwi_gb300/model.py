"""Velocity-model classes with the reference's constructor signatures and forward() maps.

Mirrors ``ADFWI/model``:
  * ``AbstractModel``            <- base.py:39-349 (bounds, clipping, constrain_range, get/set)
  * ``AcousticModel``            <- acoustic_model.py:18-133 (Gardner rho = 310 vp^0.25 in numpy,
                                     not differentiated w.r.t. vp, new leaf every forward())
  * ``IsotropicElasticModel``    <- elastic_model.py:22-234
  * ``AnisotropicElasticModel``  <- elastic_model.py:237-476
  * parameter maps               <- parameters.py:47-213 (Lame, Thomsen -> Cij, VTI/HTI copies,
                                     staggered bx, bz and the five-point C44/C55/C66 averages)
The maps stay in PyTorch autograd: gradients of the propagator's coefficients flow back to
vp, vs, rho, eps, delta (and gamma) through them. Plotting helpers are not part of this
package.
"""
from typing import Optional, Tuple, Union

import numpy as np
import torch
from torch import Tensor

from .utils import gpu2cpu, numpy2tensor

units = {"vp": "m/s", "vs": "m/s", "rho": "kg/m^3", "lam": "Pa", "mu": "Pa", "eps": "none",
         "gamma": "none", "delta": "none", "vs_vp": "none"}
_EPS = 1e-7


class AbstractModel(torch.nn.Module):
    """Common model state: grid, boundary settings, per-parameter bounds and grad flags."""

    def __init__(self, ox: float, oz: float, nx: int, nz: int, dx: float, dz: float,
                 free_surface: Optional[bool] = False, abc_type: Optional[str] = "PML",
                 abc_jerjan_alpha: Optional[float] = 0.0053, nabc: Optional[int] = 20,
                 device="cpu", dtype=torch.float32) -> None:
        super().__init__()
        self.ox, self.oz = ox, oz
        self.dx, self.dz = dx, dz
        self.nx, self.nz = nx, nz
        self.free_surface = free_surface
        self.abc_type = abc_type
        self.abc_jerjan_alpha = abc_jerjan_alpha
        self.nabc = nabc
        self.device = device
        self.dtype = dtype
        assert self.dx == self.dz, "Model grid size dx and dz must be the same"
        self.x = np.arange(nx) * self.dx + self.ox
        self.z = np.arange(nz) * self.dz + self.oz
        self.pars = []
        self.requires_grad = {}
        self.lower_bound = {}
        self.upper_bound = {}

    def __repr__(self) -> str:
        info = f"model with parameters {self.pars}:\n"
        for par in self.pars:
            m = self.get_model(par)
            info += (f"  Model {par:4s}: {m.min():8.2f} - {m.max():8.2f} {units[par]:6s}, "
                     f"requires_grad = {self.requires_grad[par]}, "
                     f"constrain bound: {self.lower_bound[par]} - {self.upper_bound[par]}\n")
        info += f"  Model orig: ox = {self.ox:6.2f}, oz = {self.oz:6.2f} m\n"
        info += f"  Model grid: dx = {self.dx:6.2f}, dz = {self.dz:6.2f} m\n"
        info += f"  Model dims: nx = {self.nx:6d}, nz = {self.nz:6d}\n"
        info += f"  Model size: {self.nx * self.nz * len(self.pars)}\n"
        info += f"  Free surface: {self.free_surface}\n"
        info += f"  Absorbing layers: {self.nabc}\n"
        return info

    def forward(self, *args, **kwargs):
        raise NotImplementedError("Forward method must be implemented by the subclass")

    def _check_bounds(self):
        for par in self.pars:
            lo, hi = self.lower_bound[par], self.upper_bound[par]
            if lo is not None and hi is not None:
                assert lo < hi, "Lower bound must be smaller than upper bound"
            if lo is not None and lo + _EPS > self.get_model(par).min():
                self.lower_bound[par] = self.get_model(par).min() - _EPS
            if hi is not None and hi - _EPS < self.get_model(par).max():
                self.upper_bound[par] = self.get_model(par).max() + _EPS

    def check_dims(self) -> None:
        for par in self.pars:
            assert self.get_model(par).shape == (self.nz, self.nx), "Model dimensions must be (nz, nx)"

    def get_model(self, par: str) -> np.ndarray:
        if par not in self.pars:
            raise ValueError(f"Parameter {par} not in model")
        return gpu2cpu(getattr(self, par).clone())

    def set_model(self, par: str, model) -> None:
        if par not in self.pars:
            raise ValueError(f"Parameter {par} not in model")
        if model.shape != (self.nz, self.nx):
            raise ValueError("Model dimensions must be (nz, nx)")
        model = numpy2tensor(gpu2cpu(model))
        setattr(self, par, torch.nn.Parameter(model.to(torch.float32),
                                              requires_grad=self.requires_grad[par]))

    def get_bound(self, par: str):
        if par not in self.pars:
            raise ValueError("Parameter {} not in model".format(par))
        lo, hi = self.lower_bound[par], self.upper_bound[par]
        if lo is None or hi is None:
            return [None, None]
        return [lo, hi]

    def get_requires_grad(self, par: str) -> bool:
        if par not in self.pars:
            raise ValueError("Parameter {} not in model".format(par))
        return self.requires_grad[par]

    def get_grad(self, par: str) -> np.ndarray:
        if par not in self.pars:
            raise ValueError("Parameter {} not in model".format(par))
        m = getattr(self, par)
        return np.zeros(m.shape) if m.grad is None else m.grad.cpu().detach().numpy()

    def get_clone_data(self):
        kwargs = {}
        for par in self.pars:
            kwargs[par] = self.get_model(par)
            kwargs[par + "_bound"] = self.get_bound(par)
            kwargs[par + "_grad"] = self.get_requires_grad(par)
        kwargs.update(ox=self.ox, oz=self.oz, dx=self.dx, dz=self.dz, nx=self.nx, nz=self.nz,
                      free_surface=self.free_surface, nabc=self.nabc)
        return kwargs

    def save(self, filename: str) -> None:
        np.savez(filename, **self.get_clone_data())

    def clip_params(self) -> None:
        """In-place clamp of every bounded parameter (base.py:302-312)."""
        for par in self.pars:
            lo, hi = self.lower_bound[par], self.upper_bound[par]
            if lo is not None and hi is not None:
                getattr(self, par).data.clamp_(lo, hi)

    def constrain_range(self, value, min_value, max_value) -> Tensor:
        """Clamp with NaN replacement and Inf / negative / NaN checks (base.py:314-349)."""
        if min_value is None or max_value is None:
            return value
        if torch.isnan(value).any():
            value[torch.isnan(value)] = max_value
        value = torch.clamp(value, min_value, max_value)
        if torch.isinf(value).any():
            raise ValueError("Value is inf")
        if (value < 0.0).any():
            raise ValueError("Value is negative")
        if torch.isnan(value).any():
            raise ValueError("Value is nan")
        return value

    def _param(self, value, grad):
        return torch.nn.Parameter(numpy2tensor(value, self.dtype).to(self.device), requires_grad=grad)

    def _gardner_rho(self):
        """rho = 310 vp^0.25 evaluated in numpy on the host (acoustic_model.py:111-118)."""
        vp = self.vp.cpu().detach().numpy()
        rho = np.power(vp, 0.25) * 310
        self.rho = self._param(rho, self.rho_grad)


class AcousticModel(AbstractModel):
    """Acoustic model parameterised by vp and rho (rho re-derived from vp by Gardner)."""

    def __init__(self, ox: float, oz: float, nx: int, nz: int, dx: float, dz: float,
                 vp: Optional[Union[np.ndarray, Tensor]] = None,
                 rho: Optional[Union[np.ndarray, Tensor]] = None,
                 vp_bound: Optional[Tuple[float, float]] = None,
                 rho_bound: Optional[Tuple[float, float]] = None,
                 vp_grad: Optional[bool] = False, rho_grad: Optional[bool] = False,
                 free_surface: Optional[bool] = False, abc_type: Optional[str] = "PML",
                 abc_jerjan_alpha: Optional[float] = 0.0053, nabc: Optional[int] = 20,
                 device="cpu", dtype=torch.float32) -> None:
        super().__init__(ox, oz, nx, nz, dx, dz, free_surface, abc_type, abc_jerjan_alpha, nabc,
                         device, dtype)
        self.pars = ["vp", "rho"]
        self.vp_grad = vp_grad
        self.rho_grad = rho_grad
        self.vp = self._param(vp.copy(), vp_grad)
        self.rho = self._param(rho.copy(), rho_grad)
        self.lower_bound["vp"] = vp_bound[0] if vp_bound is not None else None
        self.lower_bound["rho"] = rho_bound[0] if rho_bound is not None else None
        self.upper_bound["vp"] = vp_bound[1] if vp_bound is not None else None
        self.upper_bound["rho"] = rho_bound[1] if rho_bound is not None else None
        self.requires_grad["vp"] = vp_grad
        self.requires_grad["rho"] = rho_grad
        self._check_bounds()
        self.check_dims()

    def set_rho_using_empirical_function(self):
        self._gardner_rho()

    def forward(self):
        self.clip_params()
        self.constrain_range(self.vp, self.lower_bound["vp"], self.upper_bound["vp"])
        self.set_rho_using_empirical_function()
        self.constrain_range(self.rho, self.lower_bound["rho"], self.upper_bound["rho"])
        return


def vs_vp_to_Lame(vp, vs, rho):
    """mu = vs^2 rho, lambda+2mu = vp^2 rho, lambda, buoyancy (parameters.py:47-68)."""
    mu = vs ** 2 * rho
    lamu = vp ** 2 * rho
    lam = lamu - 2 * mu
    b = 1 / rho
    return mu, lamu, lam, b


def thomsen_to_elastic_moduli(alpha_thomsen, beta_thomsen, rho, eps_thomsen, delta_thomsen, gamma_thomsen):
    """Thomsen (vp, vs, rho, eps, delta, gamma) -> C11, C13, C33, C44, C66 (parameters.py:71-107)."""
    c33 = alpha_thomsen ** 2 * rho
    c44 = beta_thomsen ** 2 * rho
    c11 = c33 * (1 + 2 * eps_thomsen)
    c66 = c44 * (1 + 2 * gamma_thomsen)
    c13 = torch.sqrt(2 * c33 * (c33 - c44) * delta_thomsen + (c33 - c44) ** 2) - c44
    return c11, c13, c33, c44, c66


def _zeros21(nz, nx, device, dtype):
    return [torch.zeros((nz, nx), dtype=dtype).to(device) for _ in range(21)]


def _five_point(a, nz, nx):
    """0.2 * (a[1:-1,1:-1] + a[2:,1:-1] + a[1:-1,2:] + a[2:,1:-1] + a[2:,2:]) (parameters.py:202-212)."""
    return 0.2 * (a[1:nz - 1, 1:nx - 1] + a[2:nz, 1:nx - 1] + a[1:nz - 1, 2:nx]
                  + a[2:nz, 1:nx - 1] + a[2:nz, 2:nx])


def parameter_staggered_grid(mu, b, C44, C55, C66, nx, nz):
    bx = 0.5 * (b[:, 0:nx - 1] + b[:, 1:nx])
    bz = 0.5 * (b[0:nz - 1, :] + b[1:nz, :])
    return bx, bz, _five_point(mu, nz, nx), _five_point(C44, nz, nx), _five_point(C55, nz, nx), \
        _five_point(C66, nz, nx)


class _ElasticBase(AbstractModel):
    anisotropic_type = "vti"

    def _parameterization_thomson(self):
        for name in ("vp", "vs", "rho", "eps", "gamma", "delta"):
            setattr(self, name, self._param(getattr(self, name), getattr(self, name + "_grad", False)))

    def _parameterization_Lame(self):
        self.mu, self.lamu, self.lam, self.b = vs_vp_to_Lame(self.vp, self.vs, self.rho)

    def _parameterization_elastic_moduli(self):
        CC = _zeros21(self.nz, self.nx, self.device, self.dtype)
        C11, C13, C33, C44, C66 = thomsen_to_elastic_moduli(self.vp, self.vs, self.rho, self.eps,
                                                            self.delta, self.gamma)
        C12 = (C11 - 2 * C66).clone()
        C55 = C44.clone()
        if self.anisotropic_type.lower() == "hti":
            # HTI ordering of parameters.py:178-180
            CC = [C33, C13, C13, CC[3], CC[4], CC[5], C11, C12, CC[8], CC[9], CC[10], C11, CC[12],
                  CC[13], CC[14], C66, CC[16], CC[17], C55, CC[19], C55]
        else:
            CC = [C11, C12, C13, CC[3], CC[4], CC[5], C11.clone(), C13.clone(), CC[8], CC[9], CC[10],
                  C33, CC[12], CC[13], CC[14], C44, CC[16], CC[17], C55, CC[19], C66]
        bx, bz, muxz, c44s, c55s, c66s = parameter_staggered_grid(self.mu, self.b, CC[15], CC[18], CC[20],
                                                                  self.nx, self.nz)
        CC[15], CC[18], CC[20] = c44s, c55s, c66s
        self.bx, self.bz, self.muxz = bx, bz, muxz
        self.CC = CC

    def set_rho_using_empirical_function(self):
        self._gardner_rho()

    def set_vp_using_empirical_function(self):
        vs = self.vs.cpu().detach().numpy()
        self.vp = self._param(vs * np.sqrt(3), self.vp_grad)

    def _finish_init(self, bounds, auto_update_rho, auto_update_vp):
        self._parameterization_Lame()
        self._parameterization_elastic_moduli()
        for par in self.pars:
            bd = bounds.get(par)
            self.lower_bound[par] = bd[0] if bd is not None else None
            self.upper_bound[par] = bd[1] if bd is not None else None
            self.requires_grad[par] = getattr(self, par + "_grad")
        self._check_bounds()
        self.check_dims()
        self.auto_update_rho = auto_update_rho
        self.auto_update_vp = auto_update_vp

    def forward(self) -> None:
        if self.auto_update_rho:
            self.set_rho_using_empirical_function()
        if self.auto_update_vp:
            self.set_vp_using_empirical_function()
        self.clip_params()
        self._parameterization_Lame()
        self._parameterization_elastic_moduli()
        return


class IsotropicElasticModel(_ElasticBase):
    """Isotropic elastic model (vp, vs, rho); eps = gamma = delta = 0."""

    def __init__(self, ox: float, oz: float, nx: int, nz: int, dx: float, dz: float,
                 vp=None, vs=None, rho=None, vp_bound=None, vs_bound=None, rho_bound=None,
                 vp_grad: Optional[bool] = False, vs_grad: Optional[bool] = False,
                 rho_grad: Optional[bool] = False, free_surface: Optional[bool] = False,
                 abc_type: Optional[str] = "PML", abc_jerjan_alpha: Optional[float] = 0.0053,
                 nabc: Optional[int] = 20, auto_update_rho: Optional[bool] = True,
                 auto_update_vp: Optional[bool] = False, device="cpu", dtype=torch.float32) -> None:
        super().__init__(ox, oz, nx, nz, dx, dz, free_surface, abc_type, abc_jerjan_alpha, nabc,
                         device, dtype)
        self.pars = ["vp", "vs", "rho"]
        self.vp, self.vs, self.rho = vp.copy(), vs.copy(), rho.copy()
        self.vp_grad, self.vs_grad, self.rho_grad = vp_grad, vs_grad, rho_grad
        self.eps = np.zeros((nz, nx))
        self.gamma = np.zeros((nz, nx))
        self.delta = np.zeros((nz, nx))
        self.anisotropic_type = "vti"
        self._parameterization_thomson()
        self._finish_init({"vp": vp_bound, "vs": vs_bound, "rho": rho_bound}, auto_update_rho,
                          auto_update_vp)


class AnisotropicElasticModel(_ElasticBase):
    """VTI / HTI elastic model (vp, vs, rho, eps, gamma, delta)."""

    def __init__(self, ox: float, oz: float, nx: int, nz: int, dx: float, dz: float,
                 vp=None, vs=None, rho=None, eps=None, gamma=None, delta=None,
                 vp_bound=None, vs_bound=None, rho_bound=None, eps_bound=None, gamma_bound=None,
                 delta_bound=None, vp_grad: Optional[bool] = False, vs_grad: Optional[bool] = False,
                 rho_grad: Optional[bool] = False, eps_grad: Optional[bool] = False,
                 gamma_grad: Optional[bool] = False, delta_grad: Optional[bool] = False,
                 free_surface: Optional[bool] = False, auto_update_rho: Optional[bool] = False,
                 auto_update_vp: Optional[bool] = False, anisotropic_type: Optional[str] = "vti",
                 abc_type: Optional[str] = "PML", abc_jerjan_alpha: Optional[float] = 0.0053,
                 nabc: Optional[int] = 20, device="cpu", dtype=torch.float32) -> None:
        super().__init__(ox, oz, nx, nz, dx, dz, free_surface, abc_type, abc_jerjan_alpha, nabc,
                         device, dtype)
        self.pars = ["vp", "vs", "rho", "eps", "gamma", "delta"]
        self.vp, self.vs, self.rho = vp.copy(), vs.copy(), rho.copy()
        self.eps, self.gamma, self.delta = eps.copy(), gamma.copy(), delta.copy()
        self.vp_grad, self.vs_grad, self.rho_grad = vp_grad, vs_grad, rho_grad
        self.eps_grad, self.gamma_grad, self.delta_grad = eps_grad, gamma_grad, delta_grad
        self.anisotropic_type = anisotropic_type
        self._parameterization_thomson()
        self._finish_init({"vp": vp_bound, "vs": vs_bound, "rho": rho_bound, "eps": eps_bound,
                           "gamma": gamma_bound, "delta": delta_bound}, auto_update_rho, auto_update_vp)
