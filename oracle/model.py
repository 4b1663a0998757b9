"""CPU restatement of the reference's model -> propagator-coefficient maps (test oracle).

Follows ``ADFWI/model/parameters.py`` of the reference: ``vs_vp_to_Lame``
(lines 47-68), ``thomsen_to_elastic_moduli`` (71-107),
``elastic_moduli_for_isotropic`` / ``_for_TI`` (135-181, which set C55 := C44),
and ``parameter_staggered_grid`` (184-213: bx, bz half-cell averages and the
five-point C55 average that repeats ``[2:nz, 1:nx-1]``); plus the Gardner
density of ``ADFWI/model/acoustic_model.py:111-118``.

Test infrastructure only: never imported by the product package.
"""
import numpy as np
import torch


def gardner_rho(vp_np):
    """rho = 310 * vp**0.25 computed in numpy, not differentiated (acoustic_model.py:111-118)."""
    return np.power(vp_np, 0.25) * 310


def elastic_coefficients(vp, vs, rho, eps, delta, gamma, anisotropic_type="vti"):
    """Differentiable map to the propagator's C11, C13, C15, C33, C35, C55, bx, bz (unpadded)."""
    nz, nx = vp.shape
    b = 1 / rho
    c33 = vp ** 2 * rho
    c44 = vs ** 2 * rho
    c11 = c33 * (1 + 2 * eps)
    c66 = c44 * (1 + 2 * gamma)
    c13 = torch.sqrt(2 * c33 * (c33 - c44) * delta + (c33 - c44) ** 2) - c44
    if anisotropic_type.lower() == "hti":
        # HTI ordering of elastic_moduli_for_TI (parameters.py:178-180): C11<-C33, C13<-C13,
        # C33<-C11, C55<-C55 (=C44); the propagator reads C11, C13, C33, C55.
        c11, c33 = c33, c11
    c55 = c44
    bx = 0.5 * (b[:, 0:nx - 1] + b[:, 1:nx])
    bz = 0.5 * (b[0:nz - 1, :] + b[1:nz, :])
    c55 = 0.2 * (c55[1:nz - 1, 1:nx - 1] + c55[2:nz, 1:nx - 1] + c55[1:nz - 1, 2:nx]
                 + c55[2:nz, 1:nx - 1] + c55[2:nz, 2:nx])
    zero = torch.zeros((nz, nx), dtype=vp.dtype)
    return {"C11": c11, "C13": c13, "C15": zero, "C33": c33, "C35": zero, "C55": c55, "bx": bx, "bz": bz}
