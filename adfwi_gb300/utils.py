"""Array helpers and source wavelets with the reference's signatures.

Mirrors ``ADFWI/utils/utils.py`` (numpy2tensor 8-16, tensor2numpy 18-25, gpu2cpu 27-38,
list2numpy / numpy2list 44-60) and ``ADFWI/utils/wavelets.py:4-36`` (``wavelet``).
"""
import numpy as np
import torch


def numpy2tensor(a, dtype=torch.float32):
    """Wrap a numpy array (or scalar/list) into a tensor; tensors pass through unchanged."""
    if torch.is_tensor(a):
        return a
    return torch.tensor(a, requires_grad=False, dtype=dtype)


def tensor2numpy(a):
    if torch.is_tensor(a):
        return a.detach().numpy()
    return a


def gpu2cpu(a):
    if torch.is_tensor(a):
        return a.detach().cpu().numpy()
    return a


def list2numpy(a):
    return np.array(a) if isinstance(a, list) else a


def numpy2list(a):
    return a if isinstance(a, list) else a.tolist()


def wavelet(nt, dt, f0, amp0=1, t0=None, type="Ricker"):
    """Source time function: Ricker, Gaussian (twice-integrated Ricker) or ramp.

    Returns ``(t, wavelet)`` with ``t = arange(nt) * dt`` and ``t0 = 1.2 / f0`` by default.
    """
    t = np.arange(nt) * dt + 0.0
    t0 = t0 if t0 is not None else 1.2 / f0
    kind = type.lower()
    if kind in ("ricker", "gaussian"):
        tau = (np.pi * f0) ** 2
        arg = tau * (t - t0) ** 2
        w = amp0 * (1 - 2 * arg) * np.exp(-arg)
        if kind == "gaussian":
            w = np.cumsum(np.cumsum(w))
    elif kind == "ramp":
        w = amp0 * 0.5 * (1.0 + np.tanh(t / t0))
    else:
        raise ValueError("Support source types: Rikcer, Guassian, Ramp. \n\nUnknown source type: {}".format(type))
    return t, w
