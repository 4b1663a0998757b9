"""CPU restatement of the reference's gradient processor (test oracle).

Follows ``ADFWI/propagator/gradient_process.py`` of the reference:

* ``smooth2d``      <- ``gauss2`` + ``smooth2d`` (lines 14-49): 'same'-size convolution with a
  normalised 2-D Gaussian of standard deviation ``span`` sampled every 2 cells over
  [-2 span, 2 span], divided by the same convolution of ones (restated here as the
  equivalent pair of 1-D passes, in float64);
* ``grad_taper``    <- ``grad_taper`` (lines 52-71): marine = zero the first ``tapersize``
  rows; land = the falling half of a Hamming window over the first ``tapersize`` columns of
  every row, smoothed, scaled to 1 - thred, and mapped to (1 - taper)^2;
* ``grad_process``  <- ``GradProcessor.forward`` (lines 91-134): taper, mask, illumination
  preconditioning, smoothing and max-abs scaling, with the reference's dtype flow (the taper
  and mask multiply a float32 gradient in place; everything after is float64).

Test infrastructure only: never imported by the product package.
"""
import numpy as np


def _weights(span):
    x = (-2.0 * span + 2.0 * np.arange(2 * span + 1)) / span
    f = np.exp(-0.5 * x * x)
    return f / f.sum()


def _conv1d_same(a, w, axis):
    span = (len(w) - 1) // 2
    a = np.moveaxis(np.asarray(a, dtype=np.float64), axis, -1)
    n = a.shape[-1]
    out = np.zeros_like(a)
    for b in range(-span, span + 1):
        lo, hi = max(0, -b), min(n, n - b)
        if lo < hi:
            out[..., lo:hi] += w[span + b] * a[..., lo + b:hi + b]
    return np.moveaxis(out, -1, axis)


def smooth2d(z, span=10):
    w = _weights(span)
    z = np.asarray(z, dtype=np.float64)
    num = _conv1d_same(_conv1d_same(z, w, 1), w, 0)
    den = _conv1d_same(_conv1d_same(np.ones_like(z), w, 1), w, 0)
    return num / den


def hamming(m):
    n = np.arange(m)
    return 0.54 - 0.46 * np.cos(2.0 * np.pi * n / (m - 1))


def grad_taper(nz, nx, tapersize=20, thred=0.05, marine_or_land="Marine"):
    if marine_or_land in ("Marine", "Offshore"):
        taper = np.ones((nz, nx))
        taper[:tapersize, :] = 0.0
        return taper
    h = hamming(2 * tapersize)[tapersize:]
    taper = np.zeros((nz, nx))
    taper[:, :tapersize] = h
    taper = smooth2d(taper, span=tapersize // 2)
    taper /= taper.max()
    taper *= (1 - thred)
    taper = -taper + 1
    return taper * taper


def grad_process(nx, nz, vmax, grad, forw=None, *, grad_mute=0, grad_smooth=0, grad_mask=None, norm_grad=True,
                 forw_illumination=True, marine_or_land="land"):
    mol = marine_or_land.lower()
    if mol in ("marine", "offshore"):
        thred = 0.0
    elif mol in ("land", "onshore"):
        thred = 0.001
    else:
        raise ValueError("not supported modeling marine_or_land: %s" % marine_or_land)
    # dtype flow of the reference: the taper and the mask multiply the float32 gradient in
    # place; the preconditioner and the land smoothing produce float64; the marine smoothing
    # writes into the array it has; the scaling keeps the array's type
    grad = np.array(grad, dtype=np.float32)
    if grad_mute > 0:
        grad = (grad * grad_taper(nz, nx, tapersize=grad_mute, thred=thred,
                                  marine_or_land=marine_or_land)).astype(np.float32)
    if grad_mask is not None:
        grad = (grad.astype(np.float64) * np.asarray(grad_mask, dtype=np.float64)).astype(np.float32)
    span = 40 if min(nz, nx) > 40 else int(min(nz, nx) / 2)
    if forw_illumination and forw is not None:
        precond = smooth2d(forw, span)
        precond = precond / np.max(precond + 1e-5)
        precond[precond < 1e-4] = 1e-4
        grad = grad / np.power(precond, 2)
    if grad_smooth > 0:
        if marine_or_land in ("marine", "offshore"):
            grad[grad_mute:, :] = smooth2d(grad[grad_mute:, :], span=grad_smooth)
        else:
            grad = smooth2d(grad, span=grad_smooth)
    if norm_grad:
        vm = np.asarray(vmax, dtype=grad.dtype)
        grad = (vm * grad) / np.abs(grad).max()
    return grad
