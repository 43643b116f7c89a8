"""FP64 oracle of the PSF / veil image convolution (TEST INFRASTRUCTURE ONLY).

out = in (*) k, 'same' size with the kernel centred (scipy.signal.fftconvolve
mode='same' semantics), in float64; plus a direct-sum evaluation at chosen
pixels for full-size checks.  The reference has no image convolution on the
flare path, so this oracle is the only pin ("parity unpinned" against the
reference itself).
"""
from __future__ import annotations

import numpy as np
from scipy.signal import fftconvolve


def conv_same(img, k):
    return fftconvolve(np.asarray(img, np.float64), np.asarray(k, np.float64), mode="same")


def conv_at(img, k, ys, xs):
    """Direct FP64 sums at pixels (ys[i], xs[i])."""
    img = np.asarray(img, np.float64)
    k = np.asarray(k, np.float64)
    kh, kw = k.shape
    cy, cx = kh // 2, kw // 2
    H, W = img.shape
    pad = np.zeros((H + kh - 1, W + kw - 1))
    pad[cy:cy + H, cx:cx + W] = img
    kf = k[::-1, ::-1]
    out = np.empty(len(ys))
    for i, (y, x) in enumerate(zip(ys, xs)):
        out[i] = np.sum(pad[y:y + kh, x:x + kw] * kf)
    return out


def psf_kernel(size: int, seed: int = 11):
    """The seeded synthetic veil kernel (input data, not an algorithm under test)."""
    from ghostlight_gb300.psf import synthetic_psf_kernel
    return synthetic_psf_kernel(size, seed)
