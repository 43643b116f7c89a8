"""PSF / veil image convolution (row e of the flare path).

``ConvPlan`` convolves three W x H float32 planes with one kh x kw float32
kernel ('same' output, kernel centred at (kh // 2, kw // 2), zero padding
outside the image) by a mixed-radix FFT route on the device: the padded
transform sizes P, Q are the smallest 2^a 3^b >= image + kernel - 1, the kernel
spectrum is built once per plan and stays resident, and one execute is three
HBM passes (rows forward; columns forward x K-hat x inverse; rows inverse and
crop).  Two colour planes share one complex transform.

The reference has no image convolution on its flare path; its nearest pieces
are the analytic veil sprite (ghostlight/src/veil_render.cu:243) and the PSF
kernel builder (ghostlight/src/psf_render.cu:34).  ``execute`` can sum a
second layer into the input on load, so the flare composite (ghosts +
starburst) is convolved without a separate add pass.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native


def synthetic_psf_kernel(size: int = 257, seed: int = 11) -> np.ndarray:
    """Seeded smooth radial kernel (1 + r^2)^-1.5 plus 2% uniform noise,
    normalised to sum 1 — the 257 x 257 FP32 veil kernel of the starburst
    precision workload."""
    rng = np.random.default_rng(seed)
    c = size // 2
    y, x = np.mgrid[0:size, 0:size].astype(np.float64)
    r = np.hypot(x - c, y - c) / (0.18 * size)
    k = (1.0 / (1.0 + r * r)) ** 1.5 + 0.02 * rng.random((size, size))
    return (k / k.sum()).astype(np.float32)


class ConvPlan:
    def __init__(self, width: int, height: int, kernel, stream=None):
        import torch
        self._lib = _native.load()
        k = np.ascontiguousarray(kernel, np.float32)
        if k.ndim != 2:
            raise ValueError("conv2d: kernel must be 2-D")
        self.width, self.height = int(width), int(height)
        self.kh, self.kw = k.shape
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        h = C.c_void_p()
        _native.check(self._lib.gl_conv2d_plan_create(self.width, self.height,
                                                      k.ctypes.data_as(C.POINTER(C.c_float)), self.kw, self.kh,
                                                      st, C.byref(h)), "conv2d")
        self._h = h
        P, Q = C.c_int(), C.c_int()
        _native.check(self._lib.gl_conv2d_plan_info(h, C.byref(P), C.byref(Q)), "conv2d")
        self.P, self.Q = P.value, Q.value

    def _check(self, planes):
        import torch
        for t in planes:
            if not (t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()
                    and tuple(t.shape) == (self.height, self.width)):
                raise ValueError("conv2d: planes must be contiguous float32 CUDA (H, W) tensors")

    def execute(self, inputs, outputs, add=None, stream=None):
        """outputs[c] = (inputs[c] (+ add[c])) conv kernel; returns launches."""
        import torch
        self._check(list(inputs) + list(outputs) + (list(add) if add is not None else []))
        st = stream if stream is not None else torch.cuda.current_stream().cuda_stream
        a = [t.data_ptr() for t in add] if add is not None else [None, None, None]
        _native.check(self._lib.gl_conv2d_plan_execute2(self._h, *[t.data_ptr() for t in inputs], *a,
                                                        *[t.data_ptr() for t in outputs], st), "conv2d")
        return _native.last_launch_count()

    def traffic_bytes(self) -> int:
        """HBM bytes of one execute by the three-pass schedule: planes in and
        out, the two-pair complex intermediate written and read twice, the
        kernel spectrum read once."""
        planes = 3 * self.width * self.height * 4
        inter = 2 * self.height * self.Q * 8
        return 2 * planes + 4 * inter + self.P * self.Q * 8

    def close(self):
        if getattr(self, "_h", None):
            self._lib.gl_conv2d_plan_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def convolve_psf(images, kernel):
    """One-shot: three (H, W) float32 CUDA tensors -> three convolved tensors."""
    import torch
    H, W = images[0].shape
    plan = ConvPlan(W, H, kernel)
    outs = [torch.empty_like(images[0]) for _ in range(3)]
    plan.execute([i.contiguous() for i in images], outs)
    torch.cuda.synchronize()
    plan.close()
    return outs
