"""Source sweep: many frames of one lens (one source each) as one CUDA graph.

A frame is the ghost layer of one point source (a stream-ordered request on
the resident lens, uniform pupil grid) plus, optionally, the lens's starburst
centred on the source's image point, added into the same planes (split-BF16
matrix DFT, rectangular output).  Every frame's enqueue — probe passes,
render, flush, DFT-matrix recentring, the two tensor-core GEMMs — is captured
once into a CUDA graph; a replay renders the whole sweep with no host work.

The reference renders such a sweep as one blocking render_point_flare call per
source (bind_renderers.cpp:85-102), each re-uploading the lens and launching
per ghost.
"""
from __future__ import annotations

import ctypes as C
import math
from typing import List, Optional

import numpy as np

from . import _native
from ._abi import gl_flare_source, gl_spectral_sample
from .serve import ResidentLens, _spectral, render_params, FlareRequest


class SourceSweep:
    def __init__(self, resident: ResidentLens, sources_rad, width: int, height: int, n_spec: int, ray_grid: int,
                 gain: float = 1000.0, starburst=None, stream=None, items_per_warp: int = 0,
                 side_streams: int = 3):
        """sources_rad: (N, 2) field angles (x, y) in radians, one frame each.
        starburst: None, or dict(plan=MdftPlan over (width, height), pupil=(n, n) tensor,
        centers=(N, 2) pixel centres)."""
        import torch
        self.torch = torch
        self._lib = _native.load()
        self.rl = resident
        self.width, self.height = int(width), int(height)
        self.n_spec, self.ray_grid = int(n_spec), int(ray_grid)
        self.items_per_warp = int(items_per_warp)
        self.stream = stream if stream is not None else torch.cuda.Stream()
        self.side = [torch.cuda.Stream() for _ in range(max(1, int(side_streams)))]
        self.starburst = starburst
        src = np.asarray(sources_rad, np.float64).reshape(-1, 2)
        self.n_frames = len(src)
        spec, corr = _spectral(self.n_spec, resident.config)
        self.spec = np.ascontiguousarray(spec, np.float32)
        apply_corr = bool(resident.config.spectral_correction) and self.n_spec != 3
        self.requests: List[C.c_void_p] = []
        P = C.POINTER
        st = self.stream.cuda_stream
        for k in range(self.n_frames):
            req = FlareRequest(lens_id=0, width=self.width, height=self.height, n_spec=self.n_spec,
                               ray_grid=self.ray_grid, field_deg=0.0, gain=gain)
            prm = render_params(resident, req, corr, apply_corr)
            s = np.array([[src[k, 0], src[k, 1], 1.0, 1.0, 1.0]], np.float32)
            h = C.c_void_p()
            _native.check(self._lib.gl_request_create(resident._h, self.ray_grid,
                                                      self.spec.ctypes.data_as(P(gl_spectral_sample)), len(self.spec),
                                                      s.ctypes.data_as(P(gl_flare_source)), 1, C.byref(prm), st,
                                                      C.byref(h)), "request_create")
            self.requests.append(h)
        self.planes = []
        for h in self.requests:
            d = C.c_void_p()
            _native.check(self._lib.gl_request_planes(h, C.byref(d)), "request_planes")
            self.planes.append(int(d.value))
        self.stream.synchronize()
        self.graph = None
        self.launches = 0

    def _enqueue_all(self) -> int:
        """Ghost frames round-robin over the side streams (a frame's probe and
        render launches overlap the previous frame's tail); the starburst of
        frame k runs on the main stream once frame k's ghost layer is written
        (one plan, one centre at a time); the main stream joins every side
        stream at the end."""
        torch = self.torch
        main = self.stream
        n = 0
        npx = self.width * self.height
        sb = self.starburst
        fork = torch.cuda.Event()
        fork.record(main)
        for s in self.side:
            s.wait_event(fork)
        for k, h in enumerate(self.requests):
            side = self.side[k % len(self.side)]
            _native.check(self._lib.gl_request_enqueue(h, None, None, None, self.items_per_warp, side.cuda_stream),
                          "request_enqueue")
            n += _native.last_launch_count()
            if sb is not None:
                ev = torch.cuda.Event()
                ev.record(side)
                main.wait_event(ev)
                cx, cy = sb["centers"][k]
                n += sb["plan"].set_center(cx, cy, stream=main.cuda_stream)
                base = self.planes[k]
                n += sb["plan"].execute_raw(sb["pupil"].data_ptr(), base, base + 4 * npx, base + 8 * npx,
                                            stream=main.cuda_stream, accumulate=True)
        for s in self.side:
            ev = torch.cuda.Event()
            ev.record(s)
            main.wait_event(ev)
        return n

    def run(self) -> int:
        """Enqueue the sweep without a graph (the same work a replay does)."""
        with self.torch.cuda.stream(self.stream):
            return self._enqueue_all()

    def capture(self):
        torch = self.torch
        with torch.cuda.stream(self.stream):
            self._enqueue_all()                    # warm: every kernel loaded, opt-ins set
            self.stream.synchronize()
            g = torch.cuda.CUDAGraph()
            with torch.cuda.graph(g, stream=self.stream):
                self.launches = self._enqueue_all()
        self.graph = g
        return g

    def replay(self):
        with self.torch.cuda.stream(self.stream):
            self.graph.replay()

    def frame(self, k: int):
        """(3, H, W) float32 CUDA tensor copy of frame k."""
        torch = self.torch
        out = torch.empty((3, self.height, self.width), dtype=torch.float32, device="cuda")
        _native.check(self._lib.gl_request_copy_out(self.requests[k], out.data_ptr(), self.stream.cuda_stream),
                      "request_copy_out")
        self.stream.synchronize()
        return out

    def copy_out(self, host, k: int):
        """Enqueue frame k's planes into `host` (pinned, 3*H*W float32)."""
        _native.check(self._lib.gl_request_copy_out(self.requests[k], host.data_ptr(), self.stream.cuda_stream),
                      "request_copy_out")

    def traced(self) -> int:
        tot = 0
        for h in self.requests:
            v = C.c_longlong()
            _native.check(self._lib.gl_request_traced(h, C.byref(v), None), "request_traced")
            tot += int(v.value)
        return tot

    def close(self):
        st = self.stream.cuda_stream
        for h in self.requests:
            self._lib.gl_request_destroy(h, st)
        self.requests = []
        self.graph = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def diagonal_sources(n: int, max_deg: float, sensor_half_w: float, sensor_half_h: float, fx: float, fy: float):
    """n field angles from on-axis to max_deg along the sensor diagonal: the
    direction whose paraxial image (fx tan ax, fy tan ay) runs to the corner."""
    d = np.array([sensor_half_w / fx, sensor_half_h / fy])
    d /= np.linalg.norm(d)
    th = np.radians(np.linspace(0.0, max_deg, n))
    return np.stack([th * d[0], th * d[1]], axis=1)


def paraxial_centers(sources_rad, fx: float, fy: float, sensor_half_w: float, sensor_half_h: float, width: int,
                     height: int):
    """Pixel position of each source's paraxial image point."""
    s = np.asarray(sources_rad, np.float64)
    x = fx * np.tan(s[:, 0])
    y = fy * np.tan(s[:, 1])
    return np.stack([(x / (2 * sensor_half_w) + 0.5) * width, (y / (2 * sensor_half_h) + 0.5) * height], axis=1)
