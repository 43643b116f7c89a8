"""render_psf (bind_renderers.cpp:148-191): a grid of per-source point-spread
tiles — each source's primary-ray spot, every pupil sample at every
wavelength, splatted into its own tile of a composite atlas.  The tile
centres come from the chief-ray pre-pass (PSFRenderer.cpp:243-430) on the
host in the reference's float32 arithmetic; the spots from one device launch
(csrc/gl_psf.cu)."""
from __future__ import annotations

import ctypes as C
import math

import numpy as np

from . import _native
from ._abi import gl_psf_cell, gl_psf_source, gl_pupil_sample, gl_spectral_sample


def _psf_spectrum(config):
    if getattr(config, "monochromatic", False):
        return np.array([[587.56, 0.0, 1.0, 0.0]], np.float32)
    ns = max(3, int(config.spectral_samples))
    if ns == 3:
        return np.array([[650.0, 1.0, 0.0, 0.0], [550.0, 0.0, 1.0, 0.0], [450.0, 0.0, 0.0, 1.0]], np.float32)
    from .flare import spectral_table
    spec, _ = spectral_table(ns, int(config.output_cs), config.custom_xyz_to_output)
    spec = spec.copy()
    d_lambda = np.float32(np.float32(700.0 - 400.0) / np.float32(ns))
    spec[:, 1:4] = (spec[:, 1:4] * d_lambda).astype(np.float32)
    return spec


def splat_footprint(splat_sigma_um, mm_pp):
    """(sigma, radius) of the Gaussian splat in pixels, in the reference's
    float32 (psf_render.cu:426-440): sigma = um / (mm_pp 1000), radius =
    ceil(2.5 sigma) in [1, 16]; (0, 0) selects the bilinear splat.  The
    float32 product matters: 2.5 x 1.6f rounds to exactly 4, where float64
    gives 4.00000006 and a radius of 5."""
    f = np.float32
    mm = f(mm_pp)
    sigma = f(f(splat_sigma_um) / f(mm * f(1000.0))) if mm > 0 else f(0.0)
    if not sigma > 0:
        return 0.0, 0
    radius = min(16, max(1, int(math.ceil(float(f(f(2.5) * sigma))))))
    return float(sigma), radius


def psf_inputs(sources, lens, config, cache=None) -> dict:
    """The host side of render_psf (PSFRenderer.cpp:243-330): checks, the
    pre-pass centring each tile, the per-tile sources, the pupil grid, the
    spectrum and the splat footprint, ready for gl_psf_render(_async).

    ``cache`` (a dict owned by a lens that does not change, e.g. a serving
    lens) keeps the pre-pass cells per (sources, centring mode) and the pupil
    grid per sampler setting: both depend on nothing else, so a repeated
    atlas skips the host pre-pass, which costs up to ~70 ms on long lenses."""
    from .flare import pupil_grid
    cfg = config
    if cfg.grid_nx <= 0 or cfg.grid_ny <= 0 or cfg.tile_w <= 0 or cfg.tile_h <= 0:
        raise ValueError("render_psf: grid and tile dimensions must be positive")
    if not (cfg.tile_extent_mm > 0.0) or not math.isfinite(cfg.tile_extent_mm):
        raise ValueError("render_psf: tile_extent_mm must be finite and positive")
    src = np.asarray(sources, np.float32)
    if src.ndim != 2 or src.shape[1] not in (5, 7):
        raise ValueError("render_psf: sources must be a (N, 5) array of [angle_x, angle_y, r, g, b] rows, "
                         "or a (N, 7) array with [.., target_x_mm, target_y_mm] appended")
    n = src.shape[0]
    if n > cfg.grid_nx * cfg.grid_ny:
        raise ValueError("render_psf: %d sources exceeds tile capacity %d" % (n, cfg.grid_nx * cfg.grid_ny))
    if not np.isfinite(src).all():
        raise ValueError("render_psf: source values must be finite")
    if lens.num_surfaces() <= 0:
        raise ValueError("render_psf: lens has no surfaces")
    s7 = np.zeros((n, 7), np.float32)
    s7[:, :src.shape[1]] = src
    lib = _native.load()
    arr = lens.to_array()
    mode = int(getattr(cfg, "center_mode", 0))
    ckey = ("cells", s7.tobytes(), mode)
    cells = cache.get(ckey) if cache is not None else None
    if cells is None:
        cells = (gl_psf_cell * max(1, n))()
        _native.check(lib.gl_psf_prepass(arr, len(arr), s7.ctypes.data_as(C.POINTER(C.c_float)), n, mode, cells),
                      "render_psf")
        if cache is not None:
            cache[ckey] = cells
    comp_w, comp_h = cfg.grid_nx * cfg.tile_w, cfg.grid_ny * cfg.tile_h
    mm_pp = float(np.float32(cfg.tile_extent_mm) / np.float32(cfg.tile_w))
    gs = (gl_psf_source * max(1, n))()
    for i in range(n):
        c = cells[i]
        gs[i] = gl_psf_source(c.beam_ax, c.beam_ay, float(s7[i, 2]), float(s7[i, 3]), float(s7[i, 4]),
                              c.chief_x_mm, c.chief_y_mm, (i % cfg.grid_nx) * cfg.tile_w,
                              (i // cfg.grid_nx) * cfg.tile_h)
    gkey = ("grid", int(cfg.ray_grid), int(cfg.pupil_jitter), int(cfg.jitter_seed),
            int(getattr(cfg, "aperture_blades", 0)), float(getattr(cfg, "aperture_rotation", 0.0)))
    grid = cache.get(gkey) if cache is not None else None
    if grid is None:
        grid = pupil_grid(lens, *gkey[1:])
        grid = np.ascontiguousarray(grid, np.float32)
        if cache is not None:
            cache[gkey] = grid
    spec = np.ascontiguousarray(_psf_spectrum(cfg), np.float32)
    sigma, radius = splat_footprint(cfg.splat_sigma_um, mm_pp)
    return dict(arr=arr, n=n, cells=cells, sources=gs, grid=grid, spec=spec, comp_w=comp_w, comp_h=comp_h,
                mm_pp=mm_pp, sigma=sigma, radius=radius, mono=int(bool(getattr(cfg, "monochromatic", 0))),
                tile_w=int(cfg.tile_w), tile_h=int(cfg.tile_h))


def psf_launch(inp: dict, out, stream, ordered: bool = False) -> None:
    """Enqueue the atlas of psf_inputs into `out` ((3, H, W) zeroed float32
    CUDA tensor) on `stream`: gl_psf_render_async when `ordered` (scratch from
    the device pool, no wait), else gl_psf_render."""
    lib = _native.load()
    P = C.POINTER
    fn = lib.gl_psf_render_async if ordered else lib.gl_psf_render
    _native.check(fn(inp["arr"], len(inp["arr"]), inp["sources"], inp["n"],
                     inp["grid"].ctypes.data_as(P(gl_pupil_sample)), len(inp["grid"]),
                     inp["spec"].ctypes.data_as(P(gl_spectral_sample)), len(inp["spec"]), inp["tile_w"],
                     inp["tile_h"], inp["comp_w"], inp["comp_h"], inp["mm_pp"], inp["mono"], inp["sigma"],
                     inp["radius"], out[0].data_ptr(), out[1].data_ptr(), out[2].data_ptr(), stream), "render_psf")


def render_psf(sources, lens, config) -> dict:
    """sources: (N, 5) [angle_x, angle_y, r, g, b] or (N, 7) with
    [target_x_mm, target_y_mm] appended.  Returns the reference's keys; the
    images r, g, b are torch CUDA tensors (composite_h, composite_w)."""
    import torch
    cfg = config
    inp = psf_inputs(sources, lens, cfg)
    n, cells = inp["n"], inp["cells"]
    comp_w, comp_h = inp["comp_w"], inp["comp_h"]
    out = torch.zeros((3, comp_h, comp_w), dtype=torch.float32, device="cuda")
    psf_launch(inp, out, torch.cuda.current_stream().cuda_stream)
    return {"composite_w": comp_w, "composite_h": comp_h, "tile_w": int(cfg.tile_w), "tile_h": int(cfg.tile_h),
            "grid_nx": int(cfg.grid_nx), "grid_ny": int(cfg.grid_ny), "tile_extent_mm": float(cfg.tile_extent_mm),
            "r": out[0], "g": out[1], "b": out[2],
            "chief_x_mm": np.array([cells[i].chief_x_mm for i in range(n)], np.float32),
            "chief_y_mm": np.array([cells[i].chief_y_mm for i in range(n)], np.float32),
            "status": np.array([cells[i].status for i in range(n)], np.uint8),
            "pupil_fraction": np.array([cells[i].pupil_fraction for i in range(n)], np.float32),
            "aim_residual_mm": np.array([cells[i].aim_residual_mm for i in range(n)], np.float32)}
