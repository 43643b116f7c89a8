"""Render configuration objects with the reference's field names
(ghostlight/src/render_config.h, bound by bind_config.cpp:70-377).  Only the
fields the flare hot path reads are acted on; the others are carried so
reference scripts that set them keep working.
"""
from __future__ import annotations

import enum
from dataclasses import dataclass, field


class InputColorSpace(enum.IntEnum):
    ACESCG = 0
    SRGB_LINEAR = 1
    CUSTOM = 2


class OutputColorSpace(enum.IntEnum):
    ACESCG = 0
    SRGB_LINEAR = 1
    P3_D65 = 2
    P3_D60 = 3
    XYZ = 4
    CUSTOM = 5


class StarburstEngine(enum.IntEnum):
    SPRITE = 0
    MDFT = 1


class GhostAovMode(enum.IntEnum):
    NONE = 0
    PER_PAIR = 1


class GhostFilterMode(enum.IntEnum):
    ALL = 0
    INCLUDE = 1
    EXCLUDE = 2


@dataclass
class GhostFilter:
    mode: GhostFilterMode = GhostFilterMode.ALL
    pairs: list = field(default_factory=list)


@dataclass
class DiffractionConfig:
    starburst: bool = False
    starburst_engine: StarburstEngine = StarburstEngine.SPRITE
    starburst_grid: int = 1024
    starburst_grid_cap: int = 8192
    pupil_fill: float = 0.30
    starburst_gain: float = 1.0
    scale_trim: float = 1.0
    spectral_samples: int = 0
    # matrix-DFT engine form: "pixel" = the reference's pixel-box-integrated
    # intensity through the pupil autocorrelation (mdft_render.cu); "field" =
    # the field E = W_y A W_x^T sampled at pixel centres, |E|^2
    mdft_form: str = "pixel"
    use_survivor_mask: bool = True
    use_surface_textures: bool = True
    survivor_grid: int = 192
    veil: bool = False
    veil_gain: float = 0.03
    veil_spread: float = 0.12
    veil_falloff: float = 1.5
    hurb: bool = False


@dataclass
class RenderConfig:
    ray_grid: int = 64
    spectral_samples: int = 16
    pupil_jitter: int = 0
    jitter_seed: int = 0
    sensor_model: int = 0
    input_cs: InputColorSpace = InputColorSpace.ACESCG
    output_cs: OutputColorSpace = OutputColorSpace.ACESCG
    custom_input_to_xyz: list = field(default_factory=lambda: [[0.0] * 3 for _ in range(3)])
    custom_xyz_to_output: list = field(default_factory=lambda: [[0.0] * 3 for _ in range(3)])
    sensor_half_w: float = 0.0
    sensor_half_h: float = 0.0
    verbose: bool = False
    collect_stats: bool = False
    spectral_correction: bool = True
    # arithmetic of the per-render source-position solve: "fp32" reproduces
    # the reference's float32 solve bit for bit; "fp64" solves in double
    setup_precision: str = "fp32"


@dataclass
class FlareConfig(RenderConfig):
    aperture_blades: int = 0
    aperture_rotation: float = 0.0
    flare_gain: float = 1000.0
    min_ghost_intensity: float = 1e-7
    ghost_normalize: bool = True
    max_area_boost: float = 100.0
    cull_dead_pairs: bool = True
    concentrate_samples: bool = True
    adaptive_sample_budgets: bool = True
    adaptive_density_boost: float = 8.0
    adaptive_min_samples: int = 1024
    aov_mode: GhostAovMode = GhostAovMode.NONE
    aov_max_pairs: int = -1
    ghost_filter: GhostFilter = field(default_factory=GhostFilter)
    diffraction: DiffractionConfig = field(default_factory=DiffractionConfig)
    # GB300 path: per-pair adaptive pupil grids (16^2..256^2, sized from each
    # ghost's probe footprint) instead of one ray_grid for every pair.
    adaptive_grids: bool = False
    adaptive_grid_min: int = 16
    adaptive_grid_max: int = 256


@dataclass
class PointFlareConfig(FlareConfig):
    source_x: float = 0.5
    source_y: float = 0.5
    source_r: float = 1.0
    source_g: float = 1.0
    source_b: float = 1.0


@dataclass
class PSFConfig(RenderConfig):
    grid_nx: int = 8
    grid_ny: int = 8
    tile_w: int = 64
    tile_h: int = 64
    tile_extent_mm: float = 0.05
    monochromatic: bool = False
    center_mode: int = 0
    splat_sigma_um: float = 4.0
    aperture_blades: int = 0
    aperture_rotation: float = 0.0


@dataclass
class LensCalibration:
    """LensCalibration (lens_calibration.h:12-55)."""
    sensor_half_w: float = 0.0
    sensor_half_h: float = 0.0
    max_half_angle_h: float = 0.0
    max_half_angle_v: float = 0.0
    image_circle_semi_w: float = 0.0
    image_circle_semi_h: float = 0.0
    focal_length_x: float = 0.0
    focal_length_y: float = 0.0
    entrance_pupil_semi_x: float = 0.0
    entrance_pupil_semi_y: float = 0.0
    f_number_x: float = 0.0
    f_number_y: float = 0.0
    pupil_area_frac: float = 1.0

    FIELDS = ("sensor_half_w", "sensor_half_h", "max_half_angle_h", "max_half_angle_v",
              "image_circle_semi_w", "image_circle_semi_h", "focal_length_x", "focal_length_y",
              "entrance_pupil_semi_x", "entrance_pupil_semi_y", "f_number_x", "f_number_y",
              "pupil_area_frac")

    @classmethod
    def from_dict(cls, d):
        return cls(**{k: float(d[k]) for k in cls.FIELDS if k in d})
