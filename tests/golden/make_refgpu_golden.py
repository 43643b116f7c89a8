"""Record the reference's own GPU renderer on the seeded configurations.

Runs on a GPU host.  It builds the reference's core library with its CUDA
renderers for sm_103a from the staged sources (oracle/build.py:build_ref_gpu,
oracle/stage_ref.py) and calls its render_point_flare / render_source_flare
(PointFlareRenderer.cpp:11, SourceFlareRenderer.cpp:24) through
oracle/ref_driver.cpp.  Three things are written to ``--out``:

* ``refgpu_selfcheck.json`` — the sm_103a build against the reference's own
  stored goldens (validation/goldens, recorded with CUDA 13.2), by max
  difference in ppm of peak, to show that this compile of the reference
  reproduces the reference;
* ``refgpu_images.npz`` + ``refgpu_meta.json`` — its images of the seeded
  configuration-1, -2 and -4 lenses with deterministic sampling
  (concentration off), and its veil and starburst layers (matrix-DFT and
  SPRITE engines, on and off axis) on the configuration-1 lens; ``--pack DIR`` turns them into the committed fixtures
  ``refgpu_seeded.npz`` / ``refgpu_seeded.json`` (15 mantissa bits kept, as
  make_refgolden.py packs) for tests/test_gpu_refgpu.py;
* ``refgpu_timing.json`` — its wall time and kernel-stage time on the
  configuration-2 frame (24 surfaces, 31 wavelengths, 2048^2, 15 deg).

    python tests/golden/make_refgpu_golden.py --out OUTDIR      (GPU host)
    python tests/golden/make_refgpu_golden.py --pack OUTDIR     (packs into tests/golden)
"""
from __future__ import annotations

import argparse
import json
import math
import pathlib
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
REPO = HERE.parents[1]
sys.path.insert(0, str(REPO))

from oracle import ref as R  # noqa: E402


def _lens(pins, meta, name):
    return pins[name + "/lens"], float(meta[name]["focal_length"]), meta[name]["calibration"]


def _ppm(img, ref):
    d = float(np.abs(img.astype(np.float64) - ref.astype(np.float64)).max())
    return d / (float(ref.sum(-1).max()) + 1e-30) * 1e6


def _hwc(planes):
    return np.ascontiguousarray(np.moveaxis(planes, 0, -1))


def selfcheck(pins, meta, imgs):
    """The two DoubleGauss point-flare-sampling goldens and the two
    aperture-baseline axial goldens that the fixtures hold."""
    out = {}
    for key in ("refgpu_pfs_dg_axial_c0", "refgpu_pfs_dg_axial_c1", "refgpu_ab_dg_axial", "refgpu_ab_hex_axial"):
        m = meta[key]
        raw, focal, cal = _lens(pins, meta, m["lens"])
        sh = (m["sensor_half"], m["sensor_half"]) if m["sensor_half"] != "calib" else \
            (cal["sensor_half_w"], cal["sensor_half_h"])
        cfg = R.RefGpuCfg(ray_grid=m["ray_grid"], spectral_samples=m["spectral_samples"],
                          pupil_jitter=m["pupil_jitter"], jitter_seed=m["jitter_seed"],
                          sensor_half_w=sh[0], sensor_half_h=sh[1], flare_gain=m["flare_gain"],
                          min_ghost_intensity=m["min_ghost_intensity"], cull_dead_pairs=int(m.get("cull", False)),
                          concentrate_samples=0, source_x=m["source_xy"][0], source_y=m["source_xy"][1],
                          source_r=m["source_rgb"], source_g=m["source_rgb"], source_b=m["source_rgb"])
        g, _, ms, _ = R.gpu_render(raw, m["W"], m["H"], cfg, calib=None, focal_length=focal)
        img = _hwc(g)
        want = imgs[key + "/image"]
        out[key] = {"max_diff_ppm_of_peak": _ppm(img, want), "ms": ms,
                    "rel_l2": float(np.linalg.norm(img.astype(np.float64) - want) / np.linalg.norm(want))}
    return out


# Seeded configurations rendered with the reference GPU path.  Sampling is
# deterministic (regular grid, concentration off); the source is placed by
# render_source_flare's angular offset from the solved centre of the frame.
CASES = {
    "cfg1": dict(lens="cfg1_double_gauss_12", W=512, H=512, ray_grid=32, spectral_samples=8,
                 min_ghost_intensity=1e-7, angle=(math.radians(10.0), 0.0), gain=1000.0),
    "cfg2": dict(lens="cfg2_wide_angle_24", W=512, H=512, ray_grid=128, spectral_samples=31,
                 min_ghost_intensity=1e-6, angle=(math.radians(15.0), 0.0), gain=1000.0),
    "cfg4": dict(lens="cfg4_anamorphic_18", W=512, H=256, ray_grid=128, spectral_samples=31,
                 min_ghost_intensity=1e-7, angle=(math.radians(7.0), math.radians(5.0)), gain=1000.0),
}


def seeded(pins, meta):
    images, info = {}, {}
    for name, c in CASES.items():
        raw, focal, cal = _lens(pins, meta, c["lens"])
        centre = R.solve_source(raw, cal, 0.0, 0.0, cal["sensor_half_w"], cal["sensor_half_h"])
        off = np.array([[c["angle"][0] - centre["angle_x"], c["angle"][1] - centre["angle_y"], 1.0]], np.float32)
        cfg = R.RefGpuCfg(ray_grid=c["ray_grid"], spectral_samples=c["spectral_samples"], pupil_jitter=0,
                          jitter_seed=0, sensor_half_w=cal["sensor_half_w"], sensor_half_h=cal["sensor_half_h"],
                          flare_gain=c["gain"], min_ghost_intensity=c["min_ghost_intensity"], cull_dead_pairs=1,
                          concentrate_samples=0, source_x=0.5, source_y=0.5)
        g, _, ms, _ = R.gpu_render(raw, c["W"], c["H"], cfg, calib=cal, focal_length=focal, offsets=off)
        images[name + "/image"] = g
        info[name] = dict(c, centre=centre, offset=off[0].tolist(), calibration=cal, ms=ms,
                          source_angle=[float(np.float32(centre["angle_x"]) + off[0, 0]),
                                        float(np.float32(centre["angle_y"]) + off[0, 1])])
    return images, info


# Layers of render_point_flare on the seeded configuration-1 lens (512^2,
# 8 wavelengths): the veiling glare (veil_render.cu:243), and the starburst by
# the matrix-DFT engine (a 1024 grid at scale_trim 15: an 87-pixel window,
# below the reference's "prominent" switch) and by the SPRITE engine, on axis
# and off axis (the cat's-eye effective pupil).
LAYERS = {
    "veil": dict(source_xy=(0.62, 0.44), veil=True),
    "mdft": dict(source_xy=(0.5, 0.5), starburst=True, engine=1, grid=1024, trim=15.0),
    "sprite": dict(source_xy=(0.5, 0.5), starburst=True, engine=0, grid=1024, trim=15.0),
    "sprite_offaxis": dict(source_xy=(0.9, 0.3), starburst=True, engine=0, grid=1024, trim=15.0),
}


def layers(pins, meta):
    images, info = {}, {}
    raw, focal, cal = _lens(pins, meta, "cfg1_double_gauss_12")
    for name, c in LAYERS.items():
        cfg = R.RefGpuCfg(ray_grid=32, spectral_samples=8, pupil_jitter=0, jitter_seed=0,
                          sensor_half_w=cal["sensor_half_w"], sensor_half_h=cal["sensor_half_h"], flare_gain=1000.0,
                          min_ghost_intensity=1e-7, cull_dead_pairs=1, concentrate_samples=0,
                          source_x=c["source_xy"][0], source_y=c["source_xy"][1], source_r=10.0, source_g=10.0,
                          source_b=10.0, veil=int(c.get("veil", False)), starburst=int(c.get("starburst", False)),
                          starburst_engine=c.get("engine", 0), starburst_grid=c.get("grid", 1024), pupil_fill=0.3,
                          scale_trim=c.get("trim", 1.0), sb_spectral_samples=8)
        g, star, ms, _, vl = R.gpu_render(raw, 512, 512, cfg, calib=cal, focal_length=focal,
                                          starburst=bool(c.get("starburst")), veil=True)
        images["layer_" + name + "/image"] = vl if c.get("veil") else star
        info["layer_" + name] = dict(c, lens="cfg1_double_gauss_12", W=512, H=512, ms=ms, calibration=cal,
                                     key="veil" if c.get("veil") else "starburst")
    return images, info


def timing(pins, meta, reps=5):
    """The configuration-2 frame: the reference at 256^2 grids with its
    deterministic sampling, and with its default concentrated sampling and
    adaptive budgets (a different, Monte-Carlo estimator)."""
    raw, focal, cal = _lens(pins, meta, "cfg2_wide_angle_24")
    centre = R.solve_source(raw, cal, 0.0, 0.0, cal["sensor_half_w"], cal["sensor_half_h"])
    off = np.array([[math.radians(15.0) - centre["angle_x"], -centre["angle_y"], 1.0]], np.float32)
    res = {}
    for tag, conc in (("grid256_concentration_off", 0), ("grid256_default_concentrated", 1)):
        cfg = R.RefGpuCfg(ray_grid=256, spectral_samples=31, sensor_half_w=cal["sensor_half_w"],
                          sensor_half_h=cal["sensor_half_h"], flare_gain=1000.0, min_ghost_intensity=1e-6,
                          cull_dead_pairs=1, concentrate_samples=conc, adaptive_sample_budgets=conc)
        R.gpu_render(raw, 2048, 2048, cfg, calib=cal, focal_length=focal, offsets=off)   # warm
        walls = []
        for _ in range(reps):
            _, _, ms, _ = R.gpu_render(raw, 2048, 2048, cfg, calib=cal, focal_length=focal, offsets=off)
            walls.append(ms)
        cfg.collect_stats = 1
        _, _, _, st = R.gpu_render(raw, 2048, 2048, cfg, calib=cal, focal_length=focal, offsets=off)
        res[tag] = {"wall_ms_median": float(np.median(walls)), "wall_ms": walls, "stats": st}
    return res


def pack_into_fixtures(src_dir):
    from make_refgolden import pack   # same directory
    src = pathlib.Path(src_dir)
    imgs = np.load(src / "refgpu_images.npz")
    meta = json.loads((src / "refgpu_meta.json").read_text())
    out = {}
    for k in imgs.files:
        out[k] = pack(imgs[k])
        meta[k.split("/")[0]]["shape"] = list(imgs[k].shape)
    meta["selfcheck"] = json.loads((src / "refgpu_selfcheck.json").read_text())
    np.savez_compressed(HERE / "refgpu_seeded.npz", **out)
    (HERE / "refgpu_seeded.json").write_text(json.dumps(meta, indent=1))
    print("refgpu_seeded.npz", (HERE / "refgpu_seeded.npz").stat().st_size // 1024, "KB")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=str(HERE))
    ap.add_argument("--skip-timing", action="store_true")
    ap.add_argument("--pack", default="")
    args = ap.parse_args()
    if args.pack:
        sys.path.insert(0, str(HERE))
        pack_into_fixtures(args.pack)
        return
    out = pathlib.Path(args.out)
    out.mkdir(parents=True, exist_ok=True)
    pins = np.load(HERE / "ref_pins.npz")
    imgs = np.load(HERE / "ref_images.npz")
    meta = json.loads((HERE / "ref_meta.json").read_text())
    t0 = time.time()
    R._load_gpu()
    print("reference GPU library built in %.1f s" % (time.time() - t0), flush=True)
    chk = selfcheck(pins, meta, imgs)
    (out / "refgpu_selfcheck.json").write_text(json.dumps(chk, indent=1))
    print(json.dumps(chk), flush=True)
    images, info = seeded(pins, meta)
    li, lm = layers(pins, meta)
    images.update(li)
    info.update(lm)
    np.savez_compressed(out / "refgpu_images.npz", **images)
    (out / "refgpu_meta.json").write_text(json.dumps(info, indent=1, default=float))
    if not args.skip_timing:
        t = timing(pins, meta)
        (out / "refgpu_timing.json").write_text(json.dumps(t, indent=1))
        print(json.dumps(t), flush=True)


if __name__ == "__main__":
    main()
