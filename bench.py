"""Flare hot-path benchmark (one JSON line on rank 0).

Workload (the configuration the metric is quoted on): the seeded 24-surface
wide-angle prescription with two even aspheres, ~250 two-reflection ghost
pairs culled at relative energy 1e-6 by the device culler, per-ghost
adaptive pupil grids 16^2..256^2 sized from each ghost's probe footprint, 31
wavelengths over 400-700 nm, one source at 15 deg field, 2048x2048 float32
RGB output.  A step is one frame of the ghost layer: the batched form is one
persistent work-queue launch (plus the colour-correction flush) replayed from
a CUDA graph; the plain form launches the same kernel once per ghost pair.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Multi-GPU: replicas only (every rank renders its own frames; no collective on
the data path); value = frames of all ranks / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import pathlib
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

# every in-flight serving request has its own stream: give each its own
# hardware work queue (must be set before CUDA starts in this process)
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

REPO = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(REPO))

METRIC = "flare frames/s & ghost rays/s (served+batched vs plain, ≤1e-3 relL2); p50/p99 lat"
UNIT = "frames/s"
W = H = 2048
N_SPEC = 31
SOURCE_DEG = 15.0
MIN_INTENSITY = 1e-6
GOLDEN = REPO / "tests" / "golden"


_T0 = time.perf_counter()


def _progress(what: str) -> None:
    """One line on stderr per finished section: where a long run spends its time."""
    print("[bench +%.1fs] %s" % (time.perf_counter() - _T0, what), file=sys.stderr, flush=True)


def _workload(name="cfg2_wide_angle_24"):
    """Seeded config-2 lens (or another seeded fixture lens) and its
    calibration (the reference's calibrate_lens values for the same records,
    committed as a fixture)."""
    from ghostlight_gb300._abi import gl_surface
    from ghostlight_gb300.optics import OpticalSystem
    pins = np.load(GOLDEN / "ref_pins.npz")
    raw = pins[name + "/lens"]
    recs = list((gl_surface * raw.shape[0]).from_buffer_copy(raw.tobytes()))
    meta = json.loads((GOLDEN / "ref_meta.json").read_text())
    cal = meta[name]["calibration"]
    return OpticalSystem.from_records(recs, name=name), cal


def _config():
    import ghostlight_gb300 as gl
    return gl.FlareConfig(spectral_samples=N_SPEC, min_ghost_intensity=MIN_INTENSITY,
                          adaptive_grids=True, adaptive_grid_min=16, adaptive_grid_max=256,
                          flare_gain=1000.0)


def _sources():
    return np.array([[math.radians(SOURCE_DEG), 0.0, 1.0, 1.0, 1.0]], np.float32)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def _peaks():
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "fallback": True}


def _flush_l2(buf):
    buf.add_(1.0)   # 512 MB write, larger than the 129 MB L2


def run_gpu(args, rank, world):
    import torch
    import ghostlight_gb300 as gl
    from ghostlight_gb300 import _native
    from ghostlight_gb300.flare import prepare_ghost_render, filter_ghosts_device

    dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", 0)))
    torch.cuda.set_device(dev)
    lens, cal = _workload()
    cfg = _config()
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    src = _sources()
    fr = filter_ghosts_device(lens, hw, hh, cfg)
    plan = prepare_ghost_render(lens, src, W, H, cfg, hw, hh, filter_result=fr)
    plain = prepare_ghost_render(lens, src, W, H, cfg, hw, hh, filter_result=fr, plain_per_pair=True)
    outs = [torch.zeros((H, W), dtype=torch.float32, device=dev) for _ in range(3)]
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream(device=dev)

    # ---- launch shape picked by the autotuner on this workload ----
    from ghostlight_gb300.autotune import Tuner, tune_ghost_plan
    tuner = Tuner(reps=3)
    tune_ghost_plan(plan, outs, stream=stream, tuner=tuner)
    _progress("autotune")

    # ---- batched form: graph-captured launch ----
    # Events around the render launch are captured into the graph (external
    # event-record nodes), so every timed replay also times the render kernel
    # alone on its own stream.
    kev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    plan.set_timing(*kev)
    with torch.cuda.stream(stream):
        for _ in range(2):
            plan.execute(*outs, stream=stream.cuda_stream)
        stream.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            launches_per_step = plan.execute(*outs, stream=stream.cuda_stream)

    def timed(fn, steps, warm, after=None):
        with torch.cuda.stream(stream):
            for _ in range(warm):
                fn()
            stream.synchronize()
            ts = []
            for _ in range(steps):
                _flush_l2(flush)
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                fn()
                e1.record(stream)
                e1.synchronize()
                ts.append(e0.elapsed_time(e1) / 1e3)
                if after is not None:
                    after()
        return ts

    kernel_ms = {"probe": [], "render": []}

    def read_kernel_events():
        kernel_ms["probe"].append(kev[0].elapsed_time(kev[1]))
        kernel_ms["render"].append(kev[1].elapsed_time(kev[2]))

    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev.index) as clk:
        t_batched = timed(graph.replay, args.steps, args.warmup, after=read_kernel_events)
        _progress("batched frames")
    torch.cuda.synchronize()
    plan.set_timing()
    frame_host = torch.stack(outs).cpu().numpy()       # the frame of the last timed replay
    traced_render, traced_probe = plan.traced_split()
    if args.quick:
        t_plain = [float("nan")]
    else:
        t_plain = timed(lambda: plain.execute(*outs, stream=stream.cuda_stream), max(2, min(args.steps, 5)),
                        max(1, min(args.warmup, 2)))

    # ---- e2e through the public API: host inputs in, host image out ----

    # Frames are pipelined the way an application streams them: the host
    # prepares frame k+1 (device culler, grids, plan upload) while the device
    # renders frame k and copies it out; each frame's own work is complete
    # (its planes in pinned host memory) before the frame after next starts.
    outs2 = [[torch.zeros((H, W), dtype=torch.float32, device=dev) for _ in range(3)] for _ in range(2)]
    host2 = [torch.empty((3, H, W), dtype=torch.float32).pin_memory() for _ in range(2)]
    done = [torch.cuda.Event(), torch.cuda.Event()]

    def e2e_run(n):
        # Frame k+1's device culler (a synchronous call) runs between frame
        # k-1's and frame k's renders, and frame k+1's plan is built on the
        # host while frame k renders, so the device waits for no host work.
        with torch.cuda.stream(stream):
            t0 = time.perf_counter()
            prev = None
            cur = prepare_ghost_render(lens, src, W, H, cfg, hw, hh,
                                       filter_result=filter_ghosts_device(lens, hw, hh, cfg))
            for k in range(n):
                fr_next = filter_ghosts_device(lens, hw, hh, cfg) if k + 1 < n else None
                o = outs2[k % 2]
                cur.execute(*o, stream=stream.cuda_stream)
                for c in range(3):
                    host2[k % 2][c].copy_(o[c], non_blocking=True)
                done[k % 2].record(stream)
                if prev is not None:                     # frame k-1 landed in host memory: release its plan
                    done[(k - 1) % 2].synchronize()
                    prev.close()
                prev = cur
                if fr_next is not None:
                    cur = prepare_ghost_render(lens, src, W, H, cfg, hw, hh, filter_result=fr_next)
            done[(n - 1) % 2].synchronize()
            prev.close()
            return time.perf_counter() - t0

    n_e2e = 0 if args.quick else max(4, min(args.steps, 10))
    if n_e2e:
        e2e_run(2)                                        # warm
        te = [e2e_run(n_e2e) / n_e2e] * n_e2e
        _progress("end-to-end frames")
    else:
        te = [float("nan")]
    h2d = int(lens.num_surfaces() * 192 + 2 * N_SPEC * lens.num_surfaces() * 4 + N_SPEC * 16 +
              sum(len(g) for g in plan.grids) * 8 + plan.n_items * 16 + len(plan.pairs) * 16 + 32)
    d2h = 3 * W * H * 4

    traced = plan.traced()            # traces of the last (timed) execute: deterministic per frame
    cfg1 = None
    if not args.quick:
        with torch.cuda.stream(stream):
            cfg1 = run_cfg1(args, dev, stream, timed)
        _progress("configuration 1")
    cfg3 = frame_res = None
    if not args.quick or args.only == "cfg3":
        with torch.cuda.stream(stream):
            cfg3, sb_inputs = run_cfg3(args, dev, stream, flush, timed)
            _progress("starburst precision / convolution / sprite")
            if not args.quick:
                frame_res = run_full_frame(args, dev, stream, timed, plan, plain, sb_inputs, sb_inputs[4])
            sb_inputs[4].close()
    value, sec = replica_rate(float(sum(t_batched)), args.steps, world, dev)
    frames = args.steps * world
    ms_step = 1e3 * sec / args.steps
    rays_per_s = traced * frames / sec
    plain_fps = len(t_plain) / sum(t_plain)
    res = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": frame_config(len(plan.pairs)),
        "frame": {"kept_pairs": int((plan.pair_hits() > 0).sum()) if hasattr(plan, "pair_hits") else None,
                  "render_traces": traced_render, "probe_traces": traced_probe, "grid_sides": plan.grid_sides},
        "rays_per_s": rays_per_s,
        "kernel_ms": {"render": float(np.mean(kernel_ms["render"])), "probe": float(np.mean(kernel_ms["probe"])),
                      "how": "CUDA events captured into the replayed graph around each launch, every timed step"},
        "traces_render": traced_render, "traces_probe": traced_probe,
        "ray_lambda_traces_per_frame": traced,
        "frame_ray_lambda_before_cull": plan.rays,
        "plain_per_pair": {"value": plain_fps, "unit": UNIT, "ms_per_step": 1e3 / plain_fps,
                           "launches_per_step": len(plan.pairs) + 1},
        "speedup_batched_vs_plain": value / world / plain_fps,
        "e2e": {"value": len(te) / sum(te), "unit": UNIT, "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "path": "per frame: the device culler (filter_ghosts_device), "
                "prepare_ghost_render (grids, uploads), execute and the pinned D2H of the 3 planes; frames "
                "pipelined: frame k+1's culler runs between frames k-1 and k, its plan is built on the host "
                "while frame k renders"},
        "gpu_launches": int(launches_per_step) * args.steps,
        "clocks": clk.summary(),
        "autotune": tuner.log,
    }
    if cfg1 is not None:
        res["cfg1"] = cfg1
    if cfg3 is not None:
        res["starburst_psf"] = cfg3
    if frame_res is not None:
        res["full_flare_frame"] = frame_res
    return res, plan, frame_host


def replica_rate(sec, steps, world, device=None):
    """Whole-job frames/s of `world` independent replicas (one rank per GPU,
    no exchange on the data path): every rank timed `steps` frames in `sec`
    seconds; the job's time is the slowest rank's (max over ranks, an
    all-reduce over the initialised process group: NCCL on GPUs, gloo on the
    host), and the job rendered steps x world frames.  Returns (frames/s,
    job seconds)."""
    if world > 1:
        import torch
        t = torch.tensor([float(sec)], dtype=torch.float64, device=device)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        sec = float(t.item())
    return steps * world / sec, sec


# ---- configuration 1: the plain small frame ------------------------------------
def run_cfg1(args, dev, stream, timed):
    """Configuration 1 on the GPU: the seeded 12-surface double Gauss (6-blade
    stop), the 2-reflection pairs of the device culler at 1e-7 that do not
    cross the stop, a 32^2 pupil grid, 8 wavelengths, a 10 deg source,
    512^2 float32 RGB, the off-sensor cull on (as the reference arm's cfg1
    CPU frame), batched (one graph) against the per-pair launches; and its
    starburst, the split-BF16 matrix DFT of the device-built 256^2 stop
    pupil to 512^2 at the same 8 wavelengths, alone and added to the frame
    in the same graph."""
    import torch
    import ghostlight_gb300 as gl
    from ghostlight_gb300.flare import GhostRenderPlan, filter_ghosts_device, pupil_grid, spectral_table
    from ghostlight_gb300.prescriptions import stop_crossing
    from ghostlight_gb300.starburst import MdftPlan, build_pupil
    lens, cal = _workload("cfg1_double_gauss_12")
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    fr = filter_ghosts_device(lens, hw, hh, gl.FlareConfig(min_ghost_intensity=1e-7))
    keep = np.array([not stop_crossing(lens.records(), int(a), int(b)) for a, b in fr.pairs], bool)
    pairs, boosts = fr.pairs[keep], fr.boosts[keep]
    spec, corr = spectral_table(8)
    grid = pupil_grid(lens, 32)
    src = np.array([[math.radians(10.0), 0.0, 1.0, 1.0, 1.0]], np.float32)
    W1 = H1 = 512
    mk = lambda plain: GhostRenderPlan(lens, pairs, boosts, src, [grid], None, spec, corr, W1, H1, hw, hh, 1000.0,
                                       apply_correction=True, plain_per_pair=plain, cull_dead_pairs=not plain)
    plan, plain = mk(False), mk(True)
    outs = torch.zeros((3, H1, W1), device=dev)
    n_sb = 256
    lam = spec[:, 0].astype(np.float64)
    s = (1.0 / (2.0 * n_sb)) * 550.0 / lam
    sb = MdftPlan(n_sb, W1, s, s, (spec[:, 1:4] / 1e3).astype(np.float32), "split_bf16",
                  center_x=W1 / 2.0, center_y=H1 / 2.0)
    pupil = build_pupil(lens, n_sb, 0.3)
    for _ in range(2):
        plan.execute(outs[0], outs[1], outs[2], stream=stream.cuda_stream)
        sb.execute(pupil, outs[0], outs[1], outs[2], stream=stream.cuda_stream, accumulate=True)
    stream.synchronize()
    g_ghost, g_frame = torch.cuda.CUDAGraph(), torch.cuda.CUDAGraph()
    with torch.cuda.graph(g_ghost, stream=stream):
        plan.execute(outs[0], outs[1], outs[2], stream=stream.cuda_stream)
    with torch.cuda.graph(g_frame, stream=stream):
        plan.execute(outs[0], outs[1], outs[2], stream=stream.cuda_stream)
        sb.execute(pupil, outs[0], outs[1], outs[2], stream=stream.cuda_stream, accumulate=True)
    steps, warm = max(args.steps, 10), max(args.warmup, 3)
    t_ghost = timed(g_ghost.replay, steps, warm)
    stream.synchronize()
    got = outs.cpu().numpy().astype(np.float64)       # the ghost frame of the last timed replay
    t_frame = timed(g_frame.replay, steps, warm)
    t_sb = timed(lambda: sb.execute(pupil, outs[0], outs[1], outs[2], stream=stream.cuda_stream), steps, warm)
    t_plain = timed(lambda: plain.execute(outs[0], outs[1], outs[2], stream=stream.cuda_stream), steps, warm)
    traced = plan.traced()
    status = sb.status()
    kept = plan.pair_hits() > 0
    plan.close(); plain.close(); sb.close()
    # the frame and its inputs, for the FP64 check of the CPU leg (cfg1_parity)
    _CFG1_CHECK[:] = [lens, pairs[kept], boosts[kept], src, grid, spec, corr, hw, hh, W1, H1, got]
    fps = len(t_ghost) / sum(t_ghost)
    plain_fps = len(t_plain) / sum(t_plain)
    return {"workload": "cfg1: seeded 12-surface double Gauss, %d non-stop-crossing pairs (device culler at "
                        "1e-7), 32^2 grid, 8 wavelengths, 10 deg, 512^2, off-sensor cull on; starburst: "
                        "split-BF16 matrix DFT of the 256^2 stop pupil to 512^2 x 8 wavelengths" % len(pairs),
            "ghost_frames_per_s": fps, "ghost_ms": 1e3 / fps, "ray_lambda_traces": traced,
            "plain_frames_per_s": plain_fps, "speedup_batched_vs_plain": fps / plain_fps,
            "starburst_ms": 1e3 * float(np.median(t_sb)), "starburst_status": status,
            "frame_frames_per_s": len(t_frame) / sum(t_frame),
            "l2": "flushed between timed steps"}


_CFG1_CHECK: list = []


def cfg1_parity():
    """The CPU leg's check of the configuration-1 frame the GPU rendered in
    its timed loop: the FP64 oracle's render of the same kept pairs, grid,
    spectrum and colour correction; relative L2 and the largest per-pixel
    error relative to the frame's peak."""
    from oracle import oracle as O
    lens, pairs, boosts, src, grid, spec, corr, hw, hh, W1, H1, got = _CFG1_CHECK
    want = O.render(lens.records(), pairs, boosts, src, [grid], spec, hw, hh, W1, H1, 1000.0, fp64=True,
                    n_threads=os.cpu_count() or 1)
    want = np.einsum("ij,jhw->ihw", corr.astype(np.float64), want)
    rel = float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300))
    mx = float(np.abs(got - want).max() / max(float(np.abs(want).max()), 1e-300))
    return {"rel_l2": rel, "max_err_rel_peak": mx, "tolerance": 1e-3, "pass": rel <= 1e-3,
            "against": "FP64 oracle, the %d pairs the off-sensor cull kept, 512^2 x 3 planes, same grid / spectral "
                       "table / colour correction" % len(pairs)}


# ---- starburst precision sweep + PSF/veil convolution (cfg3) -----------------
SB_N, SB_K = 512, 2048          # pupil side -> output side
SB_S0 = 400.0 / 550.0 / 2048.0  # DFT scale at 550 nm: the 400 nm pattern period spans the 2048 frame
CONV_K = 257


def _sb_inputs(dev):
    import torch
    from ghostlight_gb300.apertures import curved_blade_mask
    from ghostlight_gb300.flare import spectral_table
    A = curved_blade_mask(SB_N, blades=9, curvature=0.35, aa_px=2.0, dust_density=0.005, dust_r=(1.0, 4.0),
                          seed=3)
    spec, _ = spectral_table(N_SPEC)
    lam = spec[:, 0].astype(np.float64)
    sx = SB_S0 * 550.0 / lam
    sy = sx.copy()
    # cmf weights x (lambda_ref / lambda)^2, normalised so the zero-order peak is ~1
    w = spec[:, 1:4].astype(np.float64) * (550.0 / lam)[:, None] ** 2 / float(A.astype(np.float64).sum()) ** 2
    return torch.from_numpy(A).to(dev), sx, sy, w.astype(np.float32)


def _eform_fp64(A, K, sx, sy, cx, cy, w):
    """FP64 evaluation of the same field form with cuBLAS ZGEMM (the check for
    the full-size outputs; the numpy oracle pins the kernels in the tests)."""
    import torch
    dev = A.device
    n = A.shape[0]
    j = torch.arange(n, dtype=torch.float64, device=dev) - 0.5 * (n - 1)
    k = torch.arange(K, dtype=torch.float64, device=dev)
    A64 = A.to(torch.float64).to(torch.complex128)
    out = torch.zeros((3, K, K), dtype=torch.float64, device=dev)

    def W(s, c):
        ph = s * torch.outer(k - c, j)
        ph = ph - torch.round(ph)
        return torch.polar(torch.ones_like(ph), -2.0 * math.pi * ph)

    for l in range(len(sx)):
        E = W(float(sy[l]), cy) @ (A64 @ W(float(sx[l]), cx).T)
        I = E.real ** 2 + E.imag ** 2
        for c in range(3):
            out[c] += float(w[l, c]) * I
    return out


def _errs(got, ref):
    import torch
    g = torch.stack([x.to(torch.float64) for x in got]) if isinstance(got, (list, tuple)) else got.to(torch.float64)
    d = g - ref
    return {"rel_l2": float(torch.linalg.vector_norm(d) / torch.linalg.vector_norm(ref)),
            "max_err_rel_peak": float(d.abs().max() / ref.abs().max())}


def _conv_points(img_planes, kern, out_planes, n_pts=64, seed=3):
    """Direct FP64 sums of the 'same' convolution at n_pts pixels (corners,
    centre and seeded random ones) -> relative L2 over those pixels."""
    import torch
    H, W_ = img_planes[0].shape
    kh, kw = kern.shape
    rng = np.random.default_rng(seed)
    ys = np.concatenate([[0, 0, H - 1, H - 1, H // 2], rng.integers(0, H, n_pts - 5)])
    xs = np.concatenate([[0, W_ - 1, 0, W_ - 1, W_ // 2], rng.integers(0, W_, n_pts - 5)])
    kf = torch.flip(kern.to(torch.float64), (0, 1))
    num = den = 0.0
    for img, out in zip(img_planes, out_planes):
        pad = torch.nn.functional.pad(img.to(torch.float64)[None, None], (kw // 2, kw // 2, kh // 2, kh // 2))[0, 0]
        for y, x in zip(ys, xs):
            want = float((pad[y:y + kh, x:x + kw] * kf).sum())
            got = float(out[y, x])
            num += (got - want) ** 2
            den += want ** 2
    return math.sqrt(num / den) if den > 0 else 0.0


def run_cfg3(args, dev, stream, flush, timed):
    """Starburst forms at 512^2 -> 2048^2 x 31 wavelengths and the 2048^2 x 3
    (*) 257^2 convolution: times, errors, rooflines."""
    import torch
    import ghostlight_gb300 as gl
    from ghostlight_gb300.starburst import flops_per_lambda
    peaks = _peaks()
    A, sx, sy, w = _sb_inputs(dev)
    cx = cy = SB_K / 2.0
    ref = _eform_fp64(A, SB_K, sx, sy, cx, cy, w)
    flops = flops_per_lambda(SB_N, SB_K) * N_SPEC
    sb = [torch.zeros((SB_K, SB_K), dtype=torch.float32, device=dev) for _ in range(3)]
    forms = {}
    peak_tc = {"split_bf16": peaks["bf16_tflops"] / 3.0, "tf32": peaks["bf16_tflops"] / 2.0,
               "fp32": FP32_PEAK_TFLOPS}
    from ghostlight_gb300.autotune import Tuner, tune_mdft_plan
    tuner = Tuner(reps=3)
    for form in ("split_bf16", "tf32", "fp32"):
        plan = gl.MdftPlan(SB_N, SB_K, sx, sy, w, form, cx, cy, stream=stream.cuda_stream)
        if form != "fp32":
            tune_mdft_plan(plan, A, sb, stream=stream, tuner=tuner)
        steps = args.steps if form != "fp32" else max(2, min(args.steps, 5))
        ts = timed(lambda: plan.execute(A, *sb, stream=stream.cuda_stream), steps, args.warmup)
        stream.synchronize()
        if plan.status() != 0:
            raise RuntimeError("mdft %s: device wait timed out" % form)
        sec = sum(ts) / len(ts)
        ach = flops / sec / 1e12
        forms[form] = dict(ms=1e3 * sec, tflops_algorithmic=ach, launch=getattr(plan, "launch", None),
                           **_errs(sb, ref),
                           roofline={"bound": "tensor" if form != "fp32" else "fp32", "achieved": ach,
                                     "peak": peak_tc[form], "unit": "TFLOP/s", "frac": ach / peak_tc[form],
                                     "peak_note": {"split_bf16": "measured cuBLAS bf16 burst / 3 (three "
                                                                 "BF16 products per algorithmic MAC)",
                                                   "tf32": "measured cuBLAS bf16 burst / 2 (TF32 rate is "
                                                           "half of BF16)",
                                                   "fp32": "FP32 CUDA-core peak at max SM clock"}[form]})
        plan.close()
    del ref
    # ---- convolution of a 2048^2 x 3 flare image with the 257^2 kernel ----
    kern = gl.synthetic_psf_kernel(CONV_K, seed=11)
    conv = gl.ConvPlan(W, H, kern, stream=stream.cuda_stream)
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    img = [torch.rand((H, W), generator=g, device=dev) ** 8 for _ in range(3)]
    cout = [torch.empty((H, W), dtype=torch.float32, device=dev) for _ in range(3)]
    ts = timed(lambda: conv.execute(img, cout, stream=stream.cuda_stream), args.steps, args.warmup)
    stream.synchronize()
    csec = sum(ts) / len(ts)
    cbytes = conv.traffic_bytes()
    gbs = cbytes / csec / 1e9
    conv_res = {"ms": 1e3 * csec, "P": conv.P, "Q": conv.Q, "route": "FFT, 3 HBM passes",
                "rel_l2_64px_vs_fp64_direct": _conv_points(img, torch.from_numpy(kern).to(dev), cout),
                "direct_equivalent_tflops": 2.0 * W * H * CONV_K * CONV_K * 3 / csec / 1e12,
                "roofline": {"bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                             "frac": gbs / peaks["hbm_gbs"], "algorithmic_bytes": cbytes}}
    # ---- SPRITE engine: one 2048^2 FFT of the pupil, bake + box sum, splat ----
    from ghostlight_gb300.starburst import SpritePlan
    SN, SDS = 2048, 2
    padded_pupil = torch.zeros((SN, SN), dtype=torch.float32, device=dev)
    o = (SN - A.shape[0]) // 2
    padded_pupil[o:o + A.shape[0], o:o + A.shape[1]] = A
    from ghostlight_gb300.flare import spectral_table
    sspec, _ = spectral_table(N_SPEC)
    splan = SpritePlan(SN, sspec)
    sout = [torch.zeros((H, W), dtype=torch.float32, device=dev) for _ in range(3)]
    ssrc = np.array([[W / 2 + 0.3, H / 2 - 0.2, 1.0, 1.0, 1.0]], np.float32)
    px_mm = 0.018
    sx_ds = px_mm / 1.5
    srx = int(math.ceil(0.5 * (SN // SDS) * sx_ds / px_mm)) + 1
    ts_b = timed(lambda: splan.bake(padded_pupil, SDS, stream=stream.cuda_stream), args.steps, args.warmup)
    ts_s = timed(lambda: splan.splat(ssrc, sx_ds, sx_ds, px_mm, px_mm, srx, srx, 1.0, *sout,
                                     stream=stream.cuda_stream), args.steps, args.warmup)
    stream.synchronize()
    splan.close()
    bsec, ssec = sum(ts_b) / len(ts_b), sum(ts_s) / len(ts_s)
    # HBM bytes of the bake: pupil read 4 + row-FFT write 8 + column read 8 + PSF write 4
    # + PSF read 4 per grid point, sprite write 12 per coarse texel
    bbytes = SN * SN * 28.0 + 12.0 * (SN // SDS) ** 2
    # The wavelength bake reads the 16 MB PSF (L2-resident) through L1 with
    # 4 bilinear 4-byte taps per fine texel and wavelength: its bound is the
    # L1 load path, not HBM (ncu on the bake kernel: L1 72% busy, 4.09 GB of
    # L1 loads and 16.8 MB of DRAM reads per launch).  Algorithmic tap bytes:
    # (SN/ds)^2 coarse texels x ds^2 fine texels x wavelengths x 4 taps x 4 B,
    # against the nominal L1 load bandwidth (128 B per clock per SM).
    gbytes = float((SN // SDS) ** 2 * SDS * SDS * N_SPEC * 4 * 4)
    l1_peak = 152 * 128 * 2.070e9 / 1e9
    sprite_res = {"grid": SN, "ds": SDS, "wavelengths": N_SPEC, "bake_ms": 1e3 * bsec, "splat_ms": 1e3 * ssec,
                  "splat_footprint_px": (2 * srx + 1) ** 2,
                  "roofline_bake": {"bound": "l1", "achieved": gbytes / bsec / 1e9, "peak": l1_peak,
                                    "unit": "GB/s", "frac": gbytes / bsec / 1e9 / l1_peak,
                                    "algorithmic_bytes": gbytes,
                                    "peak_note": "nominal L1 load bandwidth: 152 SMs x 128 B x 2.07 GHz",
                                    "hbm": {"bytes": bbytes, "achieved": bbytes / bsec / 1e9,
                                            "frac": bbytes / bsec / 1e9 / peaks["hbm_gbs"]},
                                    "note": "the whole bake (two FFT passes + the wavelength bake) is timed; "
                                            "ncu: the bake kernel's L1 is 72% busy, its 4-byte taps spanning "
                                            "several 32-byte sectors per warp (4.09 GB moved for 2.08 GB of "
                                            "taps); HBM carries 1/250 of that"}}
    return {"autotune": tuner.log, "sprite": sprite_res,
            "workload": "512^2 9-blade curved-blade pupil (2 px AA, 0.5%% dust r 1-4 px) -> %d^2, %d wavelengths; "
                        "conv %dx%d x3 (*) %d^2 FP32" % (SB_K, N_SPEC, W, H, CONV_K),
            "gflop_algorithmic": flops / 1e9, "mdft": forms, "conv": conv_res}, (A, sx, sy, w, conv, kern)


def run_full_frame(args, dev, stream, timed, ghost_plan, plain_plan, sb_inputs, conv):
    """Full flare frame: ghost layer (cfg2) + split-BF16 starburst at the
    source's image position + PSF/veil convolution of the composite, one
    CUDA graph; against the plain form (per-pair ghost launches, the same
    starburst and convolution, no graph)."""
    import torch
    import ghostlight_gb300 as gl
    A, sx, sy, w = sb_inputs[:4]
    # the starburst is centred on the source's paraxial image point, f tan(theta) on the sensor
    # (for the 15 deg source of this lens that is beyond the frame edge: the frame shows the
    # starburst's outer rays, and the work per frame is the same)
    _, cal = _workload()
    x_mm = cal["focal_length_x"] * math.tan(math.radians(SOURCE_DEG))
    cx, cy = (x_mm / (2.0 * cal["sensor_half_w"]) + 0.5) * W, 0.5 * H
    sbp = gl.MdftPlan(SB_N, SB_K, sx, sy, w, "split_bf16", cx, cy, stream=stream.cuda_stream)
    ghost = [torch.zeros((H, W), dtype=torch.float32, device=dev) for _ in range(3)]
    star = [torch.zeros((H, W), dtype=torch.float32, device=dev) for _ in range(3)]
    final = [torch.zeros((H, W), dtype=torch.float32, device=dev) for _ in range(3)]

    side = torch.cuda.Stream()

    def frame(gp):
        # the starburst does not depend on the ghost layer: it runs on a side
        # stream beside the ghost launches, and the convolution joins both
        fork = torch.cuda.Event()
        fork.record(stream)
        side.wait_event(fork)
        n = sbp.execute(A, *star, stream=side.cuda_stream)
        n += gp.execute(*ghost, stream=stream.cuda_stream)
        join = torch.cuda.Event()
        join.record(side)
        stream.wait_event(join)
        n += conv.execute(ghost, final, add=star, stream=stream.cuda_stream)
        return n

    with torch.cuda.stream(stream):
        for _ in range(2):
            frame(ghost_plan)
        stream.synchronize()
        graph = torch.cuda.CUDAGraph()
        with torch.cuda.graph(graph, stream=stream):
            launches = frame(ghost_plan)
    tb = timed(graph.replay, args.steps, args.warmup)
    tp = timed(lambda: frame(plain_plan), max(2, min(args.steps, 5)), max(1, min(args.warmup, 2)))
    stream.synchronize()
    if sbp.status() != 0:
        raise RuntimeError("mdft: device wait timed out")
    sbp.close()
    fps = len(tb) / sum(tb)
    pfps = len(tp) / sum(tp)
    return {"value": fps, "unit": UNIT, "ms_per_step": 1e3 / fps, "launches_per_step": int(launches),
            "plain_value": pfps, "plain_ms_per_step": 1e3 / pfps, "speedup_batched_vs_plain": fps / pfps,
            "layers": "ghosts (cfg2) + split-BF16 starburst 512^2->2048^2 x 31 wavelengths + conv 257^2 "
                      "of the composite"}


# ---- serving (Poisson request mix) -----------------------------------------
SERVE_RATE = 200.0
SERVE_LENSES = 24
SERVE_BUDGET = 120 * 10 ** 9


def run_serving(args):
    """Poisson arrivals at 200 req/s; each request a seeded lens of 8-30
    surfaces from a resident pool, an output of 512^2..4096^2, 8/16/31
    wavelengths, a pupil grid of 32^2..256^2 and a source at 0-20 deg;
    admitted against a 120 GB HBM budget.  Two mixes over the same lens pool:
    the ghost layer of every request (the headline), then (--serve-starburst,
    on by default) the same arrivals with each request's starburst layer
    added from resident DFT matrices.  Each against serial plain renders
    (per-call plan, per-pair launches, per-call DFT matrices, blocking) of a
    sample of its requests."""
    import torch
    import ghostlight_gb300 as gl
    from ghostlight_gb300.serve import _spectral, serving_lens_pool
    cfg = gl.FlareConfig(min_ghost_intensity=MIN_INTENSITY)
    t0 = time.perf_counter()
    pool = serving_lens_pool(SERVE_LENSES, cfg, seed=100, n_min=8, n_max=30)
    grids = range(32, 257, 16)
    for rl in pool.values():                      # resident tables: grids and IOR slices of the mix
        for g in grids:
            rl.prepare(g)
        for ns in (8, 16, 31):
            rl.prepare(0, _spectral(ns, cfg)[0])
    setup_s = time.perf_counter() - t0
    out = _serve_mix(args, pool, cfg, False, args.serve_seconds, args.serve_dump)
    out["lens_setup_s"] = setup_s
    if args.serve_starburst:
        out["with_starburst"] = _serve_mix(args, pool, cfg, True, args.serve_sb_seconds,
                                           args.serve_dump + ".starburst.csv" if args.serve_dump else "")
    if args.serve_budget_gb > 0:
        # the same arrivals against a budget that binds: requests wait for memory
        out["binding_budget"] = _serve_mix(args, pool, cfg, False, args.serve_budget_seconds, "",
                                           budget=int(args.serve_budget_gb * 1e9))
    for rl in pool.values():
        rl.close()
    return out


def _serve_mix(args, pool, cfg, sb_on, seconds, dump, budget=SERVE_BUDGET):
    import torch
    import ghostlight_gb300 as gl
    from ghostlight_gb300.flare import GhostRenderPlan, pupil_grid
    from ghostlight_gb300.serve import (FlareRequest, FlareServer, SpriteStarbursts, _spectral, latency_stats,
                                        poisson_requests)
    reqs = poisson_requests(args.serve_rate, seconds, pool.keys(), seed=5, starburst=sb_on,
                            psf_frac=args.serve_psf_frac)
    # warm: one flare request per lens, and one PSF atlas per lens on a 2 x 2
    # source grid, which the mix never asks for (its 4 x 4 and 8 x 8 atlases
    # find no pre-pass kept: each computes its own on first use)
    srv = FlareServer(pool, budget_bytes=SERVE_BUDGET, max_inflight=args.serve_slots, items_per_warp=8)
    warm = [FlareRequest(lens_id=i, width=512, height=512, n_spec=8, ray_grid=32, field_deg=5.0, rid=i,
                         starburst=sb_on) for i in pool]
    if args.serve_psf_frac > 0:
        warm += [FlareRequest(lens_id=i, width=128, height=128, n_spec=8, ray_grid=32, field_deg=0.0,
                              rid=len(pool) + i, kind="psf", psf_grid=2) for i in pool]
    srv.run_trace(warm)
    torch.cuda.synchronize()
    warm_exec = srv.exec
    warm_exec.close()
    _progress("serving warm-up (starburst %s)" % sb_on)
    srv = FlareServer(pool, budget_bytes=budget, max_inflight=args.serve_slots, items_per_warp=8,
                      policy=args.serve_policy)
    # a pinned result buffer per slot and size: no host allocation while serving
    srv.exec.prewarm([(w, w) for w in (256, 512, 1024, 2048, 4096)], args.serve_slots)
    sb_bytes = 0
    if sb_on:                                     # resident sprites of every (lens, size, wavelength count)
        srv.exec.sprites = warm_exec.sprites
        srv.exec.prewarm_starburst([(w, w) for w in (512, 1024, 2048, 4096)], (8, 16, 31), cfg)
        torch.cuda.synchronize()
        sb_bytes = srv.exec.sprites.device_bytes()
        _progress("serving sprite bakes")
    import gc
    gc.collect()
    gc.disable()                                  # no collector pauses inside the request loop
    try:
        with ClockSampler(torch.cuda.current_device()) as clk:
            t1 = time.perf_counter()
            srv.run_trace(reqs)
            torch.cuda.synchronize()
            wall = time.perf_counter() - t1
    finally:
        gc.enable()
    _progress("serving timed mix (starburst %s)" % sb_on)
    traced = sum(r.traced for r in reqs)
    if dump:
        with open(dump, "w") as f:
            f.write("rid,kind,lens,n_surf,n_pairs,width,n_spec,grid,field,priority,est_rays,traced,arrival,start,finish\n")
            for r in reqs:
                rl = pool[r.lens_id]
                f.write("%d,%s,%d,%d,%d,%d,%d,%d,%.3f,%d,%d,%d,%.6f,%.6f,%.6f\n" % (
                    r.rid, r.kind, r.lens_id, len(rl.lens.surfaces), rl.n_pairs, r.width, r.n_spec, r.ray_grid, r.field_deg,
                    r.priority, r.est_rays, r.traced, r.arrival, r.start, r.finish))
    by_size = {"%dx%d" % (w, w): latency_stats(reqs, lambda r, w=w: r.kind == "flare" and r.width == w)
               for w in (512, 1024, 2048, 4096)}
    by_size["psf"] = latency_stats(reqs, lambda r: r.kind == "psf")
    # serial plain renders of a sample of the same requests
    rng = np.random.default_rng(9)
    sample = [reqs[i] for i in sorted(rng.choice(len(reqs), size=min(len(reqs), args.serial_sample),
                                                 replace=False))]
    ts = []
    for r in sample:
        rl = pool[r.lens_id]
        tt = time.perf_counter()
        if r.kind == "psf":                       # render_psf, blocking, as the reference serves one
            pcfg, psrc = srv.exec.psf_config(r, rl)
            po = gl.render_psf(psrc, rl.lens, pcfg)
            po["r"].cpu()
            ts.append(time.perf_counter() - tt)
            continue
        spec, corr = _spectral(r.n_spec, cfg)
        grid = pupil_grid(rl.lens, r.ray_grid, 0, 0, 0, 0.0)
        src = np.array([[math.radians(r.field_deg), 0.0, 1.0, 1.0, 1.0]], np.float32)
        plan = GhostRenderPlan(rl.lens, rl.pairs, rl.boosts, src, [grid], np.zeros(len(rl.pairs), np.int32), spec,
                               corr, r.width, r.height, rl.sensor_half_w, rl.sensor_half_h, r.gain,
                               apply_correction=True, plain_per_pair=True)
        outs = torch.empty((3, r.height, r.width), device="cuda")
        plan.execute(outs[0], outs[1], outs[2])
        if r.starburst:                           # the sprite baked for this call, as the reference renders
            cx, cy = rl.image_point(r.field_deg, r.width, r.height)
            sb = SpriteStarbursts()
            sprite, M, g = sb._bake(rl, r.width, r.height, r.n_spec)
            lib = gl._native.load()
            gl._native.check(lib.gl_sprite_splat_source(
                ctypes.c_void_p(sprite.data_ptr()), M, float(cx), float(cy), 1.0, 1.0, 1.0, g["sx_ds"], g["sy_ds"],
                g["px_mm_x"], g["px_mm_y"], g["rx"], g["ry"], g["gain"], ctypes.c_void_p(outs[0].data_ptr()),
                ctypes.c_void_p(outs[1].data_ptr()), ctypes.c_void_p(outs[2].data_ptr()), r.width, r.height,
                ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)), "starburst")
        outs.cpu()
        plan.close()
        ts.append(time.perf_counter() - tt)
    serial_req_s = len(ts) / sum(ts)
    _progress("serving serial sample")
    served_req_s = len(reqs) / wall
    srv.exec.close()
    if sb_on:
        srv.exec.sprites.close()
    return {"workload": "Poisson %.0f req/s for %.0f s (%d requests), %d resident lenses of 8-30 surfaces, "
                        "outputs 512^2-4096^2, 8/16/31 wavelengths, pupil grids 32^2-256^2, field 0-20 deg, "
                        "%.0f%% of the requests PSF atlases (4x4 or 8x8 tiles of 64^2, 64^2 pupil grid), "
                        "%d slots, %.0f GB HBM budget, %s priorities" % (
                            args.serve_rate, seconds, len(reqs), SERVE_LENSES, 100.0 * args.serve_psf_frac,
                            args.serve_slots, budget / 1e9, args.serve_policy),
            "layers": ("ghost + starburst: every request whose source images within a frame width of the frame "
                       "(%d of %d) adds its lens's SPRITE starburst (the reference's default engine: the stop "
                       "pupil's FFT baked over the request's wavelengths at the physical scale of the lens's "
                       "calibration, box-summed to the output pitch), resident per (lens, size, wavelength "
                       "count), splatted at the source's image point on the request's stream, %.2f GB of "
                       "sprites" % (sum(bool(r.starburst) for r in reqs), len(reqs), sb_bytes / 1e9))
            if sb_on else "ghost",
            "throughput_req_s": served_req_s, "wall_s": wall, "offered_req_s": len(reqs) / seconds,
            "rays_per_s": traced / wall, "ray_lambda_traces": traced,
            "latency_all": latency_stats(reqs), "latency_by_size": by_size,
            "peak_inflight": srv.sched.peak_inflight, "peak_budget_bytes": srv.sched.peak_used,
            "budget_bytes": budget, "deferred": sum(bool(r.deferred) for r in reqs),
            "rejected": len(srv.rejected), "psf_requests": sum(r.kind == "psf" for r in reqs),
            "serial_plain": {"sample": len(ts), "req_s": serial_req_s, "mean_ms": 1e3 * sum(ts) / len(ts)},
            "speedup_served_vs_serial_plain": served_req_s / serial_req_s, "clocks": clk.summary()}


# ---- anamorphic source sweep (120 frames, one graph) ---------------------------
SWEEP_N, SWEEP_W, SWEEP_H, SWEEP_GRID, SWEEP_DEG = 120, 2048, 1024, 128, 20.0
SWEEP_PUPIL, SWEEP_FILL = 256, 0.30


def run_sweep(args):
    """Seeded 18-surface 1.5x anamorphic (4 cylinders, per-element decenter
    and tilt): 120 sources along the frame diagonal from on-axis to 20 deg,
    31 wavelengths, 128^2 pupil grids, 2048x1024 frames (a 4:3 sensor inscribed
    in the lens's image circle, shown desqueezed); each frame = ghost layer +
    split-BF16 starburst at the source's paraxial image point; all 120 frames
    one CUDA graph.  Against the plain form: per-pair ghost launches and the
    same starburst, frame by frame, no graph."""
    import torch
    import ghostlight_gb300 as gl
    from ghostlight_gb300._abi import gl_surface
    from ghostlight_gb300.flare import GhostRenderPlan, pupil_grid
    from ghostlight_gb300.optics import OpticalSystem
    from ghostlight_gb300.serve import ResidentLens, _spectral
    from ghostlight_gb300.starburst import build_pupil
    from ghostlight_gb300.sweep import SourceSweep, diagonal_sources, paraxial_centers
    pins = np.load(GOLDEN / "ref_pins.npz")
    raw = pins["cfg4_anamorphic_18/lens"]
    lens = OpticalSystem.from_records(list((gl_surface * raw.shape[0]).from_buffer_copy(raw.tobytes())),
                                      name="cfg4_anamorphic_18")
    cal = json.loads((GOLDEN / "ref_meta.json").read_text())["cfg4_anamorphic_18"]["calibration"]
    a, b = cal["image_circle_semi_w"], cal["image_circle_semi_h"]
    hh = 1.0 / math.sqrt((4.0 / 3.0 / a) ** 2 + (1.0 / b) ** 2)
    hw = 4.0 / 3.0 * hh
    fx, fy = cal["focal_length_x"], cal["focal_length_y"]
    cfg = gl.FlareConfig(spectral_samples=N_SPEC, min_ghost_intensity=MIN_INTENSITY)
    rl = ResidentLens(lens, hw, hh, cfg)
    src = diagonal_sources(SWEEP_N, SWEEP_DEG, hw, hh, fx, fy)
    W_, H_ = SWEEP_W, SWEEP_H
    pupil = build_pupil(lens, SWEEP_PUPIL, SWEEP_FILL)
    spec, _ = _spectral(N_SPEC, cfg)
    lam = spec[:, 0].astype(np.float64)
    # physically proportioned pattern (pupil sample pitch 2 EP / (fill n), pixel pitch, focal
    # length per axis), trimmed so that the 400 nm period spans the frame width
    dxp = 2 * cal["entrance_pupil_semi_x"] / (SWEEP_FILL * SWEEP_PUPIL)
    dyp = 2 * cal["entrance_pupil_semi_y"] / (SWEEP_FILL * SWEEP_PUPIL)
    sx_phys = dxp * (2 * hw / W_) / (lam * 1e-6 * fx)
    sy_phys = dyp * (2 * hh / H_) / (lam * 1e-6 * fy)
    trim = float(sx_phys[np.argmin(lam)] * W_)
    sx, sy = sx_phys / trim, sy_phys / trim
    amp = float(pupil.double().sum())
    w = (spec[:, 1:4].astype(np.float64) / amp ** 2).astype(np.float32)
    centers = paraxial_centers(src, fx, fy, hw, hh, W_, H_)
    stream = torch.cuda.Stream()
    plan = gl.MdftPlan(SWEEP_PUPIL, (W_, H_), sx, sy, w, "split_bf16", stream=stream.cuda_stream)
    sb = dict(plan=plan, pupil=pupil, centers=centers)
    sweep = SourceSweep(rl, src, W_, H_, N_SPEC, SWEEP_GRID, starburst=sb, stream=stream)
    sweep.capture()
    flush = torch.empty(128 * 1024 * 1024, dtype=torch.float32, device="cuda")
    steps = max(1, min(args.steps, 3))
    with torch.cuda.stream(stream):
        sweep.replay()
        stream.synchronize()
        ts = []
        for _ in range(steps):
            flush.add_(1.0)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            sweep.replay()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
    if plan.status() != 0:
        raise RuntimeError("sweep starburst: device wait timed out")
    traced = sweep.traced()
    t = sum(ts) / len(ts)
    # e2e: replay + every frame to pinned host memory
    host = torch.empty((SWEEP_N, 3, H_, W_), dtype=torch.float32).pin_memory()
    with torch.cuda.stream(stream):
        t0 = time.perf_counter()
        sweep.replay()
        for k in range(SWEEP_N):
            sweep.copy_out(host[k], k)
        stream.synchronize()
        te = time.perf_counter() - t0
    # plain form on a sample of frames
    spec31, corr = _spectral(N_SPEC, cfg)
    grid = pupil_grid(lens, SWEEP_GRID, 0, 0, 0, 0.0)
    sample = [0, SWEEP_N // 3, 2 * SWEEP_N // 3, SWEEP_N - 1]
    outs = [torch.zeros((H_, W_), device="cuda") for _ in range(3)]
    tp = []
    for k in sample:
        s1 = np.array([[src[k, 0], src[k, 1], 1.0, 1.0, 1.0]], np.float32)
        gp = GhostRenderPlan(lens, rl.pairs, rl.boosts, s1, [grid], np.zeros(len(rl.pairs), np.int32), spec31,
                             corr, W_, H_, hw, hh, 1000.0, apply_correction=True, plain_per_pair=True)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        gp.execute(*outs)
        plan.set_center(*centers[k])
        plan.execute(pupil, *outs, accumulate=True)
        e1.record()
        e1.synchronize()
        tp.append(e0.elapsed_time(e1) / 1e3)
        gp.close()
    plain_fps = len(tp) / sum(tp)
    res = {"workload": "18-surface 1.5x anamorphic (4 cylinders, decentred/tilted elements), %d pairs, %d sources "
                       "on the diagonal 0-%.0f deg, %d wavelengths, %d^2 pupil grids, %dx%d frames, starburst %d^2 "
                       "pupil split-BF16 per frame; one CUDA graph" % (rl.n_pairs, SWEEP_N, SWEEP_DEG, N_SPEC,
                                                                       SWEEP_GRID, W_, H_, SWEEP_PUPIL),
           "frames_per_s": SWEEP_N / t, "ms_per_sweep": 1e3 * t, "graph_launches": sweep.launches,
           "ray_lambda_traces_per_sweep": traced, "rays_per_s": traced / t,
           "plain_frames_per_s": plain_fps, "plain_sample_frames": len(tp),
           "speedup_batched_vs_plain": (SWEEP_N / t) / plain_fps,
           "e2e_frames_per_s": SWEEP_N / te, "e2e_d2h_bytes": int(host.numel() * 4)}
    sweep.close(); plan.close(); rl.close()
    return res


def cpu_baseline(plan, lens, cal, gpu_frame):
    """The CPU leg, timed on the host cores and used as the FP64 parity
    reference of the timed frame:

    * timing: the reference's own code (oracle/_ref, built from the staged
      reference sources: its filter, grids and trace_ghost_ray in the
      ghost_kernel main path with the three-pass probe cull) renders the whole
      frame once on every core ("reference"); where it is not built, the
      oracle's FP32 port of the same path over the frame's kept pairs
      ("port");
    * parity: the frame the GPU rendered in the timed loop (all three planes,
      2048^2, colour-corrected) against the FP64 oracle's render of the same
      kept pairs over the same per-ghost grids and spectral table: relative L2
      and the largest per-pixel error relative to the frame's peak.  Pairs the
      off-sensor cull dropped are not rendered on either side (the cull is
      checked against uncut renders by tests/test_gpu_ghost.py)."""
    from oracle import oracle as O
    n_threads = os.cpu_count() or 1
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    hits = plan.pair_hits()
    keep = np.nonzero(hits > 0)[0]
    src = _sources()
    def oracle_frame(fp64):
        img = O.render(lens.records(), plan.pairs[keep], plan.boosts[keep], src, plan.grids, plan.spec, hw, hh, W, H,
                       1000.0, pair_grid=plan.pair_grid[keep], fp64=fp64, n_threads=n_threads)
        if plan.apply_correction:
            img = np.einsum("ij,jhw->ihw", plan.correction.astype(np.float64), img)
        return img

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    def binned(a, k=4):
        c, h, w = a.shape
        return a.reshape(c, h // k, k, w // k, k).sum(axis=(2, 4))

    t0 = time.perf_counter()
    want = oracle_frame(True)
    t_fp64 = time.perf_counter() - t0
    ieee32 = oracle_frame(False)
    got = gpu_frame.astype(np.float64)
    r64 = rel(got, want)
    floor32 = rel(ieee32, want)
    mx = float(np.abs(got - want).max() / max(float(np.abs(want).max()), 1e-300))
    parity = {"rel_l2": r64, "max_err_rel_peak": mx, "tolerance": 1e-3, "pass": r64 <= 1e-3,
              "against": "FP64 oracle (oracle/gl_oracle_impl.h, double), the %d kept pairs of the timed frame, "
                         "2048^2 x 3 planes, same grids / spectral table / colour correction" % len(keep),
              "fp32_floor_rel_l2": floor32,
              "within_fp32_floor": r64 <= floor32,
              "fp32_floor_note": "the reference's trace formulation in IEEE float32 (the oracle's float mode) "
                                 "against FP64 on the same frame: focused ghosts (spots about a pixel across at "
                                 "2048^2) turn the ~1e-5 mm float32 landing error into this image error",
              "rel_l2_vs_float32_oracle": rel(got, ieee32),
              "rel_l2_binned_4x4": rel(binned(got), binned(want)),
              "oracle_s": t_fp64, "oracle_cores": n_threads}
    try:
        from oracle import ref as R
        use_ref = R.available()
    except Exception:
        use_ref = False
    if use_ref:
        raw, rcal = _reference_lens("cfg2_wide_angle_24")
        rpairs, rboosts = R.filter_pairs(raw, hw, hh, MIN_INTENSITY)
        sides = np.array([adaptive_side(fp, hw, hh) for fp in R.ghost_footprints(raw, rpairs)], np.int32)
        spec, corr = R.spectral_table(N_SPEC)
        t0 = time.perf_counter()
        _, st = R.render_frame_cpu(raw, rpairs, rboosts, sides, src[0], spec, corr, hw, hh, W, H, 1000.0,
                                   cull=True, n_threads=n_threads)
        dt = time.perf_counter() - t0
        base = {"value": 1.0 / dt, "unit": UNIT, "cores": st["threads"], "kind": "reference",
                "sample": "one whole frame (probe cull + %d kept pairs, %d ray-wavelength traces, %.2f s) with the "
                          "reference's trace_ghost_ray" % (st["kept_pairs"], st["render_traces"] + st["probe_traces"], dt),
                "rays_per_s": (st["render_traces"] + st["probe_traces"]) / dt}
    else:
        rays = sum(len(plan.grids[int(plan.pair_grid[i])]) for i in keep) * N_SPEC
        t0 = time.perf_counter()
        O.render(lens.records(), plan.pairs[keep], plan.boosts[keep], src, plan.grids, plan.spec, hw, hh, W, H,
                 1000.0, pair_grid=plan.pair_grid[keep], fp64=False, n_threads=n_threads)
        dt = time.perf_counter() - t0
        base = {"value": 1.0 / dt, "unit": UNIT, "cores": n_threads, "kind": "port",
                "sample": "one whole frame of the %d kept pairs (%d ray-wavelength traces, %.2f s), the oracle's "
                          "FP32 port of ghost_kernel's main path" % (len(keep), rays, dt), "rays_per_s": rays / dt}
    return base, parity


def frame_config(n_pairs):
    """The workload both arms report: identical dicts, so the two lines
    describe the same frame."""
    return {"workload": "cfg2: seeded 24-surface wide-angle (2 even aspheres), %d ghost pairs after the "
                        "1e-6 culler, off-sensor cull on, adaptive pupil grids 16^2-256^2 (one pupil sample "
                        "per two output pixels across each ghost), %d wavelengths, source %.0f deg, "
                        "%dx%d float32 RGB with colour correction" % (n_pairs, N_SPEC, SOURCE_DEG, W, H),
            "pairs": int(n_pairs),
            "l2": "GPU arm: flushed (512 MB write) between timed steps; inputs resident",
            "parallelism": "replicas"}


def adaptive_side(fp, hw, hh, gmin=16, gmax=256):
    """The frame's per-ghost grid rule (one pupil sample per two output
    pixels across the ghost's landing extent, a multiple of 16 in
    [16, 256]); the product computes the same rule in
    ghostlight_gb300.flare.adaptive_grid_size."""
    fx = float(fp[0]) / (2.0 * hw) * W
    fy = float(fp[1]) / (2.0 * hh) * H
    side = 0.5 * math.sqrt(max(fx, 1.0) * max(fy, 1.0))
    return int(min(gmax, max(gmin, int(math.ceil(side / 16.0)) * 16)))


def _reference_lens(name):
    pins = np.load(GOLDEN / "ref_pins.npz")
    meta = json.loads((GOLDEN / "ref_meta.json").read_text())
    return pins[name + "/lens"], meta[name]["calibration"]


def run_reference(args):
    """CPU reference arm: the reference's own code (ghostlight/src trace.cpp,
    ghost.cpp, spectral.cpp, aperture_sampler.h, compiled from its sources by
    oracle/build.py) renders the whole frame on every host core each step:
    its filter_ghost_pairs, the footprint probe of estimate_ghost_spread for
    the per-ghost grid sides, its spectral table and correction, then the
    three-pass off-sensor cull and the main path of ghost_kernel over every
    kept pair at 2048^2 (oracle/ref_driver.cpp:ref_render_frame_cpu).
    Nothing from ghostlight_gb300 is imported."""
    from oracle import ref as R
    if not R.available():
        return {"impl": "reference", "unavailable": "the reference sources were not staged in baseline/_ref "
                                                    "(oracle/stage_ref.py), so its CPU code could not be built"}
    raw, cal = _reference_lens("cfg2_wide_angle_24")
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    pairs, boosts = R.filter_pairs(raw, hw, hh, MIN_INTENSITY)
    sides = np.array([adaptive_side(fp, hw, hh) for fp in R.ghost_footprints(raw, pairs)], np.int32)
    spec, corr = R.spectral_table(N_SPEC)
    src = _sources()[0]
    n_threads = os.cpu_count() or 1
    ts, st = [], None
    for it in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        img, st = R.render_frame_cpu(raw, pairs, boosts, sides, src, spec, corr, hw, hh, W, H, 1000.0,
                                     cull=True, n_threads=n_threads)
        if it >= args.warmup:
            ts.append(time.perf_counter() - t0)
    step = sum(ts) / len(ts)
    fps = 1.0 / step
    cfg1 = reference_cfg1(R, n_threads)
    gpu = reference_gpu_frame(R, raw, cal, pairs, sides, args) if not args.no_reference_gpu else None
    return {"metric": METRIC, "value": fps, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "impl": "reference", "config": frame_config(len(pairs)),
            "rays_per_s": (st["render_traces"] + st["probe_traces"]) / step,
            "frame": {"kept_pairs": st["kept_pairs"], "render_traces": st["render_traces"],
                      "probe_traces": st["probe_traces"], "grid_sides": np.bincount(sides).nonzero()[0].tolist()},
            "cpu_baseline": {"value": fps, "unit": UNIT, "cores": st["threads"], "kind": "reference",
                             "sample": "the whole frame every step (probe cull + %d kept pairs, %d "
                                       "ray-wavelength traces) with the reference's trace_ghost_ray"
                                       % (st["kept_pairs"], st["render_traces"] + st["probe_traces"])},
            "e2e": {"value": fps, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cfg1": cfg1, "gpu": gpu}


def reference_gpu_frame(R, raw, cal, pairs, sides, args):
    """The reference's own CUDA renderer (its core library built for sm_103a
    from the staged sources, oracle/build.py:build_ref_gpu) on the same frame:
    render_source_flare at 15 deg, concentration off, the off-sensor cull on,
    31 wavelengths, 2048^2; its API takes one pupil grid per call, so the
    frame is one call per grid side with a GhostFilter INCLUDE list of the
    pairs of that side (the per-ghost adaptive grids).  Each call is timed by
    wall clock (its host filter, uploads, probes, render, colour correction
    and the D2H of the planes); its own stage timing (collect_stats) gives the
    device part (ms_kernel).  Also the reference's single-call default
    (one 256^2 grid, concentrated sampling with adaptive budgets)."""
    try:
        R._load_gpu()
    except Exception as e:  # noqa: BLE001
        return {"unavailable": "the reference's CUDA renderer did not build here: %s" % str(e).splitlines()[0]}
    hw, hh = cal["sensor_half_w"], cal["sensor_half_h"]
    centre = R.solve_source(raw, cal, 0.0, 0.0, hw, hh)
    off = np.array([[math.radians(SOURCE_DEG) - centre["angle_x"], -centre["angle_y"], 1.0]], np.float32)
    groups = {}
    for (a, b), sd in zip(pairs, sides):
        groups.setdefault(int(sd), []).append((int(a), int(b)))

    def cfg_for(side, conc=0, stats=0):
        return R.RefGpuCfg(ray_grid=side, spectral_samples=N_SPEC, pupil_jitter=0, jitter_seed=0,
                           sensor_half_w=hw, sensor_half_h=hh, flare_gain=1000.0, min_ghost_intensity=MIN_INTENSITY,
                           cull_dead_pairs=1, concentrate_samples=conc, adaptive_sample_budgets=conc,
                           source_x=0.5, source_y=0.5, collect_stats=stats)

    def frame():
        ms = 0.0
        for side, grp in sorted(groups.items()):
            _, _, t, _ = R.gpu_render(raw, W, H, cfg_for(side), calib=cal, offsets=off, include=grp)
            ms += t
        return ms

    frame()                                          # warm: allocations, caches
    steps = max(3, min(args.steps, 10))
    with ClockSampler(0) as clk:
        walls = [frame() for _ in range(steps)]
    kern = 0.0
    for side, grp in sorted(groups.items()):
        _, _, _, st = R.gpu_render(raw, W, H, cfg_for(side, stats=1), calib=cal, offsets=off, include=grp)
        kern += st["ms_kernel"]
    dflt = []
    for _ in range(3):
        _, _, t, st = R.gpu_render(raw, W, H, cfg_for(256, conc=1), calib=cal, offsets=off)
        dflt.append(t)
    wall = float(np.median(walls))
    return {"frames_per_s": 1e3 / wall, "wall_ms_per_frame": wall, "walls_ms": walls,
            "device_ms_per_frame": kern, "calls_per_frame": len(groups),
            "how": "reference render_source_flare (ghostlight/src/SourceFlareRenderer.cpp:24), one call per grid "
                   "side with a GhostFilter INCLUDE list; wall clock per call; device_ms = the renderer's own "
                   "ms_kernel stage (probes + render + colour correction)",
            "default_grid256_concentrated_wall_ms": float(np.median(dflt)),
            "clocks": clk.summary()}


CFG1_W = CFG1_H = 512


def reference_cfg1(R, n_threads, reps=5):
    """Configuration 1 on the host with the reference's code: the seeded
    12-surface double Gauss, the 2-reflection pairs that do not cross the
    stop, a 32^2 grid, 8 wavelengths, a 10 deg source, 512^2 (frames/s)."""
    raw, cal = _reference_lens("cfg1_double_gauss_12")
    pairs, boosts = cfg1_pairs(R, raw, cal)
    spec, corr = R.spectral_table(8)
    src = np.array([math.radians(10.0), 0.0, 1.0, 1.0, 1.0], np.float32)
    sides = np.full(len(pairs), 32, np.int32)
    ts = []
    for _ in range(reps + 1):
        t0 = time.perf_counter()
        _, st = R.render_frame_cpu(raw, pairs, boosts, sides, src, spec, corr, cal["sensor_half_w"],
                                   cal["sensor_half_h"], CFG1_W, CFG1_H, 1000.0, cull=True, n_threads=n_threads)
        ts.append(time.perf_counter() - t0)
    dt = float(np.median(ts[1:]))
    return {"value": 1.0 / dt, "unit": UNIT, "ms_per_frame": 1e3 * dt, "cores": st["threads"],
            "pairs": int(len(pairs)), "traces": st["render_traces"] + st["probe_traces"],
            "workload": "cfg1: seeded 12-surface double Gauss, %d non-stop-crossing pairs, 32^2 grid, "
                        "8 wavelengths, 10 deg, 512^2" % len(pairs)}


def cfg1_pairs(R, raw, cal):
    """The reference filter at 1e-7, then the 2-reflection pairs whose
    bounces lie on one side of the stop (the configuration's "pairs that do
    not cross the stop"), in the filter's order."""
    pairs, boosts = R.filter_pairs(raw, cal["sensor_half_w"], cal["sensor_half_h"], 1e-7)
    stop = [i for i in range(len(raw)) if int(raw[i]["is_stop"])][0]
    keep = np.array([(a < stop) == (b < stop) for a, b in pairs], bool)
    return pairs[keep], boosts[keep]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true",
                    help="reference arm: skip the timing of the reference's CUDA renderer")
    ap.add_argument("--quick", action="store_true",
                    help="batched timing only (no plain / e2e / CPU legs): for profiler runs")
    ap.add_argument("--serve-seconds", type=float, default=30.0)
    ap.add_argument("--serve-slots", type=int, default=32)
    ap.add_argument("--serve-rate", type=float, default=SERVE_RATE, help="Poisson arrival rate (requests/s)")
    ap.add_argument("--serve-starburst", type=int, default=1,
                    help="1: also serve the mix with every request's starburst layer")
    ap.add_argument("--serve-sb-seconds", type=float, default=15.0, help="arrival window of the starburst mix")
    ap.add_argument("--serve-policy", default="sjf", choices=("sjf", "lsf", "sjf_fifo"),
                    help="stream priority of a request: shortest first; longest (least slack) first; or "
                         "shortest first with the long requests ranked by arrival")
    ap.add_argument("--serial-sample", type=int, default=40)
    ap.add_argument("--serve-dump", default="", help="write per-request timings (CSV) here")
    ap.add_argument("--serve-psf-frac", type=float, default=0.1,
                    help="fraction of the serving requests that are PSF atlases (render_psf)")
    ap.add_argument("--serve-budget-gb", type=float, default=1.5,
                    help="HBM budget of the extra serving run whose budget binds (0: no such run)")
    ap.add_argument("--serve-budget-seconds", type=float, default=10.0)
    ap.add_argument("--only", default="all", choices=["all", "cfg3", "serve", "sweep"],
                    help="with --quick: also run the starburst / convolution section (profiler runs)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank == 0:
            print(json.dumps(run_reference(args)))
        return
    if args.only == "sweep":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        if rank == 0:
            print(json.dumps({"anamorphic_sweep": run_sweep(args)}))
        return
    if args.only == "serve":
        import torch
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", 0)))
        if rank == 0:
            print(json.dumps({"serving": run_serving(args)}))
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    res, plan, gpu_frame = run_gpu(args, rank, world)
    if rank == 0:
        lens, cal = _workload()
        if not (args.no_cpu_baseline or args.quick):
            res["cpu_baseline"], res["parity"] = cpu_baseline(plan, lens, cal, gpu_frame)
            if _CFG1_CHECK and "cfg1" in res:
                res["cfg1"]["parity"] = cfg1_parity()
            _progress("cpu baseline and FP64 parity")
        if not args.quick:
            res["anamorphic_sweep"] = run_sweep(args)
            _progress("anamorphic sweep")
        if not args.quick and args.serve_seconds > 0:
            res["serving"] = run_serving(args)
            _progress("serving")
        res["roofline"] = roofline(res, plan)
        print(json.dumps(res))
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


def roofline(res, plan):
    """Dominant kernel: ghost_render_kernel (render launch), bound by FP32
    issue on the CUDA cores (the trace is sequential FP32 arithmetic; the
    splat is a small share).  Algorithmic FLOPs per launch = the launch's
    traced ray-wavelengths x the per-trace FP32 operation count measured once
    with ncu on this workload; duration = the launch's CUDA-event time in the
    timed replays."""
    flops_per_trace = FLOPS_PER_RAY_LAMBDA
    peak = FP32_PEAK_TFLOPS
    sec = res["kernel_ms"]["render"] / 1e3
    achieved = res["traces_render"] * flops_per_trace / sec / 1e12 if (flops_per_trace and sec > 0) else None
    return {"bound": "fp32", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": (achieved / peak) if (achieved and peak) else None, "traffic": RENDER_DRAM_BYTES,
            "kernel": "ghost_render_kernel", "kernel_ms": res["kernel_ms"]["render"],
            "flop_per_launch": res["traces_render"] * flops_per_trace,
            "peak_note": "GB300 FP32 CUDA-core peak: 152 SMs x 128 lanes x 2 FLOP x max SM clock",
            "traffic_note": "DRAM bytes of one render launch from ncu (dram__bytes_read.sum + "
                            "dram__bytes_write.sum on this frame): the image accumulator stays in L2"}


# FP32 operations per traced ray-wavelength (FADD + FMUL + 2 x FFMA, thread
# level, predicated on) of the render kernel on this workload, measured with
# ncu on one launch of the tuned shape while only the lanes of live rays ran
# the step (smsp__sass_thread_inst_executed_op_{fadd,fmul,ffma}_pred_on.sum:
# 4.926e9 + 20.971e9 + 2 x 18.993e9 = 6.388e10 FLOP over 6.007e7 traces),
# and frozen as the algorithmic count.  The branch-free step now also runs
# on the lanes of dead rays (work nobody reads: 7.5e10 counted FLOP per
# launch), which the algorithmic count leaves out.
FLOPS_PER_RAY_LAMBDA = 1063.5
# DRAM bytes (read + write) of one render launch on this frame, from the same
# capture (dram__bytes_read.sum + dram__bytes_write.sum: 40.99 + 4.94 MB).
RENDER_DRAM_BYTES = 45.93e6
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.070e9 / 1e12


if __name__ == "__main__":
    main()
