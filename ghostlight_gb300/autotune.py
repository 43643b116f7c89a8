"""Autotuner for the launch shapes of the flare path.

Times candidate launch shapes on the caller's own workload, on the running
GPU, and keeps the fastest; choices are cached per (device, workload key) in
memory and, when GL_TUNE_CACHE names a file (or ``cache_path`` is given), in a
JSON file so a server starts tuned.  Knobs:

* the ghost render: persistent work queue with 4..8 CTAs per SM, or one-shot
  CTAs of 1..8 32-sample items per warp (``GhostRenderPlan.set_launch``);
* the starburst GEMMs: the persistent grid size and the output tile width of
  the second GEMM, 128 or 64 complex columns per unit (``MdftPlan.set_launch``).

The splat has no tile to tune: each lane keeps its 2x2 footprint across the
wavelength loop and flushes on change, so there is no shared-memory tile whose
shape would matter.
"""
from __future__ import annotations

import json
import os
import threading
from typing import Callable, Dict, Hashable, List, Optional, Sequence

# (items per warp, CTAs per SM, wavelength chunks per item)
GHOST_CANDIDATES = [(0, 0, 1), (0, 0, 2), (0, 0, 4), (0, 0, 8), (0, 0, 16), (0, 6, 4), (1, 0, 4), (1, 0, 1),
                    (2, 0, 1), (4, 0, 1), (8, 0, 1)]


def mdft_candidates(sms: int) -> List[tuple]:
    """(CTAs, tile width) pairs: one CTA per SM with either tile, then fewer
    CTAs with the default tile."""
    return [(0, 128), (0, 64), (max(1, (3 * sms) // 4), 128), (max(1, sms // 2), 128)]


class Tuner:
    def __init__(self, cache_path: Optional[str] = None, reps: int = 3, warm: int = 1):
        self.cache_path = cache_path if cache_path is not None else os.environ.get("GL_TUNE_CACHE") or None
        self.reps, self.warm = int(reps), int(warm)
        self._mem: Dict[str, object] = {}
        self._lock = threading.Lock()
        self.log: List[dict] = []
        if self.cache_path and os.path.exists(self.cache_path):
            try:
                with open(self.cache_path) as f:
                    self._mem.update(json.load(f))
            except (OSError, ValueError):
                pass

    @staticmethod
    def _key(key: Sequence[Hashable]) -> str:
        return "|".join(str(k) for k in key)

    def _save(self):
        if not self.cache_path:
            return
        tmp = self.cache_path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(self._mem, f, indent=1, sort_keys=True)
        os.replace(tmp, self.cache_path)

    def _cuda_timer(self, stream):
        import torch
        st = stream if stream is not None else torch.cuda.current_stream()

        def time_one(run, c):
            with torch.cuda.stream(st):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(st)
                run(c)
                e1.record(st)
                e1.synchronize()
                return e0.elapsed_time(e1)
        return time_one

    def best(self, key: Sequence[Hashable], candidates: Sequence, run: Callable, stream=None,
             timer: Optional[Callable] = None):
        """run(candidate) enqueues one execution; returns the fastest candidate
        (median of reps; CUDA events on `stream` unless a timer(run, c) -> ms
        is given)."""
        k = self._key(key)
        with self._lock:
            if k in self._mem:
                c = self._mem[k]
                return tuple(c) if isinstance(c, list) else c
        time_one = timer if timer is not None else self._cuda_timer(stream)
        timings = []
        for c in candidates:
            for _ in range(self.warm):
                time_one(run, c)
            ts = sorted(time_one(run, c) for _ in range(self.reps))
            timings.append((ts[len(ts) // 2], c))
        timings.sort(key=lambda x: x[0])
        choice = timings[0][1]
        self.log.append({"key": k, "choice": choice, "ms": [(round(t, 4), c) for t, c in timings]})
        with self._lock:
            self._mem[k] = list(choice) if isinstance(choice, tuple) else choice
            self._save()
        return choice


_default: Optional[Tuner] = None


def default_tuner() -> Tuner:
    global _default
    if _default is None:
        _default = Tuner()
    return _default


def _device_name() -> str:
    import torch
    return torch.cuda.get_device_name(torch.cuda.current_device()).replace(" ", "_")


def tune_ghost_plan(plan, outs, stream=None, tuner: Optional[Tuner] = None, candidates=None):
    """Pick and apply the render launch shape of a GhostRenderPlan."""
    t = tuner or default_tuner()
    key = ("ghost", _device_name(), plan.n_items, plan.rays, plan.width * plan.height)
    st = stream.cuda_stream if stream is not None else None

    def run(c):
        plan.set_launch(*c)
        plan.execute(*outs, stream=st)

    choice = t.best(key, candidates or GHOST_CANDIDATES, run, stream)
    plan.set_launch(*choice)
    return choice


def tune_mdft_plan(plan, pupil, outs, stream=None, tuner: Optional[Tuner] = None, candidates=None):
    """Pick and apply the GEMM grid and output tile of an MdftPlan."""
    import torch
    t = tuner or default_tuner()
    sms = torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count
    key = ("mdft", _device_name(), plan.form, plan.n, plan.Kx, plan.Ky, plan.n_lambda)
    st = stream.cuda_stream if stream is not None else None

    def run(c):
        plan.set_launch(c)
        plan.execute(pupil, *outs, stream=st)

    choice = t.best(key, candidates or mdft_candidates(sms), run, stream)
    plan.set_launch(choice)
    return choice
