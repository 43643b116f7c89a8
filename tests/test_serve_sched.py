"""Serving admission policy and request mix, on the CPU with a fake executor."""
import numpy as np
import pytest

from ghostlight_gb300.serve import (FlareRequest, FlareServer, Scheduler, latency_stats, poisson_requests,
                                    priority_class, request_bytes)


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def __call__(self):
        return self.t


class FakeExecutor:
    """Requests take est_rays / rate seconds of fake time, run concurrently."""

    host_output = False

    def __init__(self, clock, rate=1e9, n_pairs=100):
        self.clock, self.rate, self.n_pairs = clock, rate, n_pairs
        self.started = []

    def estimate(self, req):
        req.est_rays = int(self.n_pairs * 0.8 * req.ray_grid ** 2 * req.n_spec)
        req.priority = priority_class(req.est_rays)
        req.device_bytes = request_bytes(req.width, req.height, self.n_pairs)

    def start(self, req):
        self.started.append(req.rid)
        return (req, self.clock() + req.est_rays / self.rate)

    def done(self, run):
        return self.clock() >= run[1]

    def finish(self, run):
        return None


def _serve(reqs, budget, slots, dt=1e-4):
    clock = FakeClock()
    ex = FakeExecutor(clock)
    srv = FlareServer({}, budget_bytes=budget, max_inflight=slots, executor=ex, clock=clock)
    peak_used = peak_inflight = 0
    i = 0
    reqs = sorted(reqs, key=lambda r: r.arrival)
    while i < len(reqs) or not srv.idle():
        while i < len(reqs) and reqs[i].arrival <= clock.t:
            srv.submit(reqs[i])
            i += 1
        srv.step()
        peak_used = max(peak_used, srv.sched.used)
        peak_inflight = max(peak_inflight, srv.sched.inflight)
        assert srv.sched.used <= budget and srv.sched.inflight <= slots
        clock.t += dt
    return srv, ex, peak_used, peak_inflight


def test_budget_and_slots_hold_and_every_request_completes():
    reqs = poisson_requests(200.0, 2.0, range(4), seed=1)
    budget = 3 * request_bytes(4096, 4096, 100)
    srv, ex, peak_used, peak_inflight = _serve(reqs, budget, slots=8)
    assert len(srv.completed) == len(reqs)
    assert sorted(ex.started) == sorted(r.rid for r in reqs)
    assert peak_used <= budget and peak_inflight <= 8
    assert all(r.finish >= r.start >= r.arrival for r in reqs)


def test_small_request_skips_past_one_that_does_not_fit():
    s = Scheduler(budget_bytes=request_bytes(4096, 4096, 10) + request_bytes(512, 512, 10), max_inflight=4)
    big = [FlareRequest(0, 4096, 4096, 8, 64, 0.0, rid=i) for i in range(2)]
    small = FlareRequest(0, 512, 512, 8, 64, 0.0, rid=9)
    for r in big + [small]:
        r.device_bytes = request_bytes(r.width, r.height, 10)
        s.submit(r)
    first = s.admit()
    assert [r.rid for r in first] == [0, 9]        # the second big one waits, the small one does not
    s.release(first[0])
    assert [r.rid for r in s.admit()] == [1]


def test_oversize_request_is_rejected():
    s = Scheduler(budget_bytes=1000, max_inflight=2)
    r = FlareRequest(0, 64, 64, 8, 32, 0.0)
    r.device_bytes = 5000
    with pytest.raises(ValueError):
        s.submit(r)


def test_poisson_mix_is_seeded_and_in_range():
    a = poisson_requests(200.0, 5.0, range(8), seed=3)
    b = poisson_requests(200.0, 5.0, range(8), seed=3)
    assert [(r.arrival, r.width, r.ray_grid) for r in a] == [(r.arrival, r.width, r.ray_grid) for r in b]
    assert 850 < len(a) < 1150
    assert {r.width for r in a} == {512, 1024, 2048, 4096}
    assert {r.n_spec for r in a} == {8, 16, 31}
    assert min(r.ray_grid for r in a) >= 32 and max(r.ray_grid for r in a) <= 256
    assert all(0.0 <= r.field_deg <= 20.0 for r in a)
    gaps = np.diff([r.arrival for r in a])
    assert abs(gaps.mean() - 1 / 200.0) < 0.15 / 200.0


def test_priority_is_shortest_job_first():
    assert priority_class(1e5) < priority_class(1e7) < priority_class(1e8) <= priority_class(1e10)


def test_priority_least_slack_first_reverses():
    ests = (1e5, 1e7, 1e8, 1e10)
    sjf = [priority_class(e, policy="sjf") for e in ests]
    lsf = [priority_class(e, policy="lsf") for e in ests]
    assert lsf[0] > lsf[1] > lsf[2] > lsf[3]
    assert all(-3 <= p <= 0 for p in sjf + lsf)
    assert [a + b for a, b in zip(sjf, lsf)] == [-3] * 4
    with pytest.raises(ValueError):
        priority_class(1e5, policy="fifo")


def test_fifo_levels_for_long_requests():
    from ghostlight_gb300.serve import fifo_heavy_level, fifo_light_level, size_class
    assert [size_class(e) for e in (1e5, 1e7, 1e8, 1e10)] == [0, 1, 2, 3]
    g, l = -5, 0
    assert fifo_heavy_level([], g, l) == -2                 # first long request: right below the short classes
    assert fifo_heavy_level([-2], g, l) == -1               # the next one ranks behind it
    assert fifo_heavy_level([-2, -1], g, l) == 0
    assert fifo_heavy_level([-2, -1, 0], g, l) == 0         # out of levels: the lowest
    assert fifo_heavy_level([-1], g, l) == 0                # never ahead of an older one still running
    # a device with four levels (0 .. -3): the two shortest classes share the top
    assert [fifo_light_level(c, -3, 0) for c in (0, 1, 2)] == [-3, -3, -2]
    assert fifo_heavy_level([], -3, 0) == -1 and fifo_heavy_level([-1], -3, 0) == 0
    assert [fifo_light_level(c, -5, 0) for c in (0, 1, 2)] == [-5, -4, -3]


def test_latency_stats():
    rs = []
    for i in range(100):
        r = FlareRequest(0, 512, 512, 8, 32, 0.0, rid=i, arrival=0.0)
        r.finish = (i + 1) * 1e-3
        rs.append(r)
    st = latency_stats(rs)
    assert st["n"] == 100 and abs(st["p50_ms"] - 50.5) < 1e-6 and 99.0 <= st["p99_ms"] <= 100.0


def test_default_wavelength_split():
    from ghostlight_gb300.serve import lambda_split
    assert [lambda_split(n) for n in (1, 3, 8, 16, 31, 64)] == [1, 1, 1, 2, 4, 8]


def test_poisson_mix_with_psf_requests():
    from ghostlight_gb300.serve import poisson_requests
    reqs = poisson_requests(200.0, 5.0, [0, 1, 2], seed=3, psf_frac=0.2)
    psf = [r for r in reqs if r.kind == "psf"]
    assert 0.1 * len(reqs) < len(psf) < 0.3 * len(reqs)
    for r in psf:
        assert r.psf_grid in (4, 8) and r.width == r.height == r.psf_grid * r.psf_tile and not r.starburst


def test_binding_budget_defers_and_rejects():
    """With a budget that binds, requests wait for memory (marked deferred),
    the budget holds at every step, and a request above the whole budget is
    rejected instead of queued; the rest complete."""
    from ghostlight_gb300.serve import request_bytes
    reqs = [FlareRequest(0, 2048, 2048, 8, 32, 0.0, rid=i) for i in range(8)]
    big = FlareRequest(0, 16384, 16384, 8, 32, 0.0, rid=99)
    budget = 2 * request_bytes(2048, 2048, 100)
    srv, ex, peak_used, _ = _serve(reqs + [big], budget, slots=8)
    assert big.rejected and big not in srv.completed
    assert len(srv.completed) == len(reqs)
    assert any(r.deferred for r in reqs) and peak_used <= budget
