"""Scheduler of the serving loop (ibamr_gb300.serving) on the CPU with a
fake backend: every request completes, steps of one simulation never
overlap, steps of different simulations do, the HBM budget is never
exceeded and idle simulations are evicted least recently used first."""

import numpy as np
import pytest

from ibamr_gb300 import serving


def spec(sid, dim, N, n):
    return serving.SimSpec(sid, dim, N, np.zeros(n * dim))


class TrackingBackend(serving.FakeBackend):
    def __init__(self, server_ref, **kw):
        super().__init__(**kw)
        self.server_ref = server_ref
        self.max_used = 0

    def create(self, s):
        out = super().create(s)
        srv = self.server_ref[0]
        self.max_used = max(self.max_used, srv.used + s.bytes)
        return out


def make_server(budget, n_slots, duration, sims):
    ref = [None]
    be = TrackingBackend(ref, duration=duration)
    srv = serving.Server(be, budget, n_slots=n_slots)
    ref[0] = srv
    for s in sims:
        srv.register(s)
    return srv, be


def test_all_requests_complete_with_latency_at_least_the_step():
    sims = [spec(k, 2, [64, 64], 1000) for k in range(4)]
    srv, be = make_server(1 << 40, 4, lambda s: 2e-4, sims)
    reqs = serving.poisson_requests(2000.0, 200, [s.sid for s in sims], seed=1)
    out = srv.run(reqs)
    assert out["requests"] == 200 and len(out["latency_s"]) == 200
    assert min(out["latency_s"].values()) >= 2e-4
    assert out["p99_ms"] >= out["p50_ms"] > 0
    assert out["markers_per_s"] > 0


def test_one_simulation_never_runs_twice_at_once_and_others_overlap():
    sims = [spec(k, 2, [32, 32], 100) for k in range(3)]
    dur = 3e-3
    srv, be = make_server(1 << 40, 3, lambda s: dur, sims)
    # a burst: all requests arrive at t = 0
    reqs = [serving.Request(i, 0.0, i % 3) for i in range(9)]
    srv.run(reqs)
    by_sim = {}
    for sid, slot, t in be.launches:
        by_sim.setdefault(sid, []).append(t)
    for sid, ts in by_sim.items():
        ts.sort()
        assert all(b - a >= dur * 0.999 for a, b in zip(ts, ts[1:])), sid
    # the first launches of the three simulations overlap in time
    firsts = sorted(min(ts) for ts in by_sim.values())
    assert firsts[-1] - firsts[0] < dur


def test_budget_admission_evicts_idle_lru_and_never_exceeds_budget():
    sims = [spec(k, 3, [32, 32, 32], 5000) for k in range(3)]
    budget = int(2.5 * sims[0].bytes)  # two fit, three do not
    srv, be = make_server(budget, 2, lambda s: 5e-4, sims)
    reqs = [serving.Request(i, i * 1e-3, [0, 1, 2, 0, 1, 2, 2, 0][i % 8]) for i in range(32)]
    out = srv.run(reqs)
    assert out["requests"] == 32
    assert be.max_used <= budget
    assert out["evictions"] > 0 and len(be.destroyed) == out["evictions"]
    assert srv.used <= budget
    srv.close()
    assert srv.used == 0 and not srv.resident


def test_simulation_larger_than_budget_is_refused():
    s = spec(0, 3, [64, 64, 64], 100000)
    srv = serving.Server(serving.FakeBackend(), s.bytes - 1, n_slots=1)
    with pytest.raises(ValueError):
        srv.register(s)


def test_memory_estimate_grows_with_size():
    a = serving.simulation_bytes(3, [32, 32, 32], 1000)
    b = serving.simulation_bytes(3, [64, 64, 64], 1000)
    c = serving.simulation_bytes(3, [64, 64, 64], 100000)
    assert a < b < c
