"""The plan-setting strings bench.py prints and replays (``tuning.setting_string``
/ ``parse_setting``): a round trip, and unknown knobs refused."""

import pytest

from ibamr_gb300 import tuning


def test_setting_round_trip():
    s = {"tile_shape": 1, "item_units": 128, "dense_min": 64, "dense_blocks_per_sm": 4, "visit_kernel": 2,
         "interp_kernel": 0, "step_mode": 1, "unit_cap": 16}
    text = tuning.setting_string(s)
    assert text.startswith("tile_shape=1,item_units=128,")
    assert tuning.parse_setting(text) == s
    assert tuning.parse_setting("") == {}


def test_unknown_knob_refused():
    with pytest.raises(ValueError):
        tuning.parse_setting("tile_shape=0,warp_size=64")


def test_default_candidates_cover_every_knob():
    for k in tuning.KNOBS:
        if k in ("item_units", "dense_min", "dense_blocks_per_sm"):
            continue
        assert k in tuning.DEFAULT_CANDIDATES


class _FakeGraph:
    def __init__(self, plan):
        self.plan = plan

    def launch(self, stream=None):
        self.plan.launches += 1

    def close(self):
        pass


class _FakePlan:
    """The knobs of a plan with its own interpolation targets, no device:
    a step "costs" a separable function of the knobs."""

    separate_interp = True

    def __init__(self):
        self._t = (256, 128, 2)
        self.unit_cap = 32
        self.visit_kernel = 0
        self.interp_kernel = 0
        self.step_mode = 1
        self.launches = 0

    def tuning(self):
        return self._t

    def set_tuning(self, iu, dm, bps):
        self._t = (iu, dm, bps)

    def bin(self):
        pass

    def graph(self):
        return _FakeGraph(self)

    def cost(self):
        iu, dm, bps = self._t
        c = {32: 3, 64: 2, 128: 0, 256: 1}[iu] + {1: 2, 2: 1, 4: 0}[bps] + abs(dm - 64) / 64
        c += {0: 2, 1: 1, 2: 0, 3: 1}[self.visit_kernel] + {32: 0, 16: 1, 8: 2}[self.unit_cap]
        # the interpolation form and the step mode interact: form 1 is best
        # only with mode 4, which is worst with any other form
        c += {(1, 4): 0}.get((self.interp_kernel, self.step_mode),
                             5 if self.step_mode == 4 else 1 + self.interp_kernel % 2)
        return 1.0 + c


def test_autotune_search_on_a_fake_plan(monkeypatch):
    """The staged search without a device (the graph and the timer faked): it
    times graph launches of whole steps, re-tunes the spread knobs under the
    three fastest interpolation-form/step-mode pairs, reaches the optimum of
    a separable cost whose best form/mode pair only shows once measured, and
    leaves the plan in the setting it reports."""
    import torch

    plan = _FakePlan()
    monkeypatch.setattr(torch.cuda, "current_stream", lambda *a, **k: None)

    def fake_time(fn, reps, stream):
        fn()
        return plan.cost()

    monkeypatch.setattr(tuning, "_time", fake_time)
    cand = {"visit_kernel": (0, 1, 2, 3), "interp_kernel": (0, 1, 2), "step_mode": (1, 4, 0)}
    res = tuning.autotune(plan, reps=2, candidates=cand)
    assert plan.launches > 0  # whole steps, launched from graphs
    iu, dm, bps, vk, ik, sm, cap = res["config"]
    assert (iu, dm, bps, vk, ik, sm, cap) == (128, 64, 4, 2, 1, 4, 32)
    assert res["ms"] == min(ms for _, ms in res["table"]) == 1.0
    assert plan.tuning() == (128, 64, 4) and plan.visit_kernel == 2
    assert (plan.interp_kernel, plan.step_mode, plan.unit_cap) == (1, 4, 32)
    # every form/mode pair was measured, and the spread knobs were swept
    # again under the three fastest of them
    rows = {}
    for c, _ in res["table"]:
        rows[(c[4], c[5])] = rows.get((c[4], c[5]), 0) + 1
    n_pairs = len(cand["interp_kernel"]) * len(cand["step_mode"])
    assert len(rows) == n_pairs
    dc = tuning.DEFAULT_CANDIDATES
    s1 = len(dc["dense_min"]) * len(cand["visit_kernel"])  # split with the visit form
    s2 = len(dc["item_units"]) * len(dc["dense_blocks_per_sm"]) * len(dc["unit_cap"])  # dense knobs
    # the starting pair (form 0, mode 1): stages 1 and 2, its stage-3 row and
    # a stage-4 sweep; two more pairs: a stage-3 row and a sweep; the rest one
    assert sorted(rows.values()) == sorted([s1 + s2 + 1 + s1 + s2, 1 + s1 + s2, 1 + s1 + s2] + [1] * (n_pairs - 3))
