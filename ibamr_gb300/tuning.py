"""Autotuner of the binned plan's spread.

The spread of a plan has four knobs (``ibx_plan_set_tuning``,
``ibx_plan_set_visit_kernel``): the form of the per-visit kernel, the number
of home units per CTA of the dense-tile kernel (``item_units``, markers per
block in effect), the home-marker count above which a tile is spread from
its tile+halo region rather than through per-tile visits (``dense_min``,
which decides the split between the two kernels), and the CTAs per SM of
the dense-tile kernel.  The best setting depends on the marker distribution
(clustered fibres favour regions, scattered markers favour visits), so it
is measured: every candidate runs ``bin`` + ``spread`` on the plan's own
data and the fastest is kept.

The tile shape is a property of a plan, chosen when it is created
(``autotune_shape`` builds one plan per shape, tunes each, and keeps the
fastest): shape 0 is 8x8x8 cells in 3D and 16x16 in 2D, shape 1 is 16x8x8 and
32x16 (longer rows, fewer tiles visited per marker, larger regions).

Tuning spreads into the plan's target arrays (spreading adds), so run it
before the simulation's first step or on scratch targets.
"""

import itertools

DEFAULT_CANDIDATES = {
    "dense_min": (8, 16, 32, 64, 128, 256),
    "item_units": (32, 64, 128, 256),
    "dense_blocks_per_sm": (1, 2, 4),
    "visit_kernel": (0, 1),
}

_cache = {}


def _time(fn, reps, stream):
    import torch

    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    fn()
    torch.cuda.synchronize()
    a.record(stream)
    for _ in range(reps):
        fn()
    b.record(stream)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / reps


def autotune(plan, reps=3, candidates=None, key=None, include_bin=True):
    """Measure every candidate setting of ``plan`` and keep the fastest.

    Returns {"best": (item_units, dense_min, dense_blocks_per_sm),
    "table": [((...), ms), ...], "visit_kernel": form, "visit_kernel_ms":
    [(form, ms), ...], "ms": t}, t being the time of the applied setting
    (best knobs and best form).  With ``key`` the result is cached for
    this process and later calls with the same key only apply it."""
    import torch

    if key is not None and key in _cache:
        plan.set_tuning(*_cache[key]["best"])
        plan.visit_kernel = _cache[key]["visit_kernel"]
        return _cache[key]
    cand = dict(DEFAULT_CANDIDATES)
    if candidates:
        cand.update(candidates)
    stream = torch.cuda.current_stream()

    def step():
        if include_bin:
            plan.bin()
        plan.spread()

    table = []
    # dense_min changes the binning: search it first with the other knobs
    # at their defaults, then the dense-kernel knobs at the best split.
    iu0, dm0, bps0 = plan.tuning()
    for dm in cand["dense_min"]:
        plan.set_tuning(iu0, dm, bps0)
        plan.bin()
        table.append(((iu0, dm, bps0), _time(step, reps, stream)))
    best_dm = min(table, key=lambda r: r[1])[0][1]
    for iu, bps in itertools.product(cand["item_units"], cand["dense_blocks_per_sm"]):
        plan.set_tuning(iu, best_dm, bps)
        plan.bin()
        table.append((plan.tuning(), _time(step, reps, stream)))
    best = min(table, key=lambda r: r[1])[0]
    plan.set_tuning(*best)
    plan.bin()
    # the form of the per-visit kernel, at the best knobs
    forms = []
    for form in cand.get("visit_kernel", (0, 1)):
        plan.visit_kernel = form
        forms.append((form, _time(step, reps, stream)))
    best_form, ms = min(forms, key=lambda r: r[1])
    plan.visit_kernel = best_form
    out = {"best": best, "ms": ms, "table": table, "visit_kernel": best_form, "visit_kernel_ms": forms}
    if key is not None:
        _cache[key] = out
    return out


def autotune_shape(make_plan, shapes=(0, 1), reps=3, candidates=None):
    """Create a plan per tile shape with ``make_plan(shape)``, tune each with
    ``autotune`` and keep the fastest; the other plans are closed.  Returns
    (plan, {"shape": id, "ms": t, "per_shape": {id: (best knobs, ms)}})."""
    best_plan, best, per = None, None, {}
    for sh in shapes:
        plan = make_plan(sh)
        res = autotune(plan, reps=reps, candidates=candidates)
        per[sh] = (res["best"], res["ms"])
        if best is None or res["ms"] < best["ms"]:
            if best_plan is not None:
                best_plan.close()
            best_plan, best = plan, {"shape": sh, "ms": res["ms"], "best": res["best"],
                                     "visit_kernel": res["visit_kernel"]}
        else:
            plan.close()
    best["per_shape"] = per
    return best_plan, best
