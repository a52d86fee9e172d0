"""Autotuner of the binned plan.

A plan has these knobs (``ibx_plan_set_tuning``, ``ibx_plan_set_visit_kernel``,
``ibx_plan_set_interp_kernel``, ``ibx_plan_set_step_mode``):

* ``dense_min``: the home-marker count above which a tile is spread from its
  tile+halo region rather than through per-tile visits (the split between
  the two spread kernels);
* ``visit_kernel``: the form of the per-visit spread kernel (points
  flattened over lanes, lane per visit, the tile gathered in registers, or
  gathered with the visits' weight vectors assembled in registers);
* ``item_units``, ``dense_blocks_per_sm`` and ``unit_cap``: home units per
  CTA work item, CTAs per SM of the dense-tile kernel, and most markers per
  home unit (a unit is spread by one thread per component);
* ``interp_kernel``: all markers in chunks (home order), dense-homed ones per
  home unit, all in chunks in marker order started beside the sort, or
  markers evaluated from their home tile's region staged in shared memory
  (all of them, or the dense-homed ones);
* ``step_mode``: spread and interpolation concurrent (the spread's stream
  first, both of one priority, or the interpolation's first), one after the
  other, or fused into one persistent launch in ``step``.

The best setting depends on the marker distribution (clustered fibres favour
regions, scattered markers favour visits), so it is measured: every
candidate runs ``bin`` + ``spread`` on the plan's own data (the whole
``step``, interpolation included, when the plan has its own interpolation
targets: captured with ``Plan.graph`` and replayed, as a time stepper runs
it) and the fastest is kept.

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
    "visit_kernel": (0, 1, 2, 3),
    "interp_kernel": (0, 1, 2, 3, 4),
    "step_mode": (1, 3, 4, 0, 2),
    "unit_cap": (32, 16, 8),
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
    """Measure candidate settings of ``plan`` and keep the fastest.

    The search runs in stages, each at the best setting so far: the split
    between the two spread kernels (``dense_min``) jointly with the
    per-visit kernel form; the dense-kernel knobs (``item_units``,
    ``dense_blocks_per_sm``, ``unit_cap``); for plans with their own
    interpolation targets, the interpolation form jointly with the step mode
    (concurrent, serial or fused spread and interpolation), and then, under
    each of the three fastest of those pairs, the split with the visit form
    and the dense-kernel knobs once more.  Returns {"best": (item_units, dense_min,
    dense_blocks_per_sm), "visit_kernel": form, "interp_kernel": form or
    None, "step_mode": mode or None, "unit_cap": cap, "ms": t, "table":
    [((item_units, dense_min, dense_blocks_per_sm, visit_kernel,
    interp_kernel, step_mode, unit_cap), ms), ...]}, t being the time of the applied setting.  With ``key`` the
    result is cached for this process and later calls with the same key only
    apply it."""
    import torch

    full = include_bin and getattr(plan, "separate_interp", False)

    def apply(cfg):
        iu, dm, bps, vk, ik, sm, cap = cfg
        plan.set_tuning(iu, dm, bps)
        plan.unit_cap = cap
        plan.visit_kernel = vk
        if full:
            plan.interp_kernel = ik
            plan.step_mode = sm
        plan.bin()

    if key is not None and key in _cache:
        apply(_cache[key]["config"])
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

    def measure(cfg):
        apply(cfg)
        if full:
            # a whole step runs as a time stepper runs it: replayed from a
            # CUDA graph (eager launches order the concurrent streams
            # differently and would rank the step modes otherwise)
            g = plan.graph()
            try:
                table.append((cfg, _time(lambda: g.launch(stream), reps, stream)))
            finally:
                g.close()
        else:
            table.append((cfg, _time(step, reps, stream)))

    def best_cfg():
        return min(table, key=lambda r: r[1])

    iu0, dm0, bps0 = plan.tuning()
    cap0 = plan.unit_cap
    ik0, sm0 = (plan.interp_kernel, plan.step_mode) if full else (None, None)
    for dm, vk in itertools.product(cand["dense_min"], cand["visit_kernel"]):
        measure((iu0, dm0 if dm is None else dm, bps0, vk, ik0, sm0, cap0))
    _, dm, _, vk, _, _, _ = best_cfg()[0]
    for iu, bps, cap in itertools.product(cand["item_units"], cand["dense_blocks_per_sm"], cand["unit_cap"]):
        measure((iu, dm, bps, vk, ik0, sm0, cap))
    if full:
        iu, dm, bps, vk, _, _, cap = best_cfg()[0]
        stage3 = len(table)
        for ik, sm in itertools.product(cand["interp_kernel"], cand["step_mode"]):
            measure((iu, dm, bps, vk, ik, sm, cap))
        # the spread knobs again under the three fastest interpolation forms
        # and step modes: beside a concurrent interpolation fewer dense CTAs
        # and another split between the spread kernels can be best, one after
        # the other more
        ranked = sorted(table[stage3:], key=lambda r: r[1])
        pairs = list(dict.fromkeys((c[4], c[5]) for c, _ in ranked))[:3]
        for ik, sm in pairs:
            for dm2, vk2 in itertools.product(cand["dense_min"], cand["visit_kernel"]):
                measure((iu, dm2, bps, vk2, ik, sm, cap))
            _, dm2, _, vk2, _, _, _ = min((r for r in table if (r[0][4], r[0][5]) == (ik, sm)),
                                          key=lambda r: r[1])[0]
            for iu2, bps2, cap2 in itertools.product(cand["item_units"], cand["dense_blocks_per_sm"],
                                                     cand["unit_cap"]):
                measure((iu2, dm2, bps2, vk2, ik, sm, cap2))
    cfg, ms = best_cfg()
    apply(cfg)
    out = {"best": tuple(plan.tuning()), "ms": ms, "table": table, "config": cfg, "visit_kernel": cfg[3],
           "interp_kernel": cfg[4], "step_mode": cfg[5], "unit_cap": cfg[6]}
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
                                     "visit_kernel": res["visit_kernel"], "interp_kernel": res["interp_kernel"],
                                     "step_mode": res["step_mode"], "unit_cap": res["unit_cap"]}
        else:
            plan.close()
    best["per_shape"] = per
    return best_plan, best


KNOBS = ("item_units", "dense_min", "dense_blocks_per_sm", "visit_kernel", "interp_kernel", "step_mode", "unit_cap")


def setting_of(plan):
    """The plan's current setting: tile shape and every knob, as a dict."""
    iu, dm, bps = plan.tuning()
    return {"tile_shape": plan.tile_shape[0], "item_units": iu, "dense_min": dm, "dense_blocks_per_sm": bps,
            "visit_kernel": plan.visit_kernel, "interp_kernel": plan.interp_kernel, "step_mode": plan.step_mode,
            "unit_cap": plan.unit_cap}


def setting_string(setting):
    """``k=v,...`` form of a setting (the inverse of ``parse_setting``)."""
    return ",".join("%s=%d" % (k, setting[k]) for k in ("tile_shape",) + KNOBS if k in setting)


def parse_setting(text):
    """Setting dict from ``k=v,...`` (keys: tile_shape and the knobs)."""
    out = {}
    for part in text.split(","):
        if not part:
            continue
        k, v = part.split("=")
        if k not in ("tile_shape",) + KNOBS:
            raise ValueError("unknown plan knob %r" % k)
        out[k] = int(v)
    return out


def apply_setting(plan, setting):
    """Apply the knobs of a setting to a plan (the tile shape is chosen when
    the plan is created and must match)."""
    if "tile_shape" in setting and setting["tile_shape"] != plan.tile_shape[0]:
        raise ValueError("tile shape is fixed when the plan is created")
    plan.set_tuning(setting.get("item_units"), setting.get("dense_min"), setting.get("dense_blocks_per_sm"))
    for k in ("visit_kernel", "interp_kernel", "step_mode", "unit_cap"):
        if k in setting:
            setattr(plan, k, setting[k])
    plan.bin()
