"""Replays of the reference's golden tests on top of any spread/interpolate
implementation with the LEInteractor raw-array interface (oracle or CUDA)."""

import itertools
import json
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    with open(os.path.join(GOLDEN, name)) as f:
        return json.load(f)["cases"]


def dof_of(idx, comp, case):
    """SAMRAIGhostDataAccumulator DOF of position idx (None if outside a
    non-periodic domain); side normal `comp` has one extra face."""
    out = []
    for d in range(case["dim"]):
        N = case["domain_cells"][d]
        extra = 1 if (case["centering"] == 1 and d == comp) else 0
        if case["periodic"][d]:
            out.append(idx[d] % N)
        else:
            if idx[d] < 0 or idx[d] > N - 1 + extra:
                return None
            out.append(idx[d])
    return tuple(out)


def replay_ghost_accumulation(case, spread_patch):
    """spread_patch(patch_dict, Q, X) -> list of (lower_index, ndarray) per
    component: the patch's ghosted arrays after LEInteractor::spread of the
    markers in its box.  Returns {patch number: {comp: [(idx, value, golden)]}}."""
    dim = case["dim"]
    Q = np.asarray(case["Q"], dtype=np.float64)
    X = np.asarray(case["X"], dtype=np.float64)
    sums = {}
    for p in case["patches"]:
        arrays = spread_patch(p, Q, X)
        for comp, (lo, arr) in enumerate(arrays):
            shape = arr.shape[::-1]  # x first
            for k in itertools.product(*[range(n) for n in shape]):
                idx = [lo[d] + k[d] for d in range(dim)]
                dof = dof_of(idx, comp, case)
                if dof is None:
                    continue
                key = (comp, dof)
                sums[key] = sums.get(key, 0.0) + arr[tuple(k[::-1])]
    result = []
    for p in case["patches"]:
        for comp_s, entries in p["values"].items():
            comp = int(comp_s)
            for e in entries:
                idx = e[:dim]
                dof = dof_of(idx, comp, case)
                result.append((comp, tuple(idx), sums.get((comp, dof), 0.0), e[dim]))
    return result


def poly_value(fn, x):
    env = {"X_%d" % d: x[d] for d in range(len(x))}
    return eval(fn, {}, env)
