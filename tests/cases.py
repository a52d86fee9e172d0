"""Seeded problem generators shared by the parity tests."""

import numpy as np

from oracle import ibx_oracle as oracle


def random_patch_case(rng, dim, kernel, centering, q_depth=1, n_markers=64, with_shifts=True, subset=True):
    """A patch with a non-trivial box and origin, markers inside, near and
    just outside its ghost box, optional periodic shifts and an index subset."""
    ilower = rng.integers(-5, 6, size=dim)
    ncell = rng.integers(5, 10, size=dim)
    iupper = ilower + ncell - 1
    dx = rng.uniform(0.05, 0.2, size=dim)
    x_lower = ilower * dx  # SAMRAI: x_lower = ilower*dx on a uniform level
    x_upper = x_lower + ncell * dx
    g = oracle.min_ghost_width(kernel)
    gw = [g + int(rng.integers(0, 2)) for _ in range(dim)]
    # positions: mostly inside the ghost box, a few outside
    lo = x_lower - (gw[0] + 1.5) * dx
    hi = x_upper + (gw[0] + 1.5) * dx
    X = rng.uniform(lo, hi, size=(n_markers, dim)).reshape(-1)
    if subset:
        idx = np.sort(rng.choice(n_markers, size=n_markers * 3 // 4, replace=False)).astype(np.int32)
    else:
        idx = np.arange(n_markers, dtype=np.int32)
    if with_shifts:
        k = rng.integers(-1, 2, size=(idx.size, dim))
        mask = rng.uniform(size=(idx.size, 1)) < 0.3
        shifts = (k * mask * ncell[None, :] * dx[None, :]).reshape(-1)
    else:
        shifts = np.zeros(idx.size * dim)
    Q_depth = dim if centering == 1 else q_depth
    Q = rng.standard_normal(n_markers * Q_depth)
    touches = rng.integers(0, 2, size=(2, dim))
    return {
        "dim": dim, "kernel": kernel, "centering": centering, "q_depth": q_depth if centering == 0 else 1,
        "ilower": ilower.tolist(), "iupper": iupper.tolist(), "dx": dx.tolist(), "x_lower": x_lower.tolist(),
        "x_upper": x_upper.tolist(), "gcw": gw, "X": X, "Q": Q, "Q_depth": Q_depth, "indices": idx,
        "shifts": np.ascontiguousarray(shifts, dtype=np.float64), "touches_lower": touches[0].tolist(),
        "touches_upper": touches[1].tolist(), "n_markers": n_markers,
    }


def oracle_patch(case):
    P = oracle.Patch()
    P.dim = case["dim"]
    for d in range(case["dim"]):
        P.ilower[d] = case["ilower"][d]
        P.iupper[d] = case["iupper"][d]
        P.dx[d] = case["dx"][d]
        P.x_lower[d] = case["x_lower"][d]
        P.x_upper[d] = case["x_upper"][d]
        P.touches_regular_lower[d] = case["touches_lower"][d]
        P.touches_regular_upper[d] = case["touches_upper"][d]
    return P


def oracle_spread(case, q_init=None):
    """Oracle spread of a random patch case: returns the list of ghosted arrays."""
    P = oracle_patch(case)
    q = oracle.GhostedData(P, case["centering"], case["gcw"], depth=case["q_depth"])
    if q_init is not None:
        for a in range(len(q.arrays)):
            q.arrays[a][...] = q_init[a]
    rc = oracle.spread_idx(q, case["Q"], case["Q_depth"], case["X"], case["indices"], case["shifts"], case["kernel"])
    assert rc == 0, rc
    return q


def oracle_interp(case, q_arrays):
    P = oracle_patch(case)
    q = oracle.GhostedData(P, case["centering"], case["gcw"], depth=case["q_depth"])
    for a in range(len(q.arrays)):
        q.arrays[a][...] = q_arrays[a]
    Q = np.full(case["n_markers"] * case["Q_depth"], 7.25)
    rc = oracle.interpolate_idx(Q, case["Q_depth"], case["X"], case["indices"], case["shifts"], q, case["kernel"])
    assert rc == 0, rc
    return Q


def fibonacci_sphere(n, radius, centre, jitter, rng):
    i = np.arange(n) + 0.5
    z = 1.0 - 2.0 * i / n
    phi = np.arange(n) * np.pi * (3.0 - np.sqrt(5.0))
    r = np.sqrt(1.0 - z * z)
    X = np.stack([r * np.cos(phi), r * np.sin(phi), z], axis=1) * radius + centre
    X += rng.uniform(-jitter, jitter, size=X.shape)
    return X


def rel_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    scale = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (scale if scale > 0 else 1.0))
