"""The oracle against the reference's own golden outputs and known-answer tests."""

import numpy as np
import pytest

from tests import golden_replay as gr

GA = gr.load("ghost_accumulation_01.json")
KAT = gr.load("interpolate_01_exact.json")


def test_golden_inputs_are_the_reference_generator(oracle):
    # Fixture inputs are std::mt19937(42) draws: Q first, then X.
    for case in GA:
        n_q = len(case["Q"])
        draws = oracle.mt19937_uniform(42, n_q + len(case["X"]))
        assert np.array_equal(draws[:n_q], case["Q"])
        assert np.array_equal(draws[n_q:], case["X"])


@pytest.mark.parametrize("case", GA, ids=[c["name"] for c in GA])
def test_ghost_accumulation_golden(oracle, case):
    dim = case["dim"]
    gw = [case["ghost_width"]] * dim
    dlo = [0] * dim
    dhi = [n - 1 for n in case["domain_cells"]]

    def spread_patch(p, Q, X):
        P = oracle.make_patch(dim, p["ilower"], p["iupper"], p["x_lower"], p["x_upper"], dx=p["dx"],
                              periodic=case["periodic"], domain_lo=dlo, domain_hi=dhi)
        q = oracle.GhostedData(P, case["centering"], gw, depth=1)
        rc = oracle.spread_raw(q, Q, case["Q_depth"], X, p["ilower"], p["iupper"], case["kernel"])
        assert rc == 0
        return [(q.lower(a), q.arrays[a][0]) for a in range(len(q.arrays))]

    res = gr.replay_ghost_accumulation(case, spread_patch)
    got = np.array([r[2] for r in res])
    want = np.array([r[3] for r in res])
    scale = np.max(np.abs(want))
    # The goldens carry 16 significant digits; the reference compares with
    # numdiff -r 1e-6 -a 1e-10.  The restatement matches to round-off.
    assert np.max(np.abs(got - want)) <= 1e-13 * scale, np.max(np.abs(got - want)) / scale
    assert len(res) == sum(len(v) for p in case["patches"] for v in p["values"].values())


@pytest.mark.parametrize("case", KAT, ids=[c["name"] for c in KAT])
def test_interpolate_exact_kat(oracle, case):
    dim = case["dim"]
    kernel = case["kernel"]
    g = oracle.min_ghost_width(kernel)
    P = oracle.make_patch(dim, case["ilower"], case["iupper"], case["x_lower"], case["x_upper"], dx=case["dx"],
                          periodic=case["periodic"], domain_lo=[0] * dim, domain_hi=[31] * dim)
    q = oracle.GhostedData(P, 0, [g] * dim, depth=dim)
    # Exact multilinear field at every cell centre, ghosts included (the
    # reference's linear-refine ghost fill reproduces it exactly).
    arr = q.arrays[0]
    lo = q.lower()
    shape = arr.shape[1:][::-1]
    for k in np.ndindex(*shape):
        x = [case["x_lower"][d] + (lo[d] + k[d] - case["ilower"][d] + 0.5) * case["dx"][d] for d in range(dim)]
        v = gr.poly_value(case["function"], x)
        for dd in range(dim):
            arr[(dd,) + tuple(k[::-1])] = v
    X = np.asarray(case["X"], dtype=np.float64)
    Q = np.full(X.size, np.finfo(np.float64).max)
    rc = oracle.interpolate_raw(Q, dim, X, q, case["ilower"], case["iupper"], kernel)
    assert rc == 0
    for s in range(X.size // dim):
        exact = gr.poly_value(case["function"], X[dim * s: dim * s + dim])
        for dd in range(dim):
            assert abs(Q[dim * s + dd] - exact) <= case["tolerance"], (s, dd, Q[dim * s + dd], exact)
