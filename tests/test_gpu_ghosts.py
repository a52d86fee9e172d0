"""Device ghost accumulation and periodic ghost fill (ibx_accumulate_ghosts,
ibx_fill_ghosts) against the oracle's restatement of the reference flow
(SAMRAIGhostDataAccumulator on one patch covering the domain; the periodic
ghost copy), bit for bit: the device sums in the reference's array order.
Also the reference's spread golden replayed end to end on the device: patch
spread of the markers in the patch box, then ghost accumulation."""

import numpy as np
import pytest

from tests import cases
from tests import golden_replay as gr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available()
    m.lib()
    return m


def patch_problem(ibx, dim, centering, P, gcw, q_tensors, depth):
    ilo = [P.ilower[d] for d in range(dim)]
    ihi = [P.iupper[d] for d in range(dim)]
    dx = [P.dx[d] for d in range(dim)]
    xl = [P.x_lower[d] for d in range(dim)]
    xu = [P.x_upper[d] for d in range(dim)]
    dummy = torch.zeros(1, dtype=torch.float64, device="cuda")
    return ibx.make_problem(dim, centering, ibx.MODE_PATCH, ilo, ihi, dx, xl, xu, q_tensors, dummy, dummy,
                            q_depth=depth, gcw=gcw, n_markers=0)


@pytest.mark.parametrize("periodic", [(1, 1, 1), (1, 0, 1), (0, 0, 0)])
@pytest.mark.parametrize("centering,depth", [(0, 1), (0, 2), (1, 1)])
@pytest.mark.parametrize("dim", [2, 3])
def test_accumulate_and_fill_match_oracle(ibx, oracle, dim, centering, depth, periodic):
    rng = np.random.default_rng(10 * dim + 3 * centering + depth + 100 * sum(periodic))
    N = [7, 6, 5][:dim]
    P = oracle.make_patch(dim, [2, -1, 0][:dim], [2 + N[0] - 1, -1 + N[1] - 1, N[2] - 1 if dim == 3 else 0][:dim],
                          [0.0] * dim, [1.0] * dim, dx=[1.0 / n for n in N], periodic=list(periodic[:dim]))
    gcw = [3, 2, 4][:dim]
    per = list(periodic[:dim]) + [0] * (3 - dim)
    # accumulation
    q = oracle.GhostedData(P, centering, gcw, depth=depth)
    for a in q.arrays:
        a[...] = rng.standard_normal(a.shape)
    q_t = [torch.tensor(a, device="cuda") for a in q.arrays]
    prob = patch_problem(ibx, dim, centering, P, gcw, q_t if centering == 1 else q_t[0], depth)
    ilo = [P.ilower[d] for d in range(dim)]
    ihi = [P.iupper[d] for d in range(dim)]
    oracle.accumulate_ghosts_single_patch(q, ilo, ihi, per)
    ibx.accumulate_ghosts(prob, per)
    torch.cuda.synchronize()
    for a in range(len(q.arrays)):
        assert np.array_equal(q_t[a].cpu().numpy(), q.arrays[a])
    # fill (the oracle's fill is periodic in every dim)
    if all(periodic[:dim]):
        for a in q.arrays:
            a[...] = rng.standard_normal(a.shape)
        q_t = [torch.tensor(a, device="cuda") for a in q.arrays]
        prob = patch_problem(ibx, dim, centering, P, gcw, q_t if centering == 1 else q_t[0], depth)
        oracle.fill_periodic_ghosts(q)
        ibx.fill_ghosts(prob, per)
        torch.cuda.synchronize()
        for a in range(len(q.arrays)):
            assert np.array_equal(q_t[a].cpu().numpy(), q.arrays[a])


GOLD = [c for c in gr.load("ghost_accumulation_01.json") if c["name"].endswith(".a")]


@pytest.mark.parametrize("case", GOLD, ids=[c["name"] for c in GOLD])
def test_golden_spread_with_device_accumulation(ibx, oracle, case):
    """ghost_accumulation_01 (one patch): the markers in the patch box
    (LEInteractor::spread on raw arrays selects them with getCellIndex)
    spread on the device in patch mode, the ghosts accumulated on the device;
    the patch values against the golden output."""
    dim, centering = case["dim"], case["centering"]
    patch = case["patches"][0]
    P = oracle.make_patch(dim, patch["ilower"], patch["iupper"], patch["x_lower"], patch["x_upper"],
                          dx=patch["dx"], periodic=case["periodic"])
    gw = [case["ghost_width"]] * dim
    X = np.asarray(case["X"], dtype=np.float64)
    Q = np.asarray(case["Q"], dtype=np.float64)
    per = [int(v) for v in case["periodic"]] + [0] * (3 - dim)
    idx = np.empty(X.size // dim, dtype=np.int32)
    n_idx = oracle.lib().ibxo_build_local_indices(oracle.ctypes.byref(P), oracle.ivec(patch["ilower"]),
                                                  oracle.ivec(patch["iupper"]), oracle.dptr(X), X.size // dim,
                                                  oracle.iptr(idx))
    idx = idx[:n_idx]
    q = oracle.GhostedData(P, centering, gw, depth=1)
    q_t = [torch.tensor(a, device="cuda") for a in q.arrays]
    X_t = torch.tensor(X, device="cuda")
    Q_t = torch.tensor(Q, device="cuda")
    ilo = [P.ilower[d] for d in range(dim)]
    ihi = [P.iupper[d] for d in range(dim)]
    prob = ibx.make_problem(dim, centering, ibx.MODE_PATCH, ilo, ihi, [P.dx[d] for d in range(dim)],
                            [P.x_lower[d] for d in range(dim)], [P.x_upper[d] for d in range(dim)],
                            q_t if centering == 1 else q_t[0], X_t, Q_t, Q_depth=case["Q_depth"], gcw=gw,
                            indices=torch.tensor(idx, device="cuda"),
                            touches_physical_lower=list(P.touches_regular_lower)[:dim],
                            touches_physical_upper=list(P.touches_regular_upper)[:dim], n_markers=X.size // dim)
    ibx.spread(prob, "PIECEWISE_LINEAR")
    gprob = patch_problem(ibx, dim, centering, P, gw, q_t if centering == 1 else q_t[0], 1)
    ibx.accumulate_ghosts(gprob, per)
    torch.cuda.synchronize()
    got, want = [], []
    for comp_s, entries in patch["values"].items():
        comp = int(comp_s)
        arr = q_t[comp].cpu().numpy()[0]
        lo = q.lower(comp)
        for e in entries:
            k = tuple(e[d] - lo[d] for d in range(dim))[::-1]
            got.append(arr[k])
            want.append(e[dim])
    assert cases.rel_err(np.array(got), np.array(want)) <= 1e-13
