"""CUDA FP64 path (ibx_spread / ibx_interpolate) against the oracle.

Bar: max-norm relative error <= 1e-12 over the whole grid (spread) and all
markers (interpolate), the plain-form tolerance; golden replays <= 1e-13.
"""

import numpy as np
import pytest

from tests import cases
from tests import golden_replay as gr

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

KERNEL_NAMES = ["PIECEWISE_LINEAR", "PIECEWISE_CUBIC", "IB_3", "IB_4", "IB_6", "BSPLINE_4"]
TOL = 1e-12


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available(), "GPU tests need CUDA"
    m.lib()
    return m


def dev(a, dtype=torch.float64):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def gpu_patch_problem(ibx, case, q_tensors, Q_t, X_t):
    return ibx.make_problem(
        case["dim"], case["centering"], ibx.MODE_PATCH, case["ilower"], case["iupper"], case["dx"], case["x_lower"],
        case["x_upper"], q_tensors, X_t, Q_t, Q_depth=case["Q_depth"], q_depth=case["q_depth"], gcw=case["gcw"],
        indices=dev(case["indices"], torch.int32), Xshift=dev(case["shifts"]),
        touches_physical_lower=case["touches_lower"], touches_physical_upper=case["touches_upper"],
        n_markers=case["n_markers"])


@pytest.mark.parametrize("kernel", KERNEL_NAMES)
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("centering,q_depth", [(0, 1), (0, 2), (1, 1)])
def test_patch_spread_interp_parity(ibx, oracle, kernel, dim, centering, q_depth):
    rng = np.random.default_rng(1000 * dim + 10 * centering + q_depth + 7 * KERNEL_NAMES.index(kernel))
    case = cases.random_patch_case(rng, dim, kernel, centering, q_depth=q_depth, n_markers=96)
    # spread into non-zero data (spread is "+=")
    ref0 = cases.oracle_spread(case)
    init = [rng.standard_normal(a.shape) for a in ref0.arrays]
    ref = cases.oracle_spread(case, q_init=init)
    q_t = [dev(a) for a in init]
    X_t = dev(case["X"])
    Q_t = dev(case["Q"])
    ibx.spread(gpu_patch_problem(ibx, case, q_t if centering == 1 else q_t[0], Q_t, X_t), kernel)
    for a in range(len(q_t)):
        assert cases.rel_err(q_t[a].cpu().numpy(), ref.arrays[a]) <= TOL
    # interpolate a random field
    field = [rng.standard_normal(a.shape) for a in ref0.arrays]
    Qref = cases.oracle_interp(case, field)
    q_t = [dev(a) for a in field]
    Q_out = dev(np.full(case["n_markers"] * case["Q_depth"], 7.25))
    ibx.interpolate(gpu_patch_problem(ibx, case, q_t if centering == 1 else q_t[0], Q_out, X_t), kernel)
    got = Q_out.cpu().numpy()
    assert cases.rel_err(got, Qref) <= TOL
    # markers that were not selected keep their value
    untouched = np.setdiff1d(np.arange(case["n_markers"]), case["indices"])
    for s in untouched:
        assert np.all(got[s * case["Q_depth"]:(s + 1) * case["Q_depth"]] == 7.25)


GA = gr.load("ghost_accumulation_01.json")


@pytest.mark.parametrize("case", GA, ids=[c["name"] for c in GA])
def test_golden_ghost_accumulation_on_gpu(ibx, oracle, case):
    dim = case["dim"]
    gw = [case["ghost_width"]] * dim
    dlo = [0] * dim
    dhi = [n - 1 for n in case["domain_cells"]]

    def spread_patch(p, Q, X):
        P = oracle.make_patch(dim, p["ilower"], p["iupper"], p["x_lower"], p["x_upper"], dx=p["dx"],
                              periodic=case["periodic"], domain_lo=dlo, domain_hi=dhi)
        host = oracle.GhostedData(P, case["centering"], gw, depth=1)
        idx = np.empty(X.size // dim, dtype=np.int32)
        n = oracle.lib().ibxo_build_local_indices(oracle.ctypes.byref(P), oracle.ivec(p["ilower"]),
                                                  oracle.ivec(p["iupper"]), oracle.dptr(X), X.size // dim,
                                                  oracle.iptr(idx))
        q_t = [dev(a[0]) for a in host.arrays]
        prob = ibx.make_problem(dim, case["centering"], ibx.MODE_PATCH, p["ilower"], p["iupper"], p["dx"],
                                p["x_lower"], p["x_upper"], q_t if case["centering"] == 1 else q_t[0], dev(X), dev(Q),
                                Q_depth=case["Q_depth"], gcw=gw, indices=dev(idx[:n], torch.int32),
                                touches_physical_lower=list(P.touches_regular_lower)[:dim],
                                touches_physical_upper=list(P.touches_regular_upper)[:dim])
        ibx.spread(prob, case["kernel"])
        return [(host.lower(a), q_t[a].cpu().numpy()) for a in range(len(q_t))]

    res = gr.replay_ghost_accumulation(case, spread_patch)
    got = np.array([r[2] for r in res])
    want = np.array([r[3] for r in res])
    assert cases.rel_err(got, want) <= 1e-13


def periodic_side_tensors(rng, dim, N):
    shape = list(N)[::-1]
    return [rng.standard_normal(shape) for _ in range(dim)]


@pytest.mark.parametrize("kernel", KERNEL_NAMES)
@pytest.mark.parametrize("dim", [2, 3])
def test_periodic_mode_matches_reference_flow(ibx, oracle, kernel, dim):
    """Compact periodic mode against the reference flow: ghost-box markers
    with periodic shifts, clipped spreading, interior kept; interpolation from
    periodically filled ghosts."""
    rng = np.random.default_rng(77 + dim + 13 * KERNEL_NAMES.index(kernel))
    N = [16, 12, 10][:dim]
    n = 300
    X = rng.uniform(0.0, 1.0, size=n * dim)
    X[: dim * 20] = rng.uniform(0.0, 0.04, size=dim * 20)  # crowd the periodic seams
    X[dim * 20: dim * 40] = rng.uniform(0.96, 1.0, size=dim * 20)
    F = rng.standard_normal(n * dim)
    u = periodic_side_tensors(rng, dim, N)
    f_ref, U_ref = oracle.periodic_side_problem(dim, N, kernel, X, F=F, u=np.stack(u))
    f_t = [torch.zeros(list(N)[::-1], dtype=torch.float64, device="cuda") for _ in range(dim)]
    X_t, F_t = dev(X), dev(F)
    dx = [1.0 / v for v in N]
    prob = ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N], dx, [0.0] * dim,
                            [1.0] * dim, f_t, X_t, F_t)
    ibx.spread(prob, kernel)
    for a in range(dim):
        assert cases.rel_err(f_t[a].cpu().numpy(), f_ref[a]) <= TOL
    u_t = [dev(v) for v in u]
    U_t = torch.zeros(n * dim, dtype=torch.float64, device="cuda")
    prob = ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N], dx, [0.0] * dim,
                            [1.0] * dim, u_t, X_t, U_t)
    ibx.interpolate(prob, kernel)
    assert cases.rel_err(U_t.cpu().numpy(), U_ref) <= TOL


KAT = gr.load("interpolate_01_exact.json")


@pytest.mark.parametrize("case", KAT, ids=[c["name"] for c in KAT])
def test_interpolate_exact_kat_on_gpu(ibx, oracle, case):
    dim = case["dim"]
    g = oracle.min_ghost_width(case["kernel"])
    lo = [case["ilower"][d] - g for d in range(dim)]
    n = [case["iupper"][d] - case["ilower"][d] + 1 + 2 * g for d in range(dim)]
    arr = np.zeros([dim] + n[::-1])
    for k in np.ndindex(*n):
        x = [case["x_lower"][d] + (lo[d] + k[d] - case["ilower"][d] + 0.5) * case["dx"][d] for d in range(dim)]
        arr[(slice(None),) + tuple(k[::-1])] = gr.poly_value(case["function"], x)
    X = np.asarray(case["X"])
    P = oracle.make_patch(dim, case["ilower"], case["iupper"], case["x_lower"], case["x_upper"], dx=case["dx"])
    idx = np.empty(X.size // dim, dtype=np.int32)
    cnt = oracle.lib().ibxo_build_local_indices(oracle.ctypes.byref(P), oracle.ivec(case["ilower"]),
                                                oracle.ivec(case["iupper"]), oracle.dptr(X), X.size // dim,
                                                oracle.iptr(idx))
    Q_t = torch.zeros(X.size, dtype=torch.float64, device="cuda")
    prob = ibx.make_problem(dim, ibx.CELL, ibx.MODE_PATCH, case["ilower"], case["iupper"], case["dx"],
                            case["x_lower"], case["x_upper"], dev(arr), dev(X), Q_t, Q_depth=dim, q_depth=dim,
                            gcw=[g] * dim, indices=dev(idx[:cnt], torch.int32))
    ibx.interpolate(prob, case["kernel"])
    Q = Q_t.cpu().numpy()
    for s in idx[:cnt]:
        exact = gr.poly_value(case["function"], X[dim * s: dim * s + dim])
        assert np.all(np.abs(Q[dim * s: dim * s + dim] - exact) <= case["tolerance"])
    assert cnt == X.size // dim
