"""The allocation-free spread entry point (ibx_spread_noalloc).

Some callers of this library cannot allocate device memory: a real-time or
fault-handling host path, where cudaMalloc may block on the driver or fail
when memory is short, or an embedding whose own pool manager owns the whole
device.  They spread through ibx_spread_noalloc, which keeps its scratch in
a fixed array inside the library.  Its result must match the plan-based entry
point (ibx_plan_bin + ibx_plan_spread) within the mixed-precision tolerance,
and the FP64 oracle within the same tolerance, on two calls in a row -- the
second call must not see anything the first left in the shared scratch
array.  The cases cover 2D and 3D, side- and cell-centred data, IB_4, IB_6
and BSPLINE_4, and grids whose cell count is not a multiple of the tile edge
with markers crowding the periodic seam (each such marker's footprint then
touches three tiles per dimension).  This file runs last: it is the one test
that exercises the static scratch array.
"""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5

# (dim, centering, depth, N, kernel, markers, layout)
CASES = [
    (3, "side", 1, [32, 32, 32], "IB_4", 20000, "cluster+uniform"),
    (3, "side", 1, [32, 32, 32], "BSPLINE_4", 20000, "cluster+uniform"),
    (3, "side", 1, [17, 20, 18], "IB_4", 240, "seam"),
    (3, "side", 1, [20, 20, 20], "IB_6", 6000, "seam+uniform"),
    (3, "cell", 2, [24, 24, 24], "IB_6", 8000, "cluster+uniform"),
    (2, "side", 1, [100, 90], "IB_4", 12000, "cluster+uniform"),
    (2, "cell", 1, [50, 34], "IB_4", 3000, "seam+uniform"),
]


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available()
    L = m.lib()
    L.ibx_spread_noalloc.argtypes = [ctypes.POINTER(m.Problem), ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
    return m


def markers(rng, dim, N, n, layout):
    """Positions in [0,1)^dim: a tight cluster (dense home tiles) plus uniform
    markers, or markers within half a cell of the periodic corner (their
    footprints wrap in every dimension) plus uniform markers."""
    parts = []
    if layout.startswith("cluster"):
        m = n // 2
        parts.append(0.5 + 0.05 * rng.standard_normal((m, dim)))
    else:
        m = n if layout == "seam" else n // 4
        h = np.array([1.0 / v for v in N])
        parts.append(rng.uniform(-0.5, 0.5, size=(m, dim)) * h)
    parts.append(rng.uniform(0.0, 1.0, size=(n - m, dim)))
    return np.mod(np.concatenate(parts), 1.0).reshape(-1)


def grid_tensors(dim, centering, depth, N):
    if centering == "side":
        return [torch.zeros(N[::-1], dtype=torch.float32, device="cuda") for _ in range(dim)]
    return torch.zeros([depth] + N[::-1], dtype=torch.float32, device="cuda")


def make(ibx, dim, centering, depth, N, f, X, F):
    cen = ibx.SIDE if centering == "side" else ibx.CELL
    return ibx.make_problem(dim, cen, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N], [1.0 / v for v in N],
                            [0.0] * dim, [1.0] * dim, f, X, F, q_depth=1 if centering == "side" else depth)


def noalloc_spread(ibx, prob, kernel, status=None):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    sp = None if status is None else ctypes.c_void_p(status.data_ptr())
    return ibx.lib().ibx_spread_noalloc(ctypes.byref(prob), ibx.kernel_id(kernel), sp, stream)


def as_np(f):
    if isinstance(f, list):
        return np.stack([t.double().cpu().numpy() for t in f])
    return f.double().cpu().numpy()


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("case", CASES, ids=lambda c: "%dd-%s-%s-%s-%s" % (c[0], c[1], "x".join(map(str, c[3])),
                                                                              c[4], c[6]))
def test_noalloc_matches_plan_and_oracle_on_two_calls(ibx, oracle, case):
    dim, centering, depth, N, kernel, n, layout = case
    Q_depth = dim if centering == "side" else depth
    rng = np.random.default_rng(2024 + n)
    status = torch.full([1], -1, dtype=torch.int32, device="cuda")
    for call in range(2):
        # Fresh markers and forces on each call; fresh zeroed grids.
        X = markers(rng, dim, N, n, layout)
        F = rng.standard_normal(Q_depth * n)
        X_t = torch.tensor(X, device="cuda")
        F_t = torch.tensor(F, dtype=torch.float32, device="cuda")
        f_na = grid_tensors(dim, centering, depth, N)
        f_pl = grid_tensors(dim, centering, depth, N)
        status.fill_(-1)
        rc = noalloc_spread(ibx, make(ibx, dim, centering, depth, N, f_na, X_t, F_t), kernel, status)
        assert rc == ibx.OK, ibx.status_string(rc)
        plan = ibx.Plan(make(ibx, dim, centering, depth, N, f_pl, X_t, F_t), kernel, ibx.MIXED)
        plan.bin()
        plan.spread()
        torch.cuda.synchronize()
        assert plan.status() == ibx.OK
        plan.close()
        assert int(status.item()) == ibx.OK
        a, b = as_np(f_na), as_np(f_pl)
        assert rel(a, b) <= MIXED_TOL, (call, rel(a, b))
        f_ref, _ = oracle.periodic_problem(dim, N, kernel, X, F=F, centering=1 if centering == "side" else 0,
                                           depth=depth)
        assert rel(a.reshape(f_ref.shape), f_ref) <= MIXED_TOL, (call, rel(a.reshape(f_ref.shape), f_ref))


def test_noalloc_reports_nonfinite_markers(ibx, oracle):
    dim, N, n = 3, [16, 16, 16], 500
    rng = np.random.default_rng(9)
    X = rng.uniform(0.0, 1.0, size=n * dim)
    F = rng.standard_normal(n * dim)
    X_bad = X.copy()
    X_bad[3 * 7 + 1] = np.nan  # marker 7 is skipped and reported
    f = grid_tensors(dim, "side", 1, N)
    status = torch.full([1], -1, dtype=torch.int32, device="cuda")
    rc = noalloc_spread(ibx, make(ibx, dim, "side", 1, N, f, torch.tensor(X_bad, device="cuda"),
                                  torch.tensor(F, dtype=torch.float32, device="cuda")), "IB_4", status)
    assert rc == ibx.OK
    torch.cuda.synchronize()
    assert int(status.item()) == ibx.E_NONFINITE
    keep = np.ones(n, dtype=bool)
    keep[7] = False
    f_ref, _ = oracle.periodic_problem(dim, N, "IB_4", X.reshape(n, dim)[keep].reshape(-1),
                                       F=F.reshape(n, dim)[keep].reshape(-1))
    assert rel(as_np(f), f_ref) <= MIXED_TOL


def test_noalloc_rejects_oversized_problems(ibx):
    n = 32769  # one marker above IBX_NOALLOC_MAX_MARKERS
    X = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    F = torch.zeros(3 * n, dtype=torch.float32, device="cuda")
    f = [torch.zeros([16, 16, 16], dtype=torch.float32, device="cuda") for _ in range(3)]
    assert noalloc_spread(ibx, make(ibx, 3, "side", 1, [16, 16, 16], f, X, F), "IB_4") == ibx.E_TOO_LARGE
    # 33 x 33 x 33 tiles of 8^3 cells exceed IBX_NOALLOC_MAX_TILES (4096).
    N = [264, 264, 264]
    X = torch.zeros(3 * 10, dtype=torch.float64, device="cuda")
    F = torch.zeros(3 * 10, dtype=torch.float32, device="cuda")
    g = [torch.zeros([1], dtype=torch.float32, device="cuda") for _ in range(3)]
    assert noalloc_spread(ibx, make(ibx, 3, "side", 1, N, g, X, F), "IB_4") == ibx.E_TOO_LARGE
