"""The allocation-free spread entry point (ibx_spread_noalloc).

Callers that cannot allocate device memory (graph capture with a fixed
footprint, real-time paths, embeddings whose pool owns the device) spread
through ibx_spread_noalloc, which keeps its scratch in a fixed array inside
the library.  Its result must match the plan-based entry point
(ibx_plan_bin + ibx_plan_spread) within the mixed-precision tolerance, on
two calls in a row -- the second call must not see anything the first left
in the shared scratch array.  This file runs last: it is the one test that
exercises the static scratch array.
"""

import ctypes

import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available()
    L = m.lib()
    L.ibx_spread_noalloc.argtypes = [ctypes.POINTER(m.Problem), ctypes.c_int, ctypes.c_void_p]
    return m


def side_problem(ibx, N, f, X, F):
    dim = len(N)
    return ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [n - 1 for n in N], [1.0 / n for n in N],
                            [0.0] * dim, [1.0] * dim, f, X, F)


def noalloc_spread(ibx, prob, kernel):
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    return ibx.lib().ibx_spread_noalloc(ctypes.byref(prob), ibx.kernel_id(kernel), stream)


def rel(a, b):
    a = np.stack([t.double().cpu().numpy() for t in a])
    b = np.stack([t.double().cpu().numpy() for t in b])
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


@pytest.mark.parametrize("kernel", ["IB_4", "BSPLINE_4"])
def test_noalloc_matches_plan_on_two_calls(ibx, kernel):
    rng = np.random.default_rng(2024)
    N = [32, 32, 32]
    n = 20000
    grids = lambda: [torch.zeros(N[::-1], dtype=torch.float32, device="cuda") for _ in range(3)]
    f_na, f_ref = grids(), grids()
    for call in range(2):
        # Fresh markers and forces on each call: a fibre-like cluster plus
        # uniform markers, so both the dense and the sparse tile paths run.
        Xc = 0.5 + 0.05 * rng.standard_normal((n // 2, 3))
        Xu = rng.uniform(0.0, 1.0, size=(n - n // 2, 3))
        X = torch.tensor(np.mod(np.concatenate([Xc, Xu]), 1.0).reshape(-1), device="cuda")
        F = torch.tensor(rng.standard_normal(3 * n), dtype=torch.float32, device="cuda")
        rc = noalloc_spread(ibx, side_problem(ibx, N, f_na, X, F), kernel)
        assert rc == ibx.OK, ibx.status_string(rc)
        plan = ibx.Plan(side_problem(ibx, N, f_ref, X, F), kernel, ibx.MIXED)
        plan.bin()
        plan.spread()
        torch.cuda.synchronize()
        plan.close()
        assert rel(f_na, f_ref) <= MIXED_TOL, (call, rel(f_na, f_ref))


def test_noalloc_rejects_oversized_problems(ibx):
    n = 32769  # one marker above IBX_NOALLOC_MAX_MARKERS
    X = torch.zeros(3 * n, dtype=torch.float64, device="cuda")
    F = torch.zeros(3 * n, dtype=torch.float32, device="cuda")
    f = [torch.zeros([16, 16, 16], dtype=torch.float32, device="cuda") for _ in range(3)]
    assert noalloc_spread(ibx, side_problem(ibx, [16, 16, 16], f, X, F), "IB_4") == ibx.E_TOO_LARGE
    # 33 x 33 x 33 tiles of 8^3 cells exceed IBX_NOALLOC_MAX_TILES (4096).
    N = [264, 264, 264]
    X = torch.zeros(3 * 10, dtype=torch.float64, device="cuda")
    F = torch.zeros(3 * 10, dtype=torch.float32, device="cuda")
    g = [torch.zeros([1], dtype=torch.float32, device="cuda") for _ in range(3)]
    assert noalloc_spread(ibx, side_problem(ibx, N, g, X, F), "IB_4") == ibx.E_TOO_LARGE
