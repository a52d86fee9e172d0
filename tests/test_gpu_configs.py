"""The benchmark workloads at their full sizes.

- 2D ellipse of 256 spring-connected markers on a 64^2 periodic MAC grid,
  IB_4: plain FP64 form against the oracle within 1e-12, mixed form within
  1e-5.
- 3D Fibonacci sphere shell of 200,000 markers on 128^3, IB_4 and
  BSPLINE_4: the same two bars.
- 3D clustered set of 2,000,000 markers (64 helices of 25,000 + 400,000
  uniform) on 256^3, IB_4 and IB_6, mixed form: within 1e-5 of the plain FP64
  form (itself pinned to the oracle above), stencil bases bit-exact against a
  vectorised restatement of the oracle's NINT rule (checked against the oracle
  on a sample), and the counting sort a permutation grouped by home tile.
"""

import numpy as np
import pytest

from tests import cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

PLAIN_TOL = 1e-12
MIXED_TOL = 1e-5


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available()
    m.lib()
    return m


@pytest.fixture(scope="module")
def workloads():
    from ibamr_gb300 import workloads as w

    return w


def side_problem(ibx, dim, N, q, X_t, Q_t):
    return ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [N - 1] * dim, [1.0 / N] * dim,
                            [0.0] * dim, [1.0] * dim, q, X_t, Q_t)


def run_plain(ibx, dim, N, kernel, X, F, u):
    X_t = torch.tensor(X, device="cuda")
    f_t = [torch.zeros([N] * dim, dtype=torch.float64, device="cuda") for _ in range(dim)]
    ibx.spread(side_problem(ibx, dim, N, f_t, X_t, torch.tensor(F, device="cuda")), kernel)
    u_t = [torch.tensor(u[a], device="cuda") for a in range(dim)]
    U_t = torch.zeros(X.size, dtype=torch.float64, device="cuda")
    ibx.interpolate(side_problem(ibx, dim, N, u_t, X_t, U_t), kernel)
    torch.cuda.synchronize()
    return torch.stack(f_t), U_t


def run_mixed(ibx, dim, N, kernel, X, F, u):
    X_t = torch.tensor(X, device="cuda")
    f_t = [torch.zeros([N] * dim, dtype=torch.float32, device="cuda") for _ in range(dim)]
    u_t = [torch.tensor(u[a], dtype=torch.float32, device="cuda") for a in range(dim)]
    F_t = torch.tensor(F, dtype=torch.float32, device="cuda")
    U_t = torch.zeros(X.size, dtype=torch.float32, device="cuda")
    plan = ibx.Plan(side_problem(ibx, dim, N, f_t, X_t, F_t), kernel, ibx.MIXED,
                    interp_problems=[side_problem(ibx, dim, N, u_t, X_t, U_t)])
    plan.bin()
    plan.spread()
    plan.interpolate()
    torch.cuda.synchronize()
    assert plan.status() == ibx.OK
    return torch.stack(f_t), U_t, plan


def rel(a, b):
    a = torch.as_tensor(a, device="cuda", dtype=torch.float64)
    b = torch.as_tensor(b, device="cuda", dtype=torch.float64)
    return float((a - b).abs().max() / b.abs().max())


def test_ellipse_64_ib4(ibx, oracle, workloads):
    X, F = workloads.ellipse_springs(256)
    rng = np.random.default_rng(workloads.SEED + 1)
    u = rng.standard_normal((2, 64, 64))
    f_ref, U_ref = oracle.periodic_side_problem(2, [64, 64], "IB_4", X, F=F, u=u)
    f, U = run_plain(ibx, 2, 64, "IB_4", X, F, u)
    assert rel(f, f_ref) <= PLAIN_TOL and rel(U, U_ref) <= PLAIN_TOL
    fm, Um, plan = run_mixed(ibx, 2, 64, "IB_4", X, F, u)
    assert rel(fm, f_ref) <= MIXED_TOL and rel(Um, U_ref) <= MIXED_TOL
    plan.close()


@pytest.mark.parametrize("kernel", ["IB_4", "BSPLINE_4"])
def test_fibonacci_shell_128(ibx, oracle, workloads, kernel):
    X = workloads.fibonacci_shell(200_000, 128)
    rng = np.random.default_rng(workloads.SEED + 2)
    F = rng.standard_normal(X.size)
    u = rng.standard_normal((3, 128, 128, 128))
    f_ref, U_ref = oracle.periodic_side_problem(3, [128] * 3, kernel, X, F=F, u=u)
    f, U = run_plain(ibx, 3, 128, kernel, X, F, u)
    assert rel(f, f_ref) <= PLAIN_TOL and rel(U, U_ref) <= PLAIN_TOL
    fm, Um, plan = run_mixed(ibx, 3, 128, kernel, X, F, u)
    assert rel(fm, f_ref) <= MIXED_TOL and rel(Um, U_ref) <= MIXED_TOL
    plan.close()


def nint_bases(X, dim, N, width, side_axis):
    """Vectorised stencil base of the NINT kernels (IB_4: width 4, IB_6:
    width 6) at ilower = 0, shifted into [0, N) by the cell-centred base."""
    n = X.size // dim
    Xv = X.reshape(n, dim)
    dx = 1.0 / N
    out_c = np.zeros((n, dim), dtype=np.int64)
    out_s = np.zeros((n, dim), dtype=np.int64)
    for d in range(dim):
        def base(xlo):
            t = ((Xv[:, d] + 0.0) - xlo) / dx
            r = np.where(t >= 0, np.trunc(t + 0.5), np.trunc(t - 0.5)).astype(np.int64)
            return r - width // 2
        b0 = base(0.0)
        b1 = base(0.0 - 0.5 * dx)
        sh = (b0 // N) * N
        out_c[:, d] = b0 - sh
        out_s[:, d] = b1 - sh
    return out_c, out_s


@pytest.mark.parametrize("kernel,width", [("IB_4", 4), ("IB_6", 6)])
def test_helices_256_mixed(ibx, oracle, workloads, kernel, width):
    X = workloads.helices_and_uniform()
    n = X.size // 3
    assert n == 2_000_000
    rng = np.random.default_rng(workloads.SEED + 3)
    F = rng.standard_normal(X.size)
    u = rng.standard_normal((3, 256, 256, 256)).astype(np.float32)
    f, U = run_plain(ibx, 3, 256, kernel, X, F, u.astype(np.float64))
    fm, Um, plan = run_mixed(ibx, 3, 256, kernel, X, F, u)
    e_f, e_U = rel(fm, f), rel(Um, U)
    assert e_f <= MIXED_TOL and e_U <= MIXED_TOL, (e_f, e_U)
    del f, U, fm, Um
    # stencil bases: vectorised rule, itself checked against the oracle
    bc, bs, ht, ts, hl = plan.bins(n)
    ebc, ebs = nint_bases(X, 3, 256, width, None)
    for s in rng.choice(n, size=500, replace=False):
        for d in range(3):
            b0 = oracle.stencil_1d(kernel, X[3 * s + d], 0.0, 0.0, 1.0 / 256, 0, 255, 10 ** 6)[0]
            assert b0 - (b0 // 256) * 256 == ebc[s, d]
    assert np.array_equal(bc.reshape(n, 3), ebc)
    assert np.array_equal(bs.reshape(n, 3), ebs)
    # counting sort: a permutation, grouped by home tile, tiles in order
    counts = np.bincount(ht, minlength=plan.n_tiles)
    assert ts[0] == 0 and np.array_equal(np.diff(ts), counts)
    assert np.array_equal(np.sort(hl), np.arange(n))
    assert np.all(np.diff(ht[hl]) >= 0)
    plan.close()
