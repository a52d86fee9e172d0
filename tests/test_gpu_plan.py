"""Binned plan pipeline (mixed precision) against the FP64 oracle.

Bars: stencil bases and the counting sort bit-exact; spread and
interpolation within 1e-5 relative (max-norm over the grid and over the
markers) of the FP64 oracle, the tolerance the mixed form is held to.
"""

import numpy as np
import pytest

from tests import cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

KERNEL_NAMES = ["PIECEWISE_LINEAR", "PIECEWISE_CUBIC", "IB_3", "IB_4", "IB_6", "BSPLINE_4"]
MIXED_TOL = 1e-5


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available()
    m.lib()
    return m


def seam_markers(rng, n, dim):
    X = rng.uniform(0.0, 1.0, size=(n, dim))
    k = n // 8
    X[:k] = rng.uniform(0.0, 0.03, size=(k, dim))
    X[k: 2 * k] = rng.uniform(0.97, 1.0, size=(k, dim))
    return X.reshape(-1)


def run_plan(ibx, dim, N, kernel, X, F, u, centering, depth, dense_min=None, tile_shape=0, visit_kernel=0,
             interp_kernel=None):
    ncomp = dim if centering == ibx.SIDE else depth
    shape = list(N)[::-1]
    dx = [1.0 / v for v in N]
    X_t = torch.tensor(X, device="cuda")
    if centering == ibx.SIDE:
        f_t = [torch.zeros(shape, dtype=torch.float32, device="cuda") for _ in range(dim)]
        u_t = [torch.tensor(u[a], dtype=torch.float32, device="cuda") for a in range(dim)]
        fq, uq = f_t, u_t
    else:
        f_t = torch.zeros([depth] + shape, dtype=torch.float32, device="cuda")
        u_t = torch.tensor(u, dtype=torch.float32, device="cuda")
        fq, uq = f_t, u_t
    F_t = torch.tensor(F, dtype=torch.float32, device="cuda")
    U_t = torch.zeros(X.size // dim * ncomp, dtype=torch.float32, device="cuda")
    mk = lambda q, Q: ibx.make_problem(dim, centering, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N], dx,
                                       [0.0] * dim, [1.0] * dim, q, X_t, Q, q_depth=1 if centering else depth,
                                       Q_depth=ncomp)
    ps = ibx.Plan(mk(fq, F_t), kernel, ibx.MIXED, tile_shape=tile_shape)
    pi = ibx.Plan(mk(uq, U_t), kernel, ibx.MIXED, tile_shape=tile_shape)
    if dense_min is not None:
        ps.set_tuning(dense_min=dense_min)
        pi.set_tuning(dense_min=dense_min)
    ps.visit_kernel = visit_kernel
    if interp_kernel is not None:
        pi.interp_kernel = interp_kernel
    ps.bin()
    ps.spread()
    pi.bin()
    pi.interpolate()
    torch.cuda.synchronize()
    f = np.stack([t.double().cpu().numpy() for t in f_t]) if centering == ibx.SIDE else f_t.double().cpu().numpy()
    return f, U_t.double().cpu().numpy(), ps, pi


# dense_min 0: every tile spread by its home region (tile + halo, global
# atomics); 2^30: every marker spread through its visits (owner
# read-modify-write); None: the default split.
@pytest.mark.parametrize("tile_shape", [0, 1])
@pytest.mark.parametrize("dense_min", [None, 0, 1 << 30])
@pytest.mark.parametrize("kernel", KERNEL_NAMES)
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("centering,depth", [(1, 1), (0, 1), (0, 3)])
def test_plan_mixed_matches_fp64_oracle(ibx, oracle, kernel, dim, centering, depth, dense_min, tile_shape):
    rng = np.random.default_rng(11 + dim + 100 * centering + 10 * depth + 1000 * KERNEL_NAMES.index(kernel))
    N = [32, 24, 20][:dim] if dim == 3 else [48, 40]
    n = 3000
    X = seam_markers(rng, n, dim)
    ncomp = dim if centering == 1 else depth
    F = rng.standard_normal(n * ncomp)
    u = rng.standard_normal([ncomp] + list(N)[::-1])
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=centering, depth=depth)
    f, U, ps, pi = run_plan(ibx, dim, N, kernel, X, F, u, centering, depth, dense_min=dense_min,
                            tile_shape=tile_shape)
    assert cases.rel_err(f, f_ref) <= MIXED_TOL
    assert cases.rel_err(U, U_ref) <= MIXED_TOL
    assert ps.status() == ibx.OK and pi.status() == ibx.OK
    assert ps.tile_shape[0] == tile_shape
    ps.close()
    pi.close()


@pytest.mark.parametrize("tile_shape", [0, 1])
@pytest.mark.parametrize("dense_min", [0, 1 << 30])
@pytest.mark.parametrize("kernel", ["IB_4", "IB_6", "PIECEWISE_LINEAR"])
@pytest.mark.parametrize("dim,N", [(2, [37, 23]), (3, [19, 13, 11])])
@pytest.mark.parametrize("centering", [0, 1])
def test_plan_odd_grid_sizes(ibx, oracle, kernel, dim, N, centering, dense_min, tile_shape):
    """Grids whose sizes are not multiples of the tile edge or of 4 (partial
    tiles, scalar row updates, regions wrapping across the periodic seam)."""
    rng = np.random.default_rng(7 + dim + 31 * centering + (dense_min > 0))
    n = 1500
    X = seam_markers(rng, n, dim)
    ncomp = dim if centering == 1 else 1
    F = rng.standard_normal(n * ncomp)
    u = rng.standard_normal([ncomp] + list(N)[::-1])
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=centering, depth=1)
    f, U, ps, pi = run_plan(ibx, dim, N, kernel, X, F, u, centering, 1, dense_min=dense_min, tile_shape=tile_shape)
    assert cases.rel_err(f, f_ref) <= MIXED_TOL
    assert cases.rel_err(U, U_ref) <= MIXED_TOL
    assert ps.status() == ibx.OK
    ps.close()
    pi.close()


def expected_bases(oracle, kernel, X, dim, N):
    """Stencil bases by the oracle's Fortran rules, relative to ilower = 0,
    both shifted by the multiple of N that puts the cell-centred one in [0, N)."""
    n = X.size // dim
    bc = np.zeros((n, 3), dtype=np.int64)
    bs = np.zeros((n, 3), dtype=np.int64)
    for s in range(n):
        for d in range(dim):
            dx = 1.0 / N[d]
            b0 = oracle.stencil_1d(kernel, X[dim * s + d], 0.0, 0.0, dx, 0, N[d] - 1, 10 ** 6)[0]
            b1 = oracle.stencil_1d(kernel, X[dim * s + d], 0.0, 0.0 - 0.5 * dx, dx, 0, N[d] - 1, 10 ** 6)[0]
            sh = (b0 // N[d]) * N[d]
            bc[s, d] = b0 - sh
            bs[s, d] = b1 - sh
    return bc, bs


def adversarial_positions(rng, dim, N, n):
    """Positions on and one ulp either side of the decision boundaries of the
    index rules (cell faces, quarter points, cell centres), plus 0, 1-ulp and
    tiny values, drawn independently per dimension."""
    cols = []
    for d in range(dim):
        base = []
        for k in range(0, N[d], max(1, N[d] // 16)):
            for frac in (0.0, 0.25, 0.5, 0.75):
                x = (k + frac) / N[d]
                base += [x, np.nextafter(x, -1.0), np.nextafter(x, 2.0)]
        base += [0.0, np.nextafter(1.0, 0.0), 5e-324, 1e-300]
        base = np.array([b for b in base if 0.0 <= b < 1.0])
        cols.append(rng.choice(base, size=n))
    return np.stack(cols, axis=1).reshape(-1)


@pytest.mark.parametrize("tile_shape", [0, 1])
@pytest.mark.parametrize("kernel", KERNEL_NAMES)
@pytest.mark.parametrize("dim", [2, 3])
def test_binning_bit_exact(ibx, oracle, kernel, dim, tile_shape):
    rng = np.random.default_rng(5 + dim + 17 * KERNEL_NAMES.index(kernel))
    N = [64, 64, 64][:dim] if dim == 3 else [128, 96]
    n = 4000
    X = np.concatenate([rng.uniform(0.0, 1.0, size=n * dim), adversarial_positions(rng, dim, N, n)])
    n = X.size // dim
    F = np.zeros(n * dim)
    u = np.zeros([dim] + list(N)[::-1])
    _, _, ps, pi = run_plan(ibx, dim, N, kernel, X, F, u, 1, 1, tile_shape=tile_shape)
    bc, bs, ht, ts, hl = ps.bins(n)
    ebc, ebs = expected_bases(oracle, kernel, X, dim, N)
    assert np.array_equal(bc.reshape(n, 3)[:, :dim], ebc[:, :dim])
    assert np.array_equal(bs.reshape(n, 3)[:, :dim], ebs[:, :dim])
    # counting sort: tile_start is the exclusive scan of the home-tile counts,
    # and every tile's segment holds exactly its markers.
    counts = np.bincount(ht, minlength=ps.n_tiles)
    assert ts[0] == 0 and np.array_equal(np.diff(ts), counts)
    assert np.array_equal(np.sort(hl), np.arange(n))
    for t in rng.choice(ps.n_tiles, size=min(64, ps.n_tiles), replace=False):
        seg = hl[ts[t]:ts[t + 1]]
        assert np.all(ht[seg] == t)
    ps.close()
    pi.close()


def test_batched_plan_matches_per_problem(ibx, oracle):
    """Several problems of different sizes in one plan give the oracle's
    answer for each (the batched form used for many independent problems)."""
    rng = np.random.default_rng(99)
    dim, kernel = 2, "IB_4"
    sizes = [32, 64, 48, 128]
    X_t, F_t, U_t, f_t, u_t, probs_s, probs_i, refs = [], [], [], [], [], [], [], []
    for N0 in sizes:
        N = [N0, N0]
        n = int(rng.integers(100, 2000))
        X = seam_markers(rng, n, dim)
        F = rng.standard_normal(n * dim)
        u = rng.standard_normal([dim, N0, N0])
        refs.append(oracle.periodic_problem(dim, N, kernel, X, F=F, u=u))
        xt = torch.tensor(X, device="cuda")
        ft = [torch.zeros([N0, N0], dtype=torch.float32, device="cuda") for _ in range(dim)]
        ut = [torch.tensor(u[a], dtype=torch.float32, device="cuda") for a in range(dim)]
        Ft = torch.tensor(F, dtype=torch.float32, device="cuda")
        Ut = torch.zeros(n * dim, dtype=torch.float32, device="cuda")
        dx = [1.0 / N0] * 2
        probs_s.append(ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0, 0], [N0 - 1] * 2, dx, [0, 0], [1, 1], ft,
                                        xt, Ft))
        probs_i.append(ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0, 0], [N0 - 1] * 2, dx, [0, 0], [1, 1], ut,
                                        xt, Ut))
        f_t.append(ft)
        U_t.append(Ut)
    ps = ibx.Plan(probs_s, kernel, ibx.MIXED)
    pi = ibx.Plan(probs_i, kernel, ibx.MIXED)
    ps.bin()
    ps.spread()
    pi.bin()
    pi.interpolate()
    torch.cuda.synchronize()
    for k in range(len(sizes)):
        f = np.stack([t.double().cpu().numpy() for t in f_t[k]])
        assert cases.rel_err(f, refs[k][0]) <= MIXED_TOL
        assert cases.rel_err(U_t[k].double().cpu().numpy(), refs[k][1]) <= MIXED_TOL
    ps.close()
    pi.close()


def test_nonfinite_marker_is_reported_and_skipped(ibx, oracle):
    rng = np.random.default_rng(3)
    dim, N, kernel = 3, [16, 16, 16], "IB_4"
    n = 500
    X = rng.uniform(0, 1, size=n * dim)
    X[7 * dim + 1] = np.nan
    F = rng.standard_normal(n * dim)
    F[7 * dim: 8 * dim] = 0.0
    u = rng.standard_normal([dim] + N)
    keep = np.ones(n, bool)
    keep[7] = False
    Xk = X.reshape(n, dim)[keep].reshape(-1)
    f_ref, _ = oracle.periodic_problem(dim, N, kernel, Xk, F=F.reshape(n, dim)[keep].reshape(-1), u=u)
    f, U, ps, pi = run_plan(ibx, dim, N, kernel, X, F, u, 1, 1)
    assert ps.status() == ibx.E_NONFINITE
    assert ps.status() == ibx.OK  # the word is cleared by reading it
    assert cases.rel_err(f, f_ref) <= MIXED_TOL
    ps.close()
    pi.close()


def test_autotune_applies_a_measured_setting(ibx, oracle):
    """The autotuner times every candidate, keeps the fastest, and the tuned
    plan still matches the oracle (tuning changes the schedule, not the sums
    beyond FP32 rounding)."""
    from ibamr_gb300 import tuning

    rng = np.random.default_rng(21)
    dim, N, kernel = 3, [32, 32, 32], "IB_4"
    n = 4000
    X = seam_markers(rng, n, dim)
    F = rng.standard_normal(n * dim)
    u = rng.standard_normal([dim] + N)
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=1)
    X_t = torch.tensor(X, device="cuda")
    f_t = [torch.zeros(N, dtype=torch.float32, device="cuda") for _ in range(dim)]
    F_t = torch.tensor(F, dtype=torch.float32, device="cuda")
    mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * 3, [31] * 3, [1 / 32] * 3, [0.0] * 3,
                                       [1.0] * 3, q, X_t, Q)
    plan = ibx.Plan(mk(f_t, F_t), kernel, ibx.MIXED)
    res = tuning.autotune(plan, reps=1, candidates={"dense_min": (0, 32, 1 << 30), "item_units": (32, 256),
                                                    "dense_blocks_per_sm": (1, 2), "unit_cap": (32,)})
    forms = tuning.DEFAULT_CANDIDATES["visit_kernel"]
    assert len(res["table"]) == 3 * len(forms) + 4 and res["visit_kernel"] in forms
    assert plan.tuning() == res["best"] and plan.visit_kernel == res["visit_kernel"]
    cfg, ms = min(res["table"], key=lambda r: r[1])
    assert res["best"] == cfg[:3] and res["ms"] == ms
    for t in f_t:
        t.zero_()
    plan.bin()
    plan.spread()
    torch.cuda.synchronize()
    f = np.stack([t.double().cpu().numpy() for t in f_t])
    assert cases.rel_err(f, f_ref) <= MIXED_TOL
    plan.close()


def test_plan_edge_cases_empty_and_boundary_positions(ibx, oracle):
    """A problem without markers next to one with markers exactly on the
    periodic boundary (x = 0 and x = 1, the same point), in one plan."""
    dim, kernel = 2, "IB_4"
    N = [32, 32]
    dx = [1.0 / 32] * 2
    X1 = np.array([0.0, 0.0, 1.0, 1.0, 0.5, 1.0, 1.0, 0.25, 0.999999999999, 1e-300])
    n1 = X1.size // 2
    rng = np.random.default_rng(8)
    F1 = rng.standard_normal(n1 * 2)
    u1 = rng.standard_normal((2, 32, 32))
    X1w = np.mod(X1, 1.0)  # the oracle's periodic flow takes positions in [0, 1)
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X1w, F=F1, u=u1)
    tensors = []

    def prob(X, F, U, f, u):
        xt = torch.tensor(X, device="cuda")
        tensors.extend([xt])
        return (ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0, 0], [31, 31], dx, [0, 0], [1, 1], f, xt, F,
                                 n_markers=X.size // 2),
                ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0, 0], [31, 31], dx, [0, 0], [1, 1], u, xt, U,
                                 n_markers=X.size // 2))

    f0 = [torch.zeros(32, 32, dtype=torch.float32, device="cuda") for _ in range(2)]
    u0 = [torch.zeros(32, 32, dtype=torch.float32, device="cuda") for _ in range(2)]
    f1 = [torch.zeros(32, 32, dtype=torch.float32, device="cuda") for _ in range(2)]
    u1t = [torch.tensor(u1[a], dtype=torch.float32, device="cuda") for a in range(2)]
    e = torch.zeros(2, dtype=torch.float32, device="cuda")
    F1t = torch.tensor(F1, dtype=torch.float32, device="cuda")
    U1t = torch.zeros(n1 * 2, dtype=torch.float32, device="cuda")
    s0, i0 = prob(np.zeros(0), e, e, f0, u0)
    s1, i1 = prob(X1, F1t, U1t, f1, u1t)
    for dense_min in (0, 1 << 30):
        for t in f1:
            t.zero_()
        plan = ibx.Plan([s0, s1], kernel, ibx.MIXED, interp_problems=[i0, i1])
        plan.set_tuning(dense_min=dense_min)
        plan.bin()
        plan.spread()
        plan.interpolate()
        torch.cuda.synchronize()
        assert plan.status() == ibx.OK
        f = np.stack([t.double().cpu().numpy() for t in f1])
        assert cases.rel_err(f, f_ref) <= MIXED_TOL
        assert cases.rel_err(U1t.double().cpu().numpy(), U_ref) <= MIXED_TOL
        assert all(float(t.abs().max()) == 0.0 for t in f0)
        plan.close()


def test_autotune_shape_keeps_the_fastest_plan(ibx, oracle):
    from ibamr_gb300 import tuning

    rng = np.random.default_rng(22)
    dim, N, kernel = 2, [64, 48], "IB_4"
    n = 3000
    X = seam_markers(rng, n, dim)
    F = rng.standard_normal(n * dim)
    u = rng.standard_normal([dim] + N[::-1])
    f_ref, _ = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=1)
    X_t = torch.tensor(X, device="cuda")
    f_t = [torch.zeros(N[::-1], dtype=torch.float32, device="cuda") for _ in range(dim)]
    F_t = torch.tensor(F, dtype=torch.float32, device="cuda")
    make = lambda sh: ibx.Plan(ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0, 0], [63, 47],
                                                [1 / 64, 1 / 48], [0, 0], [1, 1], f_t, X_t, F_t), kernel,
                               ibx.MIXED, tile_shape=sh)
    plan, res = tuning.autotune_shape(make, reps=1, candidates={"dense_min": (0, 1 << 30), "item_units": (64,),
                                                                "dense_blocks_per_sm": (2,)})
    assert set(res["per_shape"]) == {0, 1}
    assert plan.tile_shape[0] == res["shape"]
    assert res["ms"] == min(v[1] for v in res["per_shape"].values())
    for t in f_t:
        t.zero_()
    plan.bin()
    plan.spread()
    torch.cuda.synchronize()
    f = np.stack([t.double().cpu().numpy() for t in f_t])
    assert cases.rel_err(f, f_ref) <= MIXED_TOL
    plan.close()


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("step_mode", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("interp_form", [0, 1, 2, 3, 4])
def test_plan_step_overlapped_equals_separate_calls(ibx, oracle, dim, interp_form, step_mode):
    """ibx_plan_step (spread and interpolation on two streams, the spread's
    first, both of one priority or the interpolation's first, or one after
    the other, or fused; the
    marker-order interpolation forked before the counting sort) gives the
    oracle's answer, step after step."""
    rng = np.random.default_rng(61 + dim)
    N = [24, 20, 16][:dim] if dim == 3 else [40, 36]
    n = 2500
    X = seam_markers(rng, n, dim)
    F = rng.standard_normal(n * dim)
    u = rng.standard_normal([dim] + list(N)[::-1])
    f_ref, U_ref = oracle.periodic_problem(dim, N, "IB_4", X, F=F, u=u, centering=1)
    X_t = torch.tensor(X, device="cuda")
    f_t = [torch.zeros(list(N)[::-1], dtype=torch.float32, device="cuda") for _ in range(dim)]
    u_t = [torch.tensor(u[a], dtype=torch.float32, device="cuda") for a in range(dim)]
    F_t = torch.tensor(F, dtype=torch.float32, device="cuda")
    U_t = torch.zeros(n * dim, dtype=torch.float32, device="cuda")
    mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N],
                                       [1.0 / v for v in N], [0.0] * dim, [1.0] * dim, q, X_t, Q)
    plan = ibx.Plan(mk(f_t, F_t), "IB_4", ibx.MIXED, interp_problems=[mk(u_t, U_t)])
    plan.interp_kernel = interp_form
    plan.step_mode = step_mode
    for _ in range(2):
        for t in f_t:
            t.zero_()
        U_t.zero_()
        plan.step()
        torch.cuda.synchronize()
        f = np.stack([t.double().cpu().numpy() for t in f_t])
        assert cases.rel_err(f, f_ref) <= MIXED_TOL
        assert cases.rel_err(U_t.double().cpu().numpy(), U_ref) <= MIXED_TOL
    assert plan.status() == ibx.OK
    plan.close()


@pytest.mark.parametrize("tile_shape", [0, 1])
@pytest.mark.parametrize("dense_min", [None, 0, 1 << 30])
@pytest.mark.parametrize("kernel", KERNEL_NAMES)
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("centering,depth", [(1, 1), (0, 3)])
def test_fused_step_matches_oracle_and_separate_launches(ibx, oracle, kernel, dim, centering, depth, tile_shape,
                                                         dense_min):
    """Step mode 2 (spread and interpolation of the binned markers in one
    persistent launch) against the oracle, step after step, and its
    interpolation bit-identical to the separate launches (step mode 0)."""
    rng = np.random.default_rng(131 + dim + 10 * centering + 100 * KERNEL_NAMES.index(kernel) + tile_shape)
    N = [26, 21, 18][:dim] if dim == 3 else [44, 37]
    n = 3000
    X = seam_markers(rng, n, dim)
    ncomp = dim if centering == 1 else depth
    F = rng.standard_normal(n * ncomp)
    u = rng.standard_normal([ncomp] + list(N)[::-1])
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=centering, depth=depth)
    shape = list(N)[::-1]
    X_t = torch.tensor(X, device="cuda")
    if centering == ibx.SIDE:
        f_t = [torch.zeros(shape, dtype=torch.float32, device="cuda") for _ in range(dim)]
        u_t = [torch.tensor(u[a], dtype=torch.float32, device="cuda") for a in range(dim)]
    else:
        f_t = torch.zeros([depth] + shape, dtype=torch.float32, device="cuda")
        u_t = torch.tensor(u, dtype=torch.float32, device="cuda")
    F_t = torch.tensor(F, dtype=torch.float32, device="cuda")
    U_t = torch.zeros(n * ncomp, dtype=torch.float32, device="cuda")
    mk = lambda q, Q: ibx.make_problem(dim, centering, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N],
                                       [1.0 / v for v in N], [0.0] * dim, [1.0] * dim, q, X_t, Q,
                                       q_depth=1 if centering else depth, Q_depth=ncomp)
    plan = ibx.Plan(mk(f_t, F_t), kernel, ibx.MIXED, interp_problems=[mk(u_t, U_t)], tile_shape=tile_shape)
    if dense_min is not None:
        plan.set_tuning(dense_min=dense_min)
    got = {}
    for mode in (0, 2, 2):
        plan.step_mode = mode
        assert plan.step_mode == mode
        for t in (f_t if centering == ibx.SIDE else [f_t]):
            t.zero_()
        U_t.zero_()
        plan.step()
        torch.cuda.synchronize()
        assert plan.status() == ibx.OK
        f = np.stack([t.double().cpu().numpy() for t in f_t]) if centering == ibx.SIDE else f_t.double().cpu().numpy()
        U = U_t.double().cpu().numpy()
        assert cases.rel_err(f, f_ref) <= MIXED_TOL
        assert cases.rel_err(U, U_ref) <= MIXED_TOL
        if mode in got:
            assert np.array_equal(U, got[mode])
        got[mode] = U
    assert np.array_equal(got[0], got[2])
    plan.close()


@pytest.mark.parametrize("x_source", ["pinned", "device"])
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("step_mode", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("interp_form", [1, 2])
def test_step_io_host_buffers_eager_and_captured(ibx, oracle, dim, step_mode, interp_form, x_source):
    """ibx_plan_step_io moves positions and forces in from pinned host memory
    (positions read by the binning straight from the host buffer, or copied
    from a device buffer) and the interpolated values out: the oracle's
    answer eagerly, and from a CUDA graph of the call replayed with new host
    forces and positions; the plan's position array holds the positions
    afterwards either way."""
    rng = np.random.default_rng(151 + dim + 3 * step_mode)
    N = [24, 20, 16][:dim] if dim == 3 else [40, 36]
    n = 2500
    X = seam_markers(rng, n, dim)
    F = rng.standard_normal(n * dim)
    u = rng.standard_normal([dim] + list(N)[::-1])
    X_t = torch.full((n * dim,), 0.5, dtype=torch.float64, device="cuda")
    f_t = [torch.zeros(list(N)[::-1], dtype=torch.float32, device="cuda") for _ in range(dim)]
    u_t = [torch.tensor(u[a], dtype=torch.float32, device="cuda") for a in range(dim)]
    F_t = torch.zeros(n * dim, dtype=torch.float32, device="cuda")
    U_t = torch.zeros(n * dim, dtype=torch.float32, device="cuda")
    Xh = torch.tensor(X).pin_memory() if x_source == "pinned" else torch.tensor(X, device="cuda")
    Fh = torch.tensor(F, dtype=torch.float32).pin_memory()
    Uh = torch.zeros(n * dim, dtype=torch.float32).pin_memory()
    mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N],
                                       [1.0 / v for v in N], [0.0] * dim, [1.0] * dim, q, X_t, Q)
    plan = ibx.Plan(mk(f_t, F_t), "IB_4", ibx.MIXED, interp_problems=[mk(u_t, U_t)])
    plan.interp_kernel = interp_form
    plan.step_mode = step_mode
    io = dict(in_X=[(X_t, Xh)], in_Q=[(F_t, Fh)], out_Q=[(Uh, U_t)])

    def check(Xc, Fc):
        f_ref, U_ref = oracle.periodic_problem(dim, N, "IB_4", Xc, F=Fc, u=u, centering=1)
        f = np.stack([t.double().cpu().numpy() for t in f_t])
        assert cases.rel_err(f, f_ref) <= MIXED_TOL
        assert cases.rel_err(Uh.double().numpy(), U_ref) <= MIXED_TOL
        assert np.array_equal(X_t.cpu().numpy(), Xc)

    plan.step_io(**io)
    torch.cuda.synchronize()
    assert plan.status() == ibx.OK
    check(X, F)
    # captured: the graph reads the host buffers at every replay
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        plan.step_io(**io, stream=s)
    for rep in range(2):
        X2 = seam_markers(rng, n, dim)
        F2 = rng.standard_normal(n * dim)
        Xh.copy_(torch.tensor(X2))
        Fh.copy_(torch.tensor(F2, dtype=torch.float32))
        Uh.zero_()
        for t in f_t:
            t.zero_()
        torch.cuda.synchronize()
        g.replay()
        torch.cuda.synchronize()
        assert plan.status() == ibx.OK
        check(X2, F2)
    del g
    plan.close()


@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("step_mode", [0, 1, 2, 3, 4])
@pytest.mark.parametrize("with_io", [False, True])
def test_plan_graph_replays_the_step(ibx, oracle, dim, step_mode, with_io):
    """ibx_plan_graph: a step (or a step with its host transfers) captured
    into a graph instantiated with the plan's stream priorities, launched on
    the current stream with new forces and positions: the oracle's answer at
    every launch, the graph's kernel count that of an eager step."""
    rng = np.random.default_rng(191 + dim + 3 * step_mode + 10 * with_io)
    N = [24, 20, 16][:dim] if dim == 3 else [40, 36]
    n = 2500
    u = rng.standard_normal([dim] + list(N)[::-1])
    X_t = torch.zeros(n * dim, dtype=torch.float64, device="cuda")
    f_t = [torch.zeros(list(N)[::-1], dtype=torch.float32, device="cuda") for _ in range(dim)]
    u_t = [torch.tensor(u[a], dtype=torch.float32, device="cuda") for a in range(dim)]
    F_t = torch.zeros(n * dim, dtype=torch.float32, device="cuda")
    U_t = torch.zeros(n * dim, dtype=torch.float32, device="cuda")
    Xh = torch.zeros(n * dim, dtype=torch.float64).pin_memory()
    Fh = torch.zeros(n * dim, dtype=torch.float32).pin_memory()
    Uh = torch.zeros(n * dim, dtype=torch.float32).pin_memory()
    mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N],
                                       [1.0 / v for v in N], [0.0] * dim, [1.0] * dim, q, X_t, Q)
    plan = ibx.Plan(mk(f_t, F_t), "IB_4", ibx.MIXED, interp_problems=[mk(u_t, U_t)])
    plan.interp_kernel = 1
    plan.step_mode = step_mode
    io = dict(in_X=[(X_t, Xh)], in_Q=[(F_t, Fh)], out_Q=[(Uh, U_t)]) if with_io else {}
    X_t.copy_(torch.tensor(seam_markers(rng, n, dim)))
    l0 = ibx.kernel_launches()
    plan.step()
    eager_kernels = ibx.kernel_launches() - l0
    torch.cuda.synchronize()
    g = plan.graph(**io)
    assert g.kernels == eager_kernels
    for rep in range(2):
        X2 = seam_markers(rng, n, dim)
        F2 = rng.standard_normal(n * dim)
        if with_io:
            Xh.copy_(torch.tensor(X2))
            Fh.copy_(torch.tensor(F2, dtype=torch.float32))
        else:
            X_t.copy_(torch.tensor(X2))
            F_t.copy_(torch.tensor(F2, dtype=torch.float32))
        for t in f_t:
            t.zero_()
        torch.cuda.synchronize()
        g.launch()
        torch.cuda.synchronize()
        assert plan.status() == ibx.OK
        f_ref, U_ref = oracle.periodic_problem(dim, N, "IB_4", X2, F=F2, u=u, centering=1)
        f = np.stack([t.double().cpu().numpy() for t in f_t])
        U = Uh if with_io else U_t
        assert cases.rel_err(f, f_ref) <= MIXED_TOL
        assert cases.rel_err(U.double().cpu().numpy(), U_ref) <= MIXED_TOL
    g.close()
    plan.close()


def test_step_io_several_transfers_per_list(ibx, oracle):
    """Positions and forces in two transfers each (halves of the arrays) and
    the velocities out in two: the copy path of ibx_plan_step_io, against
    the oracle."""
    rng = np.random.default_rng(171)
    dim, N, n = 3, [24, 20, 16], 3001
    X = seam_markers(rng, n, dim)
    F = rng.standard_normal(n * dim)
    u = rng.standard_normal([dim] + list(N)[::-1])
    X_t = torch.zeros(n * dim, dtype=torch.float64, device="cuda")
    f_t = [torch.zeros(list(N)[::-1], dtype=torch.float32, device="cuda") for _ in range(dim)]
    u_t = [torch.tensor(u[a], dtype=torch.float32, device="cuda") for a in range(dim)]
    F_t = torch.zeros(n * dim, dtype=torch.float32, device="cuda")
    U_t = torch.zeros(n * dim, dtype=torch.float32, device="cuda")
    Xh = torch.tensor(X).pin_memory()
    Fh = torch.tensor(F, dtype=torch.float32).pin_memory()
    Uh = torch.zeros(n * dim, dtype=torch.float32).pin_memory()
    mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N],
                                       [1.0 / v for v in N], [0.0] * dim, [1.0] * dim, q, X_t, Q)
    plan = ibx.Plan(mk(f_t, F_t), "IB_4", ibx.MIXED, interp_problems=[mk(u_t, U_t)])
    h = (n // 2) * dim
    plan.step_io(in_X=[(X_t[:h], Xh[:h]), (X_t[h:], Xh[h:])], in_Q=[(F_t[:h], Fh[:h]), (F_t[h:], Fh[h:])],
                 out_Q=[(Uh[:h], U_t[:h]), (Uh[h:], U_t[h:])])
    torch.cuda.synchronize()
    assert plan.status() == ibx.OK
    f_ref, U_ref = oracle.periodic_problem(dim, N, "IB_4", X, F=F, u=u, centering=1)
    f = np.stack([t.double().cpu().numpy() for t in f_t])
    assert cases.rel_err(f, f_ref) <= MIXED_TOL
    assert cases.rel_err(Uh.double().numpy(), U_ref) <= MIXED_TOL
    assert np.array_equal(X_t.cpu().numpy(), X)
    plan.close()


@pytest.mark.parametrize("form", [1, 2, 3])
@pytest.mark.parametrize("tile_shape", [0, 1])
@pytest.mark.parametrize("kernel", KERNEL_NAMES)
@pytest.mark.parametrize("dim", [2, 3])
@pytest.mark.parametrize("centering,depth", [(1, 1), (0, 2)])
def test_visit_kernel_forms(ibx, oracle, kernel, dim, centering, depth, tile_shape, form):
    """The lane-per-(visit, component) form (1), the tile-gather form (2) and
    the tile gather with register-assembled weight vectors (3) of the
    per-visit kernel, every marker spread through its visits, against the
    oracle."""
    rng = np.random.default_rng(71 + dim + 10 * centering + 100 * KERNEL_NAMES.index(kernel) + tile_shape)
    N = [29, 22, 18][:dim] if dim == 3 else [45, 38]
    n = 2500
    X = seam_markers(rng, n, dim)
    ncomp = dim if centering == 1 else depth
    F = rng.standard_normal(n * ncomp)
    u = rng.standard_normal([ncomp] + list(N)[::-1])
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=centering, depth=depth)
    f, U, ps, pi = run_plan(ibx, dim, N, kernel, X, F, u, centering, depth, dense_min=1 << 30,
                            tile_shape=tile_shape, visit_kernel=form)
    assert ps.visit_kernel == form
    assert cases.rel_err(f, f_ref) <= MIXED_TOL
    assert cases.rel_err(U, U_ref) <= MIXED_TOL
    ps.close()
    pi.close()


# Grids (52 x 35), (40 x 36 x 32) and (64 x 48) hold tiles whose staged
# interpolation region lies inside the grid (tensor copies); 27 x 20 x 34 is
# not a multiple of 4 along x (plain loads only); 32 x 20 x 18 has no
# interior region for 3D stencils.
@pytest.mark.parametrize("tile_shape", [0, 1])
@pytest.mark.parametrize("kernel", KERNEL_NAMES)
@pytest.mark.parametrize("dim,N", [(2, [52, 35]), (2, [64, 48]), (3, [27, 20, 34]), (3, [32, 20, 18]),
                                   (3, [40, 36, 32])])
@pytest.mark.parametrize("centering,depth", [(1, 1), (0, 3)])
@pytest.mark.parametrize("dense_min", [0, 8])
def test_interp_forms_identical(ibx, oracle, kernel, dim, N, centering, depth, tile_shape, dense_min):
    """Every interpolation form (chunks in home order, dense-homed markers per
    home unit, chunks in marker order, regions staged in shared memory for
    every marker or for the dense-homed ones) sums in the same order:
    bit-identical results (every tile dense, then a mix), all within the bar
    of the oracle."""
    rng = np.random.default_rng(91 + N[0] + 10 * centering + 100 * KERNEL_NAMES.index(kernel) + tile_shape)
    n = 2000
    X = seam_markers(rng, n, dim)
    ncomp = dim if centering == 1 else depth
    F = rng.standard_normal(n * ncomp)
    u = rng.standard_normal([ncomp] + list(N)[::-1])
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=centering, depth=depth)
    got = []
    for form in (1, 2, 3, 4, 0):
        f, U, ps, pi = run_plan(ibx, dim, N, kernel, X, F, u, centering, depth, dense_min=dense_min,
                                tile_shape=tile_shape, interp_kernel=form)
        assert pi.interp_kernel == form
        assert pi.status() == ibx.OK
        assert cases.rel_err(U, U_ref) <= MIXED_TOL
        got.append(U)
        ps.close()
        pi.close()
    for g in got[:-1]:
        assert np.array_equal(g, got[-1])


@pytest.mark.parametrize("kernel", ["IB_4", "IB_6", "BSPLINE_4"])
@pytest.mark.parametrize("dim,N,tma", [(3, [64, 48, 40], 1), (3, [62, 48, 40], 0), (2, [96, 80], 1)])
def test_staged_interpolation_uses_tensor_copies(ibx, oracle, kernel, dim, N, tma):
    """The staged interpolation form loads interior regions by tensor copies
    where the layout allows (x extent a multiple of 4 values) and by plain
    loads otherwise; both give the chunked form's values bit for bit, on
    clustered (dense) and uniform (sparse) markers, within the bar of the
    oracle."""
    rng = np.random.default_rng(17 + N[0] + 3 * KERNEL_NAMES.index(kernel))
    n = 6000
    X = np.concatenate([0.5 + 0.04 * rng.standard_normal((n // 2, dim)),
                        rng.uniform(0.0, 1.0, size=(n - n // 2, dim))])
    X = np.mod(X, 1.0).reshape(-1)
    F = rng.standard_normal(n * dim)
    u = rng.standard_normal([dim] + list(N)[::-1])
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=1)
    got = []
    for form in (3, 0):
        f, U, ps, pi = run_plan(ibx, dim, N, kernel, X, F, u, 1, 1, interp_kernel=form)
        assert pi.tma_problems == tma
        assert pi.status() == ibx.OK
        assert cases.rel_err(U, U_ref) <= MIXED_TOL
        got.append(U)
        ps.close()
        pi.close()
    assert np.array_equal(got[0], got[1])


@pytest.mark.parametrize("cap", [1, 5, 32])
@pytest.mark.parametrize("kernel", ["IB_4", "IB_6", "PIECEWISE_LINEAR"])
@pytest.mark.parametrize("dim", [2, 3])
def test_unit_cap(ibx, oracle, kernel, dim, cap):
    """Home units capped at 1, 5 and 32 markers (every tile dense): the
    counting sort stays exact and the spread and interpolation stay within
    the bar of the oracle."""
    rng = np.random.default_rng(301 + dim + 7 * cap + 100 * KERNEL_NAMES.index(kernel))
    N = [24, 20, 16][:dim] if dim == 3 else [40, 36]
    n = 3000
    # clustered markers: long runs of equal stencil bases
    X = (rng.uniform(0.4, 0.45, size=(n, dim)) + rng.uniform(0, 1e-3, size=(n, dim))).reshape(-1)
    F = rng.standard_normal(n * dim)
    u = rng.standard_normal([dim] + list(N)[::-1])
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=1)
    X_t = torch.tensor(X, device="cuda")
    f_t = [torch.zeros(N[::-1], dtype=torch.float32, device="cuda") for _ in range(dim)]
    u_t = [torch.tensor(u[a], dtype=torch.float32, device="cuda") for a in range(dim)]
    F_t = torch.tensor(F, dtype=torch.float32, device="cuda")
    U_t = torch.zeros(n * dim, dtype=torch.float32, device="cuda")
    mk = lambda q, Q: ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0] * dim, [v - 1 for v in N],
                                       [1.0 / v for v in N], [0.0] * dim, [1.0] * dim, q, X_t, Q)
    plan = ibx.Plan(mk(f_t, F_t), kernel, ibx.MIXED, interp_problems=[mk(u_t, U_t)])
    plan.set_tuning(dense_min=0)
    plan.unit_cap = cap
    assert plan.unit_cap == cap
    plan.step()
    torch.cuda.synchronize()
    f = np.stack([t.double().cpu().numpy() for t in f_t])
    assert cases.rel_err(f, f_ref) <= MIXED_TOL
    assert cases.rel_err(U_t.double().cpu().numpy(), U_ref) <= MIXED_TOL
    plan.close()


@pytest.mark.parametrize("N", [[256, 250], [4128, 4096]])
def test_counting_sort_scans_small_and_large_tile_counts(ibx, N):
    """The counting sort's scans: one CTA up to 8,192 tile counters, three
    launches above (4128 x 4096 cells = 66,048 tiles of 16 x 16); tile
    starts are the exclusive scan of the home-tile counts, bit-exact, and
    the spread matches the per-marker plain form's mass."""
    rng = np.random.default_rng(404 + N[0])
    dim, n = 2, 60000
    X = rng.uniform(0.0, 1.0, size=n * dim)
    X_t = torch.tensor(X, device="cuda")
    f_t = [torch.zeros(N[::-1], dtype=torch.float32, device="cuda") for _ in range(dim)]
    F_t = torch.ones(n * dim, dtype=torch.float32, device="cuda")
    prob = ibx.make_problem(dim, ibx.SIDE, ibx.MODE_PERIODIC, [0, 0], [N[0] - 1, N[1] - 1], [1.0 / N[0], 1.0 / N[1]],
                            [0.0, 0.0], [1.0, 1.0], f_t, X_t, F_t)
    plan = ibx.Plan(prob, "IB_4", ibx.MIXED)
    plan.set_tuning(dense_min=4)
    plan.bin()
    plan.spread()
    torch.cuda.synchronize()
    bc, bs, ht, ts, hl = plan.bins(n)
    counts = np.bincount(ht, minlength=plan.n_tiles)
    assert plan.n_tiles == ((N[0] + 15) // 16) * ((N[1] + 15) // 16)
    assert ts[0] == 0 and np.array_equal(np.diff(ts), counts)
    assert np.array_equal(np.sort(hl), np.arange(n))
    # unit forces: every component's grid sum is n / (dx dy) (weights sum to 1)
    for a in range(dim):
        total = float(f_t[a].double().sum()) / (N[0] * N[1])
        assert abs(total - n) <= 1e-4 * n
    assert plan.status() == ibx.OK
    plan.close()


@pytest.mark.parametrize("kernel", ["IB_4", "IB_6", "BSPLINE_4", "IB_3"])
@pytest.mark.parametrize("dim,N,n", [(3, [64, 64, 48], 5000), (3, [40, 48, 56], 3000), (2, [200, 180], 4000)])
@pytest.mark.parametrize("centering,depth", [(1, 1), (0, 3)])
def test_visit_gather_one_pass(ibx, oracle, kernel, dim, N, n, centering, depth):
    """Sparse uniform markers (a few dozen visits per tile: one or two
    batches) plus a cluster (tiles with hundreds of visits: many batches
    folded into double-FP32 pairs), every tile spread through visits: the
    gather forms 2 and 3 within the bar of the oracle."""
    rng = np.random.default_rng(808 + N[0] + 17 * KERNEL_NAMES.index(kernel) + centering)
    X = np.concatenate([rng.uniform(0.0, 1.0, size=(n, dim)), 0.3 + 0.01 * rng.standard_normal((n // 10, dim))])
    X = np.mod(X, 1.0).reshape(-1)
    m = X.size // dim
    ncomp = dim if centering == 1 else depth
    F = rng.standard_normal(m * ncomp)
    u = rng.standard_normal([ncomp] + list(N)[::-1])
    f_ref, _ = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=centering, depth=depth)
    for form in (2, 3):
        f, U, ps, pi = run_plan(ibx, dim, N, kernel, X, F, u, centering, depth, dense_min=1 << 30,
                                visit_kernel=form)
        assert ps.status() == ibx.OK
        assert cases.rel_err(f, f_ref) <= MIXED_TOL, form
        ps.close()
        pi.close()
