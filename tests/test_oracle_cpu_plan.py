"""The timed CPU baseline (oracle CpuPlan: the reference's per-patch flow over
box patches cut by marker workload, run on a pool of host threads) computes
the same spread and interpolation as the single-patch reference flow
(oracle.periodic_problem), up to the order of FP64 additions."""

import numpy as np
import pytest


@pytest.mark.parametrize("dim,N,kernel", [(2, [48, 40], "IB_4"), (3, [24, 20, 28], "IB_4"),
                                          (3, [24, 24, 24], "IB_6"), (2, [40, 44], "BSPLINE_4")])
@pytest.mark.parametrize("threads,boxes", [(1, 1), (3, 7), (4, 16)])
def test_cpu_plan_matches_single_patch_flow(oracle, dim, N, kernel, threads, boxes):
    rng = np.random.default_rng(5 + dim + boxes)
    n = 3000
    # a cluster (small boxes around it) plus uniform markers and markers at the seams
    X = np.concatenate([0.5 + 0.05 * rng.standard_normal((n // 2, dim)),
                        rng.uniform(0.0, 1.0, size=(n // 4, dim)),
                        rng.uniform(-0.02, 0.02, size=(n - n // 2 - n // 4, dim))])
    X = np.mod(X, 1.0).reshape(-1)
    F = rng.standard_normal(n * dim)
    u = rng.standard_normal([dim] + N[::-1])
    f_ref, U_ref = oracle.periodic_problem(dim, N, kernel, X, F=F, u=u, centering=1)
    plan = oracle.CpuPlan(dim, N, kernel, X, threads=threads, boxes=boxes)
    assert 1 <= plan.patches <= boxes
    vol = int(np.prod(N))
    for step in range(2):
        f = np.zeros(dim * vol)
        U = np.zeros(n * dim)
        plan.step(F, f, u.reshape(-1).copy(), U)
        f = f.reshape([dim] + N[::-1])
        assert np.max(np.abs(f - f_ref)) <= 1e-12 * np.max(np.abs(f_ref)), step
        assert np.max(np.abs(U - U_ref)) <= 1e-12 * np.max(np.abs(U_ref)), step
