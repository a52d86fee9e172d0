"""The measured configurations at their full sizes, against the FP64 oracle.

- 2,000,000 clustered markers (64 helices of 25,000 + 400,000 uniform) on a
  256^3 periodic staggered grid, IB_4 and IB_6: the plain FP64 form within
  1e-12 and the mixed form within 1e-5 of the reference's per-patch CPU flow
  (oracle CpuPlan, run on every host thread; itself pinned to the
  single-patch reference flow by tests/test_oracle_cpu_plan.py).
- The 512-problem batch (2D, N uniform in {32, ..., 512}, 100-20,000 markers
  per problem on Fourier curves, IB_4), autotuned, captured in one CUDA graph
  and replayed: every problem's spread and interpolation within 1e-5 of the
  oracle, N = 512 problems included.
- The serving mix (32 resident simulations, 2D N in [64, 512], 3D N in
  [32, 192], 1e3-5e5 markers): every simulation's result alone within 1e-5
  of the oracle, and every request of a Poisson stream the same in the mix
  as alone within 1e-5.

Reference flow: LDataManager::spread / interp applied patch by patch
(ibtk/src/lagrangian/LDataManager.cpp:552-811).
"""

import concurrent.futures
import os

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


def rel(a, b):
    a = torch.as_tensor(a, device="cuda", dtype=torch.float64)
    b = torch.as_tensor(b, device="cuda", dtype=torch.float64)
    return float((a - b).abs().max() / b.abs().max())


@pytest.mark.parametrize("kernel", ["IB_4", "IB_6"])
def test_helices_256_plain_and_mixed_against_oracle(ibx, oracle, kernel):
    from ibamr_gb300 import workloads

    X = workloads.helices_and_uniform()
    n, N = X.size // 3, 256
    rng = np.random.default_rng(workloads.SEED + 30)
    F = rng.standard_normal(X.size)
    u = np.random.default_rng(11).standard_normal(3 * N ** 3)
    threads = os.cpu_count() or 1
    cpu = oracle.CpuPlan(3, [N] * 3, kernel, X, threads=threads, boxes=4 * threads)
    f_ref = np.zeros(3 * N ** 3)
    U_ref = np.zeros(X.size)
    cpu.step(F, f_ref, u, U_ref)
    f_ref = f_ref.reshape(3, N, N, N)
    dx = [1.0 / N] * 3
    mk = lambda q, Xt, Q: ibx.make_problem(3, ibx.SIDE, ibx.MODE_PERIODIC, [0] * 3, [N - 1] * 3, dx, [0.0] * 3,
                                           [1.0] * 3, q, Xt, Q)
    X_t = torch.tensor(X, device="cuda")
    u3 = u.reshape(3, N, N, N)
    # plain FP64 form
    f_t = [torch.zeros([N] * 3, dtype=torch.float64, device="cuda") for _ in range(3)]
    u_t = [torch.tensor(u3[a], device="cuda") for a in range(3)]
    U_t = torch.zeros(X.size, dtype=torch.float64, device="cuda")
    ibx.spread(mk(f_t, X_t, torch.tensor(F, device="cuda")), kernel)
    ibx.interpolate(mk(u_t, X_t, U_t), kernel)
    torch.cuda.synchronize()
    assert rel(torch.stack(f_t), f_ref) <= PLAIN_TOL
    assert rel(U_t, U_ref) <= PLAIN_TOL
    del f_t, u_t, U_t
    # mixed form, default setting and the staged interpolation
    for interp_form in (0, 3):
        f_m = [torch.zeros([N] * 3, dtype=torch.float32, device="cuda") for _ in range(3)]
        u_m = [torch.tensor(u3[a], dtype=torch.float32, device="cuda") for a in range(3)]
        F_m = torch.tensor(F, dtype=torch.float32, device="cuda")
        U_m = torch.zeros(X.size, dtype=torch.float32, device="cuda")
        plan = ibx.Plan(mk(f_m, X_t, F_m), kernel, ibx.MIXED, interp_problems=[mk(u_m, X_t, U_m)])
        plan.interp_kernel = interp_form
        plan.step()
        torch.cuda.synchronize()
        assert plan.status() == ibx.OK
        assert rel(torch.stack(f_m), f_ref) <= MIXED_TOL
        assert rel(U_m, U_ref) <= MIXED_TOL
        plan.close()
        del f_m, u_m, F_m, U_m
    torch.cuda.empty_cache()


def oracle_pool(fn, items):
    """Runs fn over items on every host thread (the oracle's calls release
    the interpreter lock)."""
    with concurrent.futures.ThreadPoolExecutor(max_workers=os.cpu_count() or 1) as ex:
        return list(ex.map(fn, items))


def test_batched_512_full_size_against_oracle(ibx, oracle):
    from ibamr_gb300 import batch, workloads

    problems = [([N, N], X) for N, X in workloads.batched_2d(512)]
    assert {N[0] for N, _ in problems} == {32, 64, 128, 256, 512}
    B = batch.BatchedProblems(problems, dim=2, kernel="IB_4", tune=False)
    nm = int(B.marker_offsets[-1])
    rng = np.random.default_rng(workloads.SEED + 40)
    F = rng.standard_normal(nm * 2)
    u = [rng.standard_normal((2, N[1], N[0])) for N, _ in problems]
    B.F.copy_(torch.tensor(F, dtype=torch.float32))
    for k in range(len(problems)):
        for a, t in enumerate(B.grid("u", k)):
            t.copy_(torch.tensor(u[k][a], dtype=torch.float32))
    B.autotune(reps=1)  # the batch's own setting, as the benchmark runs it
    B.capture()
    B.f.zero_()
    B.replay()
    torch.cuda.synchronize()
    assert B.status() == ibx.OK

    def ref(k):
        N, X = problems[k]
        Fk = F[B.marker_offsets[k] * 2: B.marker_offsets[k + 1] * 2]
        return oracle.periodic_problem(2, N, "IB_4", X, F=Fk, u=u[k], centering=1)

    refs = oracle_pool(ref, range(len(problems)))
    for k, (f_ref, U_ref) in enumerate(refs):
        f = np.stack([t.double().cpu().numpy() for t in B.grid("f", k)])
        assert cases.rel_err(f, f_ref) <= MIXED_TOL, (k, problems[k][0])
        assert cases.rel_err(B.markers(B.U, k).double().cpu().numpy(), U_ref) <= MIXED_TOL, (k, problems[k][0])
    B.close()


def test_serving_mix_full_size(ibx, oracle):
    from ibamr_gb300 import serving, workloads

    specs = [serving.SimSpec(sid, dim, N, X, F=F, u=u) for sid, dim, N, X, F, u in workloads.serving_mix()]
    assert max(s.n_markers for s in specs) > 2e5
    assert any(s.dim == 3 and s.N[0] > 160 for s in specs) and any(s.dim == 2 and s.N[0] > 400 for s in specs)
    # every simulation alone (eager launches), against the oracle
    alone = {}
    for s in specs:
        srv = serving.Server(serving.CudaBackend("IB_4", graphs=False), 1 << 38, n_slots=1)
        srv.register(s)
        out = srv.run([serving.Request(0, 0.0, s.sid)], keep_results=True)
        torch.cuda.synchronize()
        U, f = out["results"][0]
        alone[s.sid] = (U.double().cpu().numpy(), [t.double().cpu().numpy() for t in f])
        srv.close()
    refs = oracle_pool(lambda s: oracle.periodic_problem(s.dim, s.N, "IB_4", s.X, F=s.F,
                                                         u=s.u.astype(np.float64), centering=1), specs)
    for s, (f_ref, U_ref) in zip(specs, refs):
        assert cases.rel_err(alone[s.sid][0], U_ref) <= MIXED_TOL, s.sid
        assert cases.rel_err(np.stack(alone[s.sid][1]), f_ref) <= MIXED_TOL, s.sid
    # the mix: a Poisson stream at 2000 requests/s over all simulations, 8 slots
    backend = serving.CudaBackend("IB_4")
    srv = serving.Server(backend, 150 * 10 ** 9, n_slots=8)
    for s in specs:
        srv.register(s)
    reqs = serving.poisson_requests(2000.0, 96, [s.sid for s in specs], seed=21)
    out = srv.run(reqs, keep_results=True)
    torch.cuda.synchronize()
    assert out["requests"] == len(reqs)
    for r in reqs:
        U, f = out["results"][r.rid]
        Ua, fa = alone[r.sid]
        assert cases.rel_err(U.double().cpu().numpy(), Ua) <= MIXED_TOL, r
        for a in range(len(f)):
            assert cases.rel_err(f[a].double().cpu().numpy(), fa[a]) <= MIXED_TOL, r
    srv.close()
