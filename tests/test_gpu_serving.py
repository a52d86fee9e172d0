"""Serving loop on the GPU: each request's result is the same alone (eager
launches) and in a mix of overlapping requests for other simulations (CUDA
graph replays), within the mixed-form tolerance (the sums differ only in the
order of FP32 atomics); a result matches the oracle, and the admission
estimate bounds the plan's real scratch memory."""

import numpy as np
import pytest

from tests import cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5


@pytest.fixture(scope="module")
def serving():
    from ibamr_gb300 import ibx, serving as s

    assert torch.cuda.is_available()
    ibx.lib()
    return s


def make_specs(serving):
    from ibamr_gb300 import workloads

    rng = np.random.default_rng(55)
    specs = []
    shapes = [(2, [64, 64], 3000), (3, [32, 32, 32], 8000), (2, [128, 96], 6000), (3, [40, 32, 24], 5000),
              (2, [48, 48], 1000), (3, [48, 48, 48], 20000)]
    for sid, (dim, N, n) in enumerate(shapes):
        if dim == 2:
            X = workloads.fourier_curve(n, 300 + sid)
        else:
            X = rng.uniform(0.0, 1.0, size=n * 3)
        F = rng.standard_normal(n * dim)
        u = rng.standard_normal([dim] + N[::-1])
        specs.append(serving.SimSpec(sid, dim, N, X, F=F, u=u))
    return specs


def test_results_alone_equal_results_in_the_mix(serving, oracle):
    specs = make_specs(serving)
    alone = {}
    for s in specs:
        # alone: eager launches; in the mix below: graph replays
        srv = serving.Server(serving.CudaBackend("IB_4", graphs=False), 1 << 36, n_slots=1)
        srv.register(s)
        out = srv.run([serving.Request(0, 0.0, s.sid)], keep_results=True)
        torch.cuda.synchronize()
        U, f = out["results"][0]
        alone[s.sid] = (U.double().cpu().numpy(), [t.double().cpu().numpy() for t in f])
        srv.close()
    # one alone result against the oracle
    s = specs[1]
    f_ref, U_ref = oracle.periodic_problem(s.dim, s.N, "IB_4", s.X, F=s.F, u=s.u, centering=1)
    assert cases.rel_err(alone[1][0], U_ref) <= MIXED_TOL
    assert cases.rel_err(np.stack(alone[1][1]), f_ref) <= MIXED_TOL
    # the mix: a Poisson stream over all simulations, 4 overlapping slots
    backend = serving.CudaBackend("IB_4")
    srv = serving.Server(backend, 1 << 36, n_slots=4)
    for s in specs:
        srv.register(s)
    reqs = serving.poisson_requests(20000.0, 60, [s.sid for s in specs], seed=9)
    out = srv.run(reqs, keep_results=True)
    torch.cuda.synchronize()
    assert out["requests"] == 60
    # every request replayed its simulation's captured step of library kernels
    assert backend.kernel_launches == sum(srv.resident[r.sid].kernels_per_step for r in reqs) > 0
    for r in reqs:
        U, f = out["results"][r.rid]
        Ua, fa = alone[r.sid]
        assert cases.rel_err(U.double().cpu().numpy(), Ua) <= MIXED_TOL, r
        for a in range(len(f)):
            assert cases.rel_err(f[a].double().cpu().numpy(), fa[a]) <= MIXED_TOL, r
    # admission estimate bounds the real plan scratch
    for sid, sim in srv.resident.items():
        spec = srv.specs[sid]
        assert serving.plan_bytes_estimate(spec.dim, spec.N, spec.n_markers) >= sim.plan.scratch_bytes
    srv.close()


def test_budget_admission_on_the_gpu(serving):
    specs = make_specs(serving)[:3]
    budget = int(sum(s.bytes for s in specs[:2]) + 1)
    srv = serving.Server(serving.CudaBackend("IB_4"), budget, n_slots=2)
    for s in specs:
        srv.register(s)
    reqs = [serving.Request(i, 0.0, [0, 1, 2][i % 3]) for i in range(12)]
    out = srv.run(reqs)
    torch.cuda.synchronize()
    assert out["requests"] == 12 and out["evictions"] > 0 and srv.used <= budget
    srv.close()
