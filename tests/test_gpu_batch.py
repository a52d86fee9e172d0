"""Batched independent problems (uneven grid and marker sizes) in one plan,
captured in a CUDA graph and replayed: every problem's spread and
interpolation match the oracle within the mixed-form tolerance, on the
first replay and on a second one (the graph re-bins moved markers)."""

import numpy as np
import pytest

from tests import cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5


@pytest.fixture(scope="module")
def batch_mod():
    from ibamr_gb300 import batch, ibx

    assert torch.cuda.is_available()
    ibx.lib()
    return batch


def make_problems(rng, n_problems):
    from ibamr_gb300 import workloads

    out = []
    for p in range(n_problems):
        N = int(rng.choice([16, 32, 48, 64, 96]))
        n = int(np.floor(np.exp(rng.uniform(np.log(50.0), np.log(3000.0)))))
        out.append(([N, N], workloads.fourier_curve(n, 1000 + p)))
    return out


def check_against_oracle(oracle, B, problems, F, u):
    for k, (N, X) in enumerate(problems):
        Fk = F[B.marker_offsets[k] * 2: B.marker_offsets[k + 1] * 2]
        f_ref, U_ref = oracle.periodic_problem(2, N, "IB_4", X, F=Fk, u=u[k], centering=1)
        f = np.stack([t.double().cpu().numpy() for t in B.grid("f", k)])
        assert cases.rel_err(f, f_ref) <= MIXED_TOL, k
        assert cases.rel_err(B.markers(B.U, k).double().cpu().numpy(), U_ref) <= MIXED_TOL, k


def test_batched_graph_replay_matches_oracle(batch_mod, oracle):
    rng = np.random.default_rng(404)
    problems = make_problems(rng, 40)
    B = batch_mod.BatchedProblems(problems, dim=2, kernel="IB_4", tune=True, tune_reps=1)
    nm = int(B.marker_offsets[-1])
    F = rng.standard_normal(nm * 2)
    u = [rng.standard_normal((2, N[1], N[0])) for N, _ in problems]
    B.F.copy_(torch.tensor(F, dtype=torch.float32))
    for k in range(len(problems)):
        for a, t in enumerate(B.grid("u", k)):
            t.copy_(torch.tensor(u[k][a], dtype=torch.float32))
    B.capture()  # runs one eager warm-up step (spreads once)
    B.f.zero_()
    B.replay()
    torch.cuda.synchronize()
    assert B.status() == 0
    check_against_oracle(oracle, B, problems, F, u)
    # move the markers and replay the same graph: it re-bins them
    moved = [(N, np.mod(X + 0.013, 1.0)) for N, X in problems]
    B.X.copy_(torch.from_numpy(np.concatenate([X for _, X in moved])))
    B.f.zero_()
    B.replay()
    torch.cuda.synchronize()
    check_against_oracle(oracle, B, moved, F, u)
    B.close()


def test_batched_graph_with_host_transfers_matches_oracle(batch_mod, oracle):
    """One CUDA graph per step holding the host transfers (ibx_plan_step_io):
    positions read by the binning straight from pinned host memory across
    all problems, forces uploaded beside the binning, velocities downloaded
    beside the spread.  Replayed with new host positions and forces, every
    problem matches the oracle and the device position array follows the
    host one."""
    rng = np.random.default_rng(405)
    problems = make_problems(rng, 24)
    B = batch_mod.BatchedProblems(problems, dim=2, kernel="IB_4", tune=False)
    nm = int(B.marker_offsets[-1])
    u = [rng.standard_normal((2, N[1], N[0])) for N, _ in problems]
    for k in range(len(problems)):
        for a, t in enumerate(B.grid("u", k)):
            t.copy_(torch.tensor(u[k][a], dtype=torch.float32))
    Xh = B.X.cpu().pin_memory()
    Fh = torch.zeros(nm * 2, dtype=torch.float32).pin_memory()
    Uh = torch.zeros(nm * 2, dtype=torch.float32).pin_memory()
    B.capture(B.host_io(Xh, Fh, Uh))
    for rep in range(2):
        # move every marker a little and draw new forces, on the host
        X = Xh.numpy().reshape(-1, 2) + rng.uniform(-2e-3, 2e-3, size=(nm, 2))
        X = np.mod(X, 1.0)
        F = rng.standard_normal(nm * 2)
        Xh.copy_(torch.tensor(X.reshape(-1)))
        Fh.copy_(torch.tensor(F, dtype=torch.float32))
        B.f.zero_()
        torch.cuda.synchronize()
        B.replay()
        torch.cuda.synchronize()
        assert B.status() == 0
        assert np.array_equal(B.X.cpu().numpy(), Xh.numpy())
        B.U.copy_(Uh)  # the downloaded velocities, checked like the device ones
        moved = [(N, X[B.marker_offsets[k]: B.marker_offsets[k + 1]].reshape(-1)) for k, (N, _) in
                 enumerate(problems)]
        check_against_oracle(oracle, B, moved, F, u)
    B.close()
