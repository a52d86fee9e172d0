"""Device spring forces (ibx_spring_forces) against a sequential restatement
of the reference loop (IBStandardForceGen::computeLagrangianSpringForce with
the default linear spring), and the 2D ellipse workload's closed-loop
springs feeding the spread in one stream."""

import numpy as np
import pytest

from tests import cases

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ibx():
    from ibamr_gb300 import ibx as m

    assert torch.cuda.is_available()
    m.lib()
    return m


def reference_springs(X, dim, mastr, slave, K, R0, F):
    """src/IB/IBStandardForceGen.cpp:825-900, sequentially."""
    Xv = X.reshape(-1, dim)
    Fv = F.reshape(-1, dim)
    for k in range(mastr.size):
        D = Xv[slave[k]] - Xv[mastr[k]]
        R = np.sqrt(np.sum(D * D))
        if R < np.finfo(np.float64).eps:
            continue
        T_over_R = K[k] * (R - R0[k]) / R
        Fv[mastr[k]] += T_over_R * D
        Fv[slave[k]] -= T_over_R * D
    return F


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("dim", [2, 3])
def test_spring_forces_match_reference_loop(ibx, dim, dtype):
    rng = np.random.default_rng(3 + dim)
    n, ns = 500, 1500
    X = rng.uniform(0, 1, size=n * dim)
    mastr = rng.integers(0, n, size=ns).astype(np.int32)
    slave = ((mastr + rng.integers(1, n, size=ns)) % n).astype(np.int32)
    slave[:5] = mastr[:5]  # zero-length springs are skipped
    K = rng.uniform(0.5, 2.0, size=ns)
    R0 = rng.uniform(0.0, 0.1, size=ns)
    F0 = rng.standard_normal(n * dim)
    F_ref = reference_springs(X, dim, mastr, slave, K, R0, F0.copy())
    tdt = torch.float64 if dtype == "float64" else torch.float32
    F_t = torch.tensor(F0, dtype=tdt, device="cuda")
    dev = lambda a: torch.tensor(a, device="cuda")
    st = ibx.spring_forces(dim, dev(X), dev(mastr), dev(slave), dev(K), dev(R0), F_t, accumulate=True)
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    tol = 1e-12 if dtype == "float64" else 1e-5
    assert cases.rel_err(F_t.double().cpu().numpy(), F_ref) <= tol
    # accumulate = False zeroes F first
    F_t.fill_(123.0)
    ibx.spring_forces(dim, dev(X), dev(mastr), dev(slave), dev(K), dev(R0), F_t)
    F_ref2 = reference_springs(X, dim, mastr, slave, K, R0, np.zeros(n * dim))
    torch.cuda.synchronize()
    assert cases.rel_err(F_t.double().cpu().numpy(), F_ref2) <= tol


def test_bad_node_index_is_reported(ibx):
    dev = lambda a: torch.tensor(a, device="cuda")
    X = dev(np.zeros(6))
    F = torch.zeros(6, dtype=torch.float64, device="cuda")
    st = ibx.spring_forces(2, X, dev(np.array([0, 5], np.int32)), dev(np.array([1, 2], np.int32)),
                           dev(np.ones(2)), dev(np.zeros(2)), F)
    torch.cuda.synchronize()
    assert int(st.item()) & 1


def test_ellipse_springs_then_spread(ibx, oracle):
    """The 2D ellipse workload (256 markers, closed loop, K = 1, rest 0):
    forces on the device, spread on the same stream, against the oracle
    spreading the workload's host-computed forces."""
    from ibamr_gb300 import workloads

    X, F_host = workloads.ellipse_springs(256)
    n = X.size // 2
    mastr = np.arange(n, dtype=np.int32)
    slave = ((mastr + 1) % n).astype(np.int32)
    dev = lambda a: torch.tensor(a, device="cuda")
    X_t = dev(X)
    F_t = torch.zeros(n * 2, dtype=torch.float64, device="cuda")
    ibx.spring_forces(2, X_t, dev(mastr), dev(slave), dev(np.ones(n)), dev(np.zeros(n)), F_t)
    f_t = [torch.zeros(64, 64, dtype=torch.float64, device="cuda") for _ in range(2)]
    prob = ibx.make_problem(2, ibx.SIDE, ibx.MODE_PERIODIC, [0, 0], [63, 63], [1 / 64] * 2, [0, 0], [1, 1], f_t,
                            X_t, F_t)
    ibx.spread(prob, "IB_4")
    torch.cuda.synchronize()
    assert cases.rel_err(F_t.cpu().numpy(), F_host) <= 1e-12
    f_ref, _ = oracle.periodic_side_problem(2, [64, 64], "IB_4", X, F=F_host)
    f = np.stack([t.cpu().numpy() for t in f_t])
    assert cases.rel_err(f, f_ref) <= 1e-12
